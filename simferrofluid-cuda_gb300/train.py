"""Train the learned solver's U-Net on (coefficients, rhs, solution) triples from the plain solver.

Each triple is generated on the GPU from a seeded random scene at 128^3 (pool of depth U[0.1, 0.3] united
with 1-8 spheres of radius U[0.05, 0.25] at uniform centres, chi U[0.5, 3], walls on the grid faces) and one
of the two systems of the path:
  * pressure: a seeded random MAC velocity (N(0, 0.5^2)) -> ghost-fluid projection system;
  * potential: a seeded uniform applied field of random direction and magnitude -> FDM magnetostatic system.
The plain FP64 MGPCG solves it to 1e-8; the network's input is the system (sf_system_features_dev) and its
target the solution.  Samples stream through Adam (no dataset is stored).  Training runs entirely in the
library's own CUDA kernels (tensor-core forward, input-gradient and weight-gradient convolutions, Adam).

  python -m <package>.train --samples 2000 --n 128 --out weights.f32
"""
from __future__ import annotations

import argparse
import importlib
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _pkg():
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    return importlib.import_module(os.path.basename(HERE))


def random_scene_phi(torch, n, rng, device):
    """Level set of a pool of random depth united with 1-8 random spheres (cell centres of [0, 1]^3)."""
    h = 1.0 / n
    c = (torch.arange(n, device=device, dtype=torch.float64) + 0.5) * h
    X, Y, Z = c.view(n, 1, 1), c.view(1, n, 1), c.view(1, 1, n)
    phi = (Y - rng.uniform(0.1, 0.3)).expand(n, n, n).clone()
    for _ in range(int(rng.integers(1, 9))):
        cx, cy, cz = rng.uniform(0, 1, 3)
        r = rng.uniform(0.05, 0.25)
        phi = torch.minimum(phi, torch.sqrt((X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2) - r)
    return phi.contiguous()


class SampleSource:
    """Generates training/evaluation systems on a context (device-resident inputs)."""

    def __init__(self, ctx, n, seed):
        import torch
        self.torch = torch
        self.sf = _pkg()
        self.scenes = importlib.import_module(self.sf.__name__ + ".scenes")
        self.ctx = ctx
        self.n = n
        self.g = self.scenes.unit_grid(n)
        self.dev = torch.device("cuda", ctx.device)
        self.frac = [torch.from_numpy(f).to(self.dev) for f in self.scenes.box_fractions(self.g)]
        self.rng = np.random.default_rng(seed)
        self.P = self.sf.Pressure(self.g, ctx)
        self.M = self.sf.MagneticField(self.g, 1.0, 2 * self.g.spacing, ctx)
        self.feat = torch.zeros((self.g.num_cells, 16), dtype=torch.bfloat16, device=self.dev)
        self.sol = torch.zeros(self.g.num_cells, dtype=torch.float32, device=self.dev)

    def system(self, kind):
        """Assemble and solve one system; returns the solver statistics (features in .feat, solution in .sol)."""
        torch, g, sf = self.torch, self.g, self.sf
        phi = random_scene_phi(torch, self.n, self.rng, self.dev)
        gen = torch.Generator(device=self.dev)
        gen.manual_seed(int(self.rng.integers(1 << 62)))
        if kind == 0:
            vel = [torch.randn(g.face_shape(a), dtype=torch.float64, device=self.dev, generator=gen) * 0.5
                   for a in range(3)]
            st = self.P.project(vel, phi, self.frac, device=True,
                                opts=sf.options("pressure", precision="fp64", tol=1e-8))
        else:
            self.M.set_susceptibility(self.rng.uniform(0.5, 3.0))
            d = self.rng.normal(size=3)
            d = d / np.linalg.norm(d) * self.rng.uniform(0.5, 2.0)
            hext = [torch.full(g.face_shape(a), float(d[a]), dtype=torch.float64, device=self.dev)
                    for a in range(3)]
            psi = torch.zeros(g.shape, dtype=torch.float64, device=self.dev)
            H = [torch.zeros(g.face_shape(a), dtype=torch.float64, device=self.dev) for a in range(3)]
            st = self.M.solve(phi, hext, device=True, psi_out=psi, H_out=H,
                              opts=sf.options("magnetic", precision="fp64", tol=1e-8, warm_start=0))
        torch.cuda.synchronize(self.dev)
        self.ctx.system_features(kind, self.feat, self.sol)
        return st


def train(ctx, net, samples=2000, n=128, lr=1e-3, seed=2024, log_every=50, log=None):
    src = SampleSource(ctx, n, seed)
    losses = []
    t0 = time.time()
    for i in range(samples):
        src.system(i % 2)
        cur = lr * 0.5 * (1 + math.cos(math.pi * i / samples))  # cosine decay
        loss = net.train_step(src.g, src.feat, src.sol, max(cur, lr * 0.02))
        losses.append(loss)
        if log and (i % log_every == 0 or i == samples - 1):
            log(f"sample {i:5d} kind {i % 2} loss {loss:.4f} lr {cur:.2e} t {time.time() - t0:.1f}s")
    return losses


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--samples", type=int, default=2000)
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--out", default=os.path.join(HERE, "weights", "unet.f32"))
    ap.add_argument("--init", default=None, help="start from these weights")
    args = ap.parse_args()
    sf = _pkg()
    import torch
    torch.cuda.set_device(0)
    ctx = sf.Context(0)
    net = sf.Network(ctx)
    if args.init:
        net.load(args.init)
    else:
        from_rng = np.random.default_rng(args.seed)
        flat = []
        for L in _layer_table():
            ci, co, taps = L
            std = math.sqrt(2.0 / (taps * ci)) if taps == 27 else math.sqrt(1.0 / ci)
            flat.append((from_rng.standard_normal(taps * co * ci) * std).astype(np.float32))
            flat.append(np.zeros(co, np.float32))
        net.set_params(np.concatenate(flat))
    ctx.set_network(net)
    losses = train(ctx, net, args.samples, args.n, args.lr, args.seed, log=lambda m: print(m, flush=True))
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    net.save(args.out)
    k = max(1, len(losses) // 10)
    print(json.dumps({"samples": args.samples, "n": args.n, "loss_first": float(np.mean(losses[:k])),
                      "loss_last": float(np.mean(losses[-k:])), "out": args.out}))


def _layer_table():
    """(cin, cout, taps) of the network's layers in parameter order."""
    return [(16, 16, 27), (16, 16, 27), (16, 32, 27), (32, 32, 27), (32, 64, 27), (64, 64, 27), (64, 64, 27),
            (64, 64, 27), (64, 64, 27), (64, 32, 27), (32, 32, 27), (32, 16, 27), (16, 16, 27), (16, 16, 27),
            (16, 1, 1)]


if __name__ == "__main__":
    main()
