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

    def draw(self, kind):
        """Seeded random inputs of one system of the given kind (0 pressure, 1 potential)."""
        torch, g = self.torch, self.g
        phi = random_scene_phi(torch, self.n, self.rng, self.dev)
        gen = torch.Generator(device=self.dev)
        gen.manual_seed(int(self.rng.integers(1 << 62)))
        if kind == 0:
            vel = [torch.randn(g.face_shape(a), dtype=torch.float64, device=self.dev, generator=gen) * 0.5
                   for a in range(3)]
            return dict(kind=0, phi=phi, vel=vel)
        d = self.rng.normal(size=3)
        d = d / np.linalg.norm(d) * self.rng.uniform(0.5, 2.0)
        hext = [torch.full(g.face_shape(a), float(d[a]), dtype=torch.float64, device=self.dev) for a in range(3)]
        return dict(kind=1, phi=phi, hext=hext, chi=float(self.rng.uniform(0.5, 3.0)))

    def solve(self, inp, precision, tol):
        """Solve a drawn system (inputs are not modified); returns the solver statistics."""
        torch, g, sf = self.torch, self.g, self.sf
        if inp["kind"] == 0:
            vel = [v.clone() for v in inp["vel"]]
            st = self.P.project(vel, inp["phi"], self.frac, device=True, raise_on_nonconv=False,
                                opts=sf.options("pressure", precision=precision, tol=tol))
        else:
            self.M.set_susceptibility(inp["chi"])
            psi = torch.zeros(g.shape, dtype=torch.float64, device=self.dev)
            H = [torch.zeros(g.face_shape(a), dtype=torch.float64, device=self.dev) for a in range(3)]
            st = self.M.solve(inp["phi"], inp["hext"], device=True, psi_out=psi, H_out=H, raise_on_nonconv=False,
                              opts=sf.options("magnetic", precision=precision, tol=tol, warm_start=0))
        torch.cuda.synchronize(self.dev)
        return st

    def system(self, kind):
        """Draw, solve with the plain FP64 method to 1e-8, and export features (.feat) and solution (.sol)."""
        inp = self.draw(kind)
        st = self.solve(inp, "fp64", 1e-8)
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


def evaluate(ctx, net, scenes=64, n=256, seed=777, tol=1e-6, log=None):
    """Ablation on unseen seeded scenes: mixed-precision MGPCG from zero against the same solver started from
    the network's prediction (with its fallback).  Returns per-scene iterations, times and guess residuals."""
    import torch
    src = SampleSource(ctx, n, seed)
    rows = []
    for i in range(scenes):
        inp = src.draw(i % 2)
        res = {}
        for prec in ("mixed", "learned"):
            torch.cuda.synchronize()
            t = time.perf_counter()
            st = src.solve(inp, prec, tol)
            res[prec] = dict(iters=st["iters"], outer=st["outer_iters"], ms=1e3 * (time.perf_counter() - t),
                             relres=st["rel_residual"], guess=st["guess_rel_residual"],
                             energy=st["guess_energy_ratio"])
        rows.append(dict(kind=i % 2, **res))
        if log:
            log(f"scene {i:3d} kind {i % 2} plain {res['mixed']['iters']:3d} it {res['mixed']['ms']:7.2f} ms | "
                f"learned {res['learned']['iters']:3d} it {res['learned']['ms']:7.2f} ms guess "
                f"{res['learned']['guess']:.3f} energy {res['learned']['energy']:.3f}")
    return rows


def time_forward(ctx, net, n, reps=5):
    """Milliseconds per network forward at n^3 (inference workspace) with the warp-MMA and the tcgen05 kernels,
    CUDA events on the context's stream; also the largest difference between the two outputs."""
    import torch
    sf = _pkg()
    g = sf.StaggeredGrid.from_origin(1.0 / n, (n, n, n))
    dev = torch.device("cuda", ctx.device)
    rng = np.random.default_rng(1)
    feat = torch.from_numpy((rng.standard_normal((n ** 3, 16)) * 0.5).astype(np.float32)).to(dev).to(torch.bfloat16)
    out, res = {}, {}
    for mode, name in ((0, "mma"), (1, "tcgen05")):
        net.set_mode(mode)
        o = torch.zeros(n ** 3, dtype=torch.float32, device=dev)
        net.forward(g, feat, o)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            net.forward(g, feat, o)
        e1.record()
        torch.cuda.synchronize(dev)
        res[name] = e0.elapsed_time(e1) / reps
        out[name] = o
    res["max_abs_diff"] = float((out["mma"] - out["tcgen05"]).abs().max())
    res["max_abs_out"] = float(out["mma"].abs().max())
    res["n"] = n
    return res


def summarize(rows):
    out = {}
    for kind in (0, 1):
        rs = [r for r in rows if r["kind"] == kind]
        if not rs:
            continue
        out["pressure" if kind == 0 else "potential"] = {
            "scenes": len(rs),
            "plain_iters": float(np.mean([r["mixed"]["iters"] for r in rs])),
            "learned_iters": float(np.mean([r["learned"]["iters"] for r in rs])),
            "plain_ms": float(np.mean([r["mixed"]["ms"] for r in rs])),
            "learned_ms": float(np.mean([r["learned"]["ms"] for r in rs])),
            "guess_rel_residual": float(np.mean([r["learned"]["guess"] for r in rs])),
            "guess_energy_ratio": float(np.mean([r["learned"]["energy"] for r in rs])),
            "plain_solves_per_s": float(1e3 / np.mean([r["mixed"]["ms"] for r in rs])),
            "learned_solves_per_s": float(1e3 / np.mean([r["learned"]["ms"] for r in rs])),
        }
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--samples", type=int, default=2000)
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--out", default=os.path.join(HERE, "weights", "unet.f32"))
    ap.add_argument("--init", default=None, help="start from these weights")
    ap.add_argument("--eval", type=int, default=0, help="then evaluate on this many unseen scenes")
    ap.add_argument("--eval-n", type=int, default=256)
    ap.add_argument("--report", default=None, help="write the training/evaluation summary (JSON) here")
    ap.add_argument("--tc", action="store_true",
                    help="every convolution on the tcgen05 kernels (Network.set_mode(1), the default)")
    ap.add_argument("--mma", action="store_true",
                    help="every convolution on the warp-level MMA kernels (Network.set_mode(0))")
    ap.add_argument("--time-forward", type=int, default=0, metavar="N",
                    help="time the network forward at N^3 with each kernel set (CUDA events, 5 passes after one "
                         "warm-up) and add it to the report")
    args = ap.parse_args()
    sf = _pkg()
    import torch
    torch.cuda.set_device(0)
    ctx = sf.Context(0, stream=torch.cuda.current_stream().cuda_stream)  # torch's stream: events time the library
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
    net.set_mode(0 if args.mma and not args.tc else 1)
    ctx.set_network(net)
    report = {"samples": args.samples, "n": args.n, "lr": args.lr, "seed": args.seed, "tcgen05": not (args.mma and not args.tc)}
    if args.samples > 0:
        t0 = time.time()
        losses = train(ctx, net, args.samples, args.n, args.lr, args.seed, log=lambda m: print(m, flush=True))
        os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
        net.save(args.out)
        k = max(1, len(losses) // 10)
        lp = [l for i, l in enumerate(losses) if i % 2 == 0]
        lm = [l for i, l in enumerate(losses) if i % 2 == 1]
        kk = max(1, len(lp) // 10)
        report.update(train_s=round(time.time() - t0, 1), loss_first=float(np.mean(losses[:k])),
                      loss_last=float(np.mean(losses[-k:])), pressure_loss_last=float(np.mean(lp[-kk:])),
                      potential_loss_last=float(np.mean(lm[-kk:])), out=args.out)
    if args.time_forward > 0:
        report["forward_ms"] = time_forward(ctx, net, args.time_forward)
        net.set_mode(0 if args.mma and not args.tc else 1)
    if args.eval > 0:
        rows = evaluate(ctx, net, args.eval, args.eval_n, log=lambda m: print(m, flush=True))
        report["eval"] = summarize(rows)
        report["eval_n"] = args.eval_n
    print(json.dumps(report), flush=True)
    if args.report:
        with open(args.report, "w") as f:
            json.dump(report, f, indent=1)
    ctx.set_network(None)
    net.close()
    ctx.close()


def _layer_table():
    """(cin, cout, taps) of the network's layers in parameter order."""
    return [(16, 16, 27), (16, 16, 27), (16, 32, 27), (32, 32, 27), (32, 64, 27), (64, 64, 27), (64, 64, 27),
            (64, 64, 27), (64, 64, 27), (64, 32, 27), (32, 32, 27), (32, 16, 27), (16, 16, 27), (16, 16, 27),
            (16, 1, 1)]


if __name__ == "__main__":
    main()
