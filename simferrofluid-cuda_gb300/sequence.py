"""A long sequence of substeps at large resolution: one magnetic potential solve (warm-started from the previous
substep's potential, as the reference's m_Sol) and one pressure projection per substep, on device-resident
inputs, for the mixed form and the plain FP64 method in turn.

Scene (seeded, synthetic): pool of depth 0.2 with a 1% height perturbation (0.01 n(x, z), n seeded uniform
[-1, 1] on an 8x8 lattice, bilinear), chi = 1.5, walls on the grid faces, vertical applied field H0 = (0, s/S, 0)
at substep s = 1..S, and per substep a fresh velocity of seeded smooth noise with |u| <= 0.5 (uniform [-1, 1] on a
9^3 lattice, trilinear, times 0.5).  Every input is generated on the device.

The collider fractions of the box walls are the library's (sf_collider_box_fractions) on a 12^3 grid of the same
spacing, extended to the full grid: a face's fraction depends only on the walls within a few cells of it (the
fast-marching distance near a wall is computed outward from the wall), so faces more than 6 cells from every
wall take the interior value.  The extension agrees with the full-size collider to the last bits of the
level-set arithmetic.

  python simferrofluid-cuda_gb300/sequence.py --n 768 --substeps 50 --precision all

Arms: the mixed form, the mixed form with the trained network's learned correction steps ("learned"), and the plain
FP64 method with row skipping ("fp64") and sweeping every row ("fp64_full").  The learned arm runs the network's
inference workspace (decoder buffers reuse the encoder's), about 90 B per cell at 768^3.
"""
from __future__ import annotations

import argparse
import importlib
import json
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


def _stretch(m_large, m_small, c):
    """Index map of a large axis onto a small one: the first and last c entries kept, the middle -> c."""
    i = np.arange(m_large)
    out = np.full(m_large, c)
    out[i < c] = i[i < c]
    hi = (m_large - 1 - i) < c
    out[hi] = (m_small - 1) - (m_large - 1 - i[hi])
    return out


def box_fractions_device(sf, scenes, torch, g, dev, c=6):
    n = 2 * c
    small = sf.StaggeredGrid.from_origin(g.spacing, (n, n, n))
    fs = scenes.box_fractions(small)
    out = []
    for a in range(3):
        idx = [torch.from_numpy(_stretch(g.shape[b] + (b == a), n + (b == a), c)).to(dev) for b in range(3)]
        src = torch.from_numpy(fs[a]).to(dev)
        out.append(src[idx[0]][:, idx[1]][:, :, idx[2]].contiguous())
    return out


def box_normals_device(sf, scenes, torch, g, dev, c=6):
    """The box collider's face normals (sf_collider_face_normals of the redistanced node level set) on a small grid,
    extended to the full grid like the fractions: they matter only on faces of fraction 1, next to the walls."""
    import ctypes as C
    n = 2 * c
    small = sf.StaggeredGrid.from_origin(g.spacing, (n, n, n))
    lib = sf.load_library()
    fs = [np.empty(small.face_shape(a)) for a in range(3)]
    ls = np.empty((n + 1, n + 1, n + 1))
    s = lib.sf_collider_box_fractions(C.byref(small.c_grid()), 0, sf._abi.p3([f.ctypes.data for f in fs]),
                                      C.c_void_p(ls.ctypes.data))
    if s != 0:
        raise RuntimeError(f"sf_collider_box_fractions failed with status {s}")
    nm = sf.collider_face_normals(small, ls)
    out = []
    for a in range(3):
        idx = [torch.from_numpy(_stretch(g.shape[b] + (b == a), n + (b == a), c)).to(dev) for b in range(3)]
        src = torch.from_numpy(nm[a]).to(dev)
        out.append(src[idx[0]][:, idx[1]][:, :, idx[2]].contiguous())
    return out


def pool_phi_device(scenes, torch, g, dev, seed, depth=0.2, noise=0.01):
    rng = np.random.default_rng(seed)
    xs, ys, zs = (scenes.cell_centres(g, a) for a in range(3))
    nz = torch.from_numpy(scenes.lattice_noise(xs, zs, rng)).to(dev)
    y = torch.from_numpy(ys).to(dev)
    return (y.view(1, -1, 1) - depth + noise * nz.view(g.shape[0], 1, g.shape[2])).contiguous()


def smooth_velocity(torch, g, dev, gen, vmax=0.5, lattice=9):
    import torch.nn.functional as F
    out = []
    for a in range(3):
        lat = torch.rand((1, 1, lattice, lattice, lattice), generator=gen, device=dev, dtype=torch.float64) * 2 - 1
        out.append((F.interpolate(lat, size=g.face_shape(a), mode="trilinear", align_corners=True)[0, 0] * vmax)
                   .contiguous())
    return out


def run(precision, n=768, substeps=50, seed=5, profile_last=True, log=None, weights=None, full_substep=False,
        use_graph=1, inner_tol=None, pressure_opts=None, magnetic_opts=None):
    """precision "mixed", "fp64" (row skipping), "fp64_full" (every row swept) or "learned" (the mixed solver with
    the trained network's correction steps, weights/unet.f32 unless `weights` names another file).

    pressure_opts / magnetic_opts: further sf_solve_opts fields for the pressure / potential solves.

    full_substep: after the two solves, the rest of the reference's substep on the device (core/Simulation.cpp:
    164-165, 236-241, 265): extrapolation of the projected velocity, Collider::Enforce, advection of the level set
    and of the velocity (dt = h / max|u|, |u| <= 0.5) and 10 reinitialisation steps.  They run on copies of phi,
    so every substep solves the same scene; their device time is reported apart (`rest_ms`)."""
    import torch
    sf = _pkg()
    scenes = importlib.import_module(sf.__name__ + ".scenes")
    dev = torch.device("cuda", 0)
    g = sf.StaggeredGrid.from_origin(1.0 / n, (n, n, n))
    t0 = time.time()
    phi = pool_phi_device(scenes, torch, g, dev, seed)
    frac = box_fractions_device(sf, scenes, torch, g, dev)
    hext = [torch.zeros(g.face_shape(a), dtype=torch.float64, device=dev) for a in range(3)]
    H = [torch.zeros(g.face_shape(a), dtype=torch.float64, device=dev) for a in range(3)]
    psi = torch.zeros(g.shape, dtype=torch.float64, device=dev)
    p_out = torch.zeros(g.shape, dtype=torch.float64, device=dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    torch.cuda.synchronize()
    setup_s = time.time() - t0
    ctx = sf.Context(0, stream=torch.cuda.current_stream().cuda_stream)
    net = None
    extra = {}
    if precision == "learned":
        net = sf.Network(ctx)
        net.load(weights or os.path.join(HERE, "weights", "unet.f32"))
        ctx.set_network(net)
    elif precision == "fp64_full":
        extra = dict(full_sweeps=1)
    prec = {"fp64_full": "fp64"}.get(precision, precision)
    extra["use_graph"] = use_graph
    if inner_tol is not None and precision in ("mixed", "learned"):
        extra["inner_tol"] = inner_tol
    M = sf.MagneticField(g, 1.5, 2 * g.spacing, ctx)
    P = sf.Pressure(g, ctx)
    if full_substep:
        normals = box_normals_device(sf, scenes, torch, g, dev)
        ext, enf = sf.Extrapolation(g, ctx), sf.ColliderEnforce(g, frac, normals, ctx=ctx)
        adv, rei = sf.Advection(g, ctx), sf.Reinitialization(g, ctx)
        e3 = torch.cuda.Event(enable_timing=True)
        rest = []
    rows = []
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    solve_ms = 0.0
    for s in range(1, substeps + 1):
        hext[1].fill_(s / substeps)
        vel = smooth_velocity(torch, g, dev, gen)
        prof = 1 if (profile_last and s == substeps) else 0
        e0.record()
        sm = M.solve(phi, hext, device=True, psi_out=psi, H_out=H,
                     opts=sf.options("magnetic", precision=prec, profile=prof, **extra, **(magnetic_opts or {})))
        e1.record()
        sp = P.project(vel, phi, frac, device=True, p_out=p_out,
                       opts=sf.options("pressure", precision=prec, tol=1e-6, profile=prof, **extra,
                                       **(pressure_opts or {})))
        e2.record()
        if full_substep:
            ext.solve(vel, phi, frac, device=True)
            enf.enforce(vel, device=True)
            phi_w = phi.clone()
            adv.solve_levelset(phi_w, vel, g.spacing, device=True)
            adv.solve_velocity(vel, g.spacing, device=True)
            rei.solve(phi_w, 10, device=True)
            e3.record()
        torch.cuda.synchronize()
        ms_m, ms_p = e0.elapsed_time(e1), e1.elapsed_time(e2)
        if full_substep:
            rest.append(e2.elapsed_time(e3))
            del phi_w
        if not prof:
            solve_ms += ms_m + ms_p
        rows.append(dict(substep=s, mag_iters=sm["iters"], mag_ms=ms_m, mag_relres=sm["rel_residual_ref"],
                         learned_steps=(sm["learned_steps"], sp["learned_steps"]),
                         pres_iters=sp["iters"], pres_ms=ms_p, pres_relres=sp["rel_residual"],
                         smooth_ms=sm["smooth_ms"] + sp["smooth_ms"], smooth_bytes=sm["smooth_bytes"] + sp["smooth_bytes"],
                         smooth_launches=sm["smooth_launches"] + sp["smooth_launches"]))
        if log:
            r = rows[-1]
            log(f"{precision} substep {s:3d}: potential {r['mag_iters']:3d} it {ms_m:8.1f} ms | pressure "
                f"{r['pres_iters']:3d} it {ms_p:8.1f} ms")
        del vel
    timed = [r for r in rows if not (profile_last and r["substep"] == substeps)]
    last = rows[-1]
    out = dict(precision=precision, grid=[n, n, n], substeps=substeps, setup_s=round(setup_s, 2),
               solve_s=round(solve_ms / 1e3, 3), solves=2 * len(timed),
               solves_per_s=round(2 * len(timed) / (solve_ms / 1e3), 3) if solve_ms > 0 else None,
               mean_ms=dict(potential=float(np.mean([r["mag_ms"] for r in timed])),
                            pressure=float(np.mean([r["pres_ms"] for r in timed]))),
               iters=dict(potential=[r["mag_iters"] for r in rows], pressure=[r["pres_iters"] for r in rows]),
               max_rel_residual=dict(potential=max(r["mag_relres"] for r in rows),
                                     pressure=max(r["pres_relres"] for r in rows)),
               device_bytes=ctx.device_bytes())
    if precision == "learned":
        out["learned_steps"] = [r["learned_steps"] for r in rows]
    if full_substep:
        out["rest_ms"] = float(np.mean(rest))
    if profile_last and last["smooth_launches"]:
        out["smoother"] = dict(ms_per_launch=last["smooth_ms"] / last["smooth_launches"],
                               bytes_per_launch=last["smooth_bytes"] / last["smooth_launches"],
                               achieved_gbs=last["smooth_bytes"] / (last["smooth_ms"] / 1e3) / 1e9)
    if net is not None:
        ctx.set_network(None)
        net.close()
    ctx.close()
    del phi, frac, hext, H, psi, p_out
    torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=768)
    ap.add_argument("--substeps", type=int, default=50)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--precision", default="both", choices=["mixed", "fp64", "fp64_full", "learned", "both", "all"],
                    help="both: mixed and fp64; all: mixed, learned, fp64 and fp64_full")
    ap.add_argument("--out", default=None)
    ap.add_argument("--inner-tol", type=float, default=None,
                    help="mixed and learned arms: floor of the inner relative reduction (library default 1e-3)")
    ap.add_argument("--no-graph", action="store_true",
                    help="launch each solver iteration's kernels from the host (for kernel profilers)")
    ap.add_argument("--full-substep", action="store_true",
                    help="also run the rest of the substep (extrapolation, enforcement, advection, reinitialisation)")
    args = ap.parse_args()
    import torch
    torch.cuda.set_device(0)
    precs = {"both": ["mixed", "fp64"], "all": ["mixed", "learned", "fp64", "fp64_full"]}.get(args.precision,
                                                                                             [args.precision])
    res = {}
    for p in precs:
        try:
            res[p] = run(p, args.n, args.substeps, args.seed, log=lambda m: print(m, flush=True),
                         full_substep=args.full_substep, use_graph=0 if args.no_graph else 1,
                         inner_tol=args.inner_tol)
        except Exception as e:  # an arm that does not fit (device memory) is reported, the others still run
            res[p] = {"error": f"{type(e).__name__}: {e}"}
            torch.cuda.empty_cache()
            print(f"{p}: {res[p]['error']}", flush=True)
    for base in ("fp64", "fp64_full"):
        for p in ("mixed", "learned"):
            if base in res and p in res and "solve_s" in res[base] and "solve_s" in res[p]:
                res[f"speedup_{p}_vs_{base}"] = round(res[base]["solve_s"] / res[p]["solve_s"], 3)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    for p in precs:
        if "smoother" in res.get(p, {}) and peaks.get("hbm_gbs"):
            res[p]["smoother"]["frac_of_measured_hbm"] = res[p]["smoother"]["achieved_gbs"] / peaks["hbm_gbs"]
    print(json.dumps(res), flush=True)
    if args.out:
        with open(args.out, "w") as f:
            json.dump(res, f, indent=1)


if __name__ == "__main__":
    main()
