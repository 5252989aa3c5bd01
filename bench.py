"""Benchmark: Poisson solves/s at 256^3 to 1e-6 relative residual (pressure projection + magnetic potential).

One step = one SimFerrofluid substep's pair of grid solves on the 256^3 pool+sphere scene (pool depth 0.2,
sphere r=0.15 at (0.5,0.55,0.5), chi=2, dipole field of moment (0,1,0) at (0.5,-0.3,0.5), velocity
N(0,0.5^2), walls on the grid faces): a fresh velocity is copied in, the pressure is projected (assembly,
MGPCG solve to 1e-6, velocity update) and the potential is solved from zero (assembly, solve to 1e-6, H on
faces).  ``value`` counts 2 solves per step, inputs resident in HBM, timed with CUDA events on the library's
stream.  ``e2e`` runs the same step through the host-pointer C ABI with pinned host buffers: the collider is
uploaded once per scene (the reference builds it once), and inside the timed region every step copies in the
level set (once for both solves), the velocity and the applied field, and copies out the corrected velocity and
the total field H (the outputs the reference's callers consume; p and psi stay private in its classes).  The
applied field is prefetched (sf_applied_field_prefetch): its copy runs on a side stream under the pressure solve.

``accuracy`` reports, outside the timed regions, each arm's errors against the oracle's FP64 answer on the same
inputs.  --impl reference times the CPU restatement of the reference's path (the oracle, pinned bit for bit to
the reference's own assembly code; amgcl itself is absent, so its SA-AMG solver is restated) on the host
cores, without loading the CUDA library.  With WORLD_SIZE > 1 every rank runs an independent replica (the path does not
shard; replicas only).
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = "simferrofluid-cuda_gb300"

METRIC = "Poisson solves/s at 256^3 to 1e-6 rel. residual (pressure + magnetic potential)"
UNIT = "solves/s"


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64-arm", action="store_true")
    ap.add_argument("--no-learned-arm", action="store_true")
    ap.add_argument("--no-graph", action="store_true",
                    help="launch each solver iteration's kernels from the host (no CUDA graphs; for kernel profilers "
                         "that do not replay kernels inside conditional graph nodes)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the errors against the oracle's FP64 answer")
    ap.add_argument("--inner-tol", type=float, default=None, help="mixed form: inner relative reduction floor")
    ap.add_argument("--coarse-dim", type=int, default=None)
    ap.add_argument("--pre", type=int, default=None)
    ap.add_argument("--post", type=int, default=None)
    ap.add_argument("--coarse-pre", type=int, default=None, help="smoothing sweeps before restriction, levels >= 2")
    ap.add_argument("--coarse-post", type=int, default=None, help="smoothing sweeps after prolongation, levels >= 2")
    ap.add_argument("--coarse-sweeps", type=int, default=None, help="symmetric sweep pairs on the coarsest level")
    ap.add_argument("--coarse-tail", type=int, default=None,
                    help="levels of at most 65,536 cells: 0 one cluster launch (16 CTAs, else 8), 8 / 16 that "
                         "cluster size, 1 separate kernels")
    ap.add_argument("--smoother", type=int, default=None,
                    help="0 two-colour, 1 fused one-pass, 2 two-colour with FP16 finest-level smoothing coefficients, "
                         "3 (default) as 2 with the finest level stored colour by colour")
    return ap.parse_args(argv)


# ------------------------------------------------------------------------------------------------ distributed
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if _cuda_ok() else "gloo"
        dist.init_process_group(backend)
    return ws, rank, local


def _cuda_ok():
    import torch
    return torch.cuda.is_available()


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if _cuda_ok() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def profiled_columns(summary):
    """(traffic, algorithmic) MB per launch for each captured launch (table column) of the ncu summary
    profiles/<summary>: traffic = dram__bytes_read.sum + dram__bytes_write.sum, written either "R + W Mbyte = T MB"
    or "R + W MB" per column.  [] without a summary or those rows."""
    if not summary:
        return []
    traffic, alg = [], []
    try:
        with open(os.path.join(ROOT, "profiles", summary)) as f:
            for line in f:
                cells = [c.strip() for c in line.strip().strip("|").split("|")]
                if line.startswith("| dram__bytes_read.sum + dram__bytes_write.sum"):
                    for c in cells[1:]:
                        if "=" in c:
                            traffic.append(float(c.split("=")[-1].split("MB")[0]))
                        else:
                            traffic.append(sum(float(x.replace("Mbyte", "").replace("MB", "")) for x in c.split("+")))
                elif line.startswith("| algorithmic bytes per launch"):
                    alg = [float(c.split("MB")[0]) for c in cells[1:]]
    except (OSError, ValueError):
        return []
    return list(zip(traffic, alg)) if traffic and len(traffic) == len(alg) else []


def profiled_traffic(summary, n, per_solve=None):
    """DRAM bytes per launch of the reported kernel from the ncu capture summarised in profiles/<summary> (256^3
    launches).  With per_solve = [(launches, algorithmic bytes per launch), ...] in the capture's column order (the
    bench's pressure and potential launches), each column's traffic is scaled by the bench's algorithmic bytes over
    the capture's and the columns are averaged over the launches; otherwise the single column is scaled by n^3
    cells.  None without a capture."""
    cols = profiled_columns(summary)
    if not cols:
        return None
    if per_solve and len(per_solve) == len(cols) and sum(k for k, _ in per_solve) > 0:
        tot = sum(k * t * (b / (a * 1e6)) for (k, b), (t, a) in zip(per_solve, cols))
        return round(tot * 1e6 / sum(k for k, _ in per_solve))
    return round(cols[0][0] * 1e6 * (n / 256.0) ** 3)


# ------------------------------------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.dev = device_index
        self.proc = None
        self.lines = []
        self.th = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.th:
            self.th.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------------ our arm
def run_ours(args, ws, rank, local):
    import torch
    pkg = importlib.import_module(PKG)
    scenes = importlib.import_module(PKG + ".scenes")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    # torch work (velocity reset) and the library share one stream, so CUDA events on it bracket both
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    ctx = pkg.Context(local, stream=stream.cuda_stream)

    t0 = time.time()
    sc = scenes.pool_sphere(args.n, seed=1234 + rank)
    t_scene = time.time() - t0
    g = sc.grid
    P = pkg.Pressure(g, ctx)
    M = pkg.MagneticField(g, sc.chi, sc.band_width, ctx)

    def todev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    phi = todev(sc.phi)
    frac = [todev(f) for f in sc.frac]
    vel0 = [todev(v) for v in sc.vel]
    vel = [v.clone() for v in vel0]
    hext = [todev(h) for h in sc.hext]
    p_out = torch.zeros(g.shape, dtype=torch.float64, device=dev)
    psi = torch.zeros(g.shape, dtype=torch.float64, device=dev)
    H = [torch.zeros(g.face_shape(a), dtype=torch.float64, device=dev) for a in range(3)]
    torch.cuda.synchronize(dev)

    full_sweeps = [0]  # FP64 arms: 1 sweeps every row, including rows without an active cell

    def opts(which, precision, profile=0):
        kw = {}
        for name, key in (("inner_tol", "inner_tol"), ("coarse_dim", "coarse_dim"), ("pre", "pre_smooth"),
                          ("coarse_pre", "coarse_pre"), ("coarse_post", "coarse_post"),
                          ("post", "post_smooth"), ("smoother", "smoother"),
                          ("coarse_tail", "coarse_tail"), ("coarse_sweeps", "coarse_sweeps")):
            v = getattr(args, name)
            if v is not None:
                kw[key] = v
        if args.no_graph:
            kw["use_graph"] = 0
        return pkg.options(which, precision=precision, tol=args.tol, warm_start=0, report_ref_residual=0,
                           profile=profile, full_sweeps=full_sweeps[0], **kw)

    def step(precision, profile=0, record=None):
        # the learned form is the mixed solver with the network's correction steps (SF_PREC_LEARNED)
        for a in range(3):
            vel[a].copy_(vel0[a])
        sp = P.project(vel, phi, frac, opts=opts("pressure", precision, profile), device=True, p_out=p_out)
        sm = M.solve(phi, hext, opts=opts("magnetic", precision, profile), device=True, psi_out=psi, H_out=H)
        if record is not None:
            record.append((sp, sm))
        return sp, sm

    def timed(precision, steps, warmup, clocks=False):
        for _ in range(warmup):
            step(precision)
        rec = []
        barrier(ws)
        torch.cuda.synchronize(dev)
        cs = ClockSampler(local) if clocks else None
        if cs:
            cs.start()
            time.sleep(0.5)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step(precision, record=rec)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        barrier(ws)
        clk = cs.stop() if cs else None
        ms = e0.elapsed_time(e1)
        return max_over_ranks(ws, ms), rec, clk

    # headline arm
    ms, rec, clk = timed(args.precision, args.steps, args.warmup, clocks=True)
    value = 2 * args.steps * ws / (ms / 1e3)
    it_p = [r[0]["iters"] for r in rec]
    it_m = [r[1]["iters"] for r in rec]
    res_p = max(r[0]["rel_residual"] for r in rec)
    res_m = max(r[1]["rel_residual"] for r in rec)
    launches = sum(r[0]["kernel_launches"] + r[1]["kernel_launches"] for r in rec) + 3 * args.steps

    # plain FP64 MGPCG arm (the denominator of the mixed-precision speed-up)
    # the plain FP64 arm skips rows without an active cell on every level, as the mixed form does (the
    # equally optimised denominator); the second FP64 arm sweeps every row
    fp64 = fp64_full = None
    if not args.no_fp64_arm and args.precision != "fp64":
        n64 = max(2, args.steps // 2)
        for full in (0, 1):
            full_sweeps[0] = full
            ms64, rec64, _ = timed("fp64", n64, 2)
            arm = {"solves_per_s": 2 * n64 * ws / (ms64 / 1e3), "ms_per_step": ms64 / n64,
                   "iters_pressure": [r[0]["iters"] for r in rec64], "iters_magnetic": [r[1]["iters"] for r in rec64]}
            if full:
                fp64_full = arm
            else:
                fp64 = arm
        full_sweeps[0] = 0

    # mixed + learned arm: the mixed solver with the trained U-Net's correction steps at the start of every inner
    # solve (weights/unet.f32; the plain MGPCG finishes every solve and the FP64 residual judges it)
    learned = None
    if not args.no_learned_arm and args.precision == "mixed":
        wpath = os.path.join(ROOT, PKG, "weights", "unet.f32")
        net = pkg.Network(ctx)
        net.load(wpath)
        ctx.set_network(net)
        nl = max(2, args.steps // 2)
        msl, recl, _ = timed("learned", nl, 2)
        ctx.set_network(None)
        net.close()
        learned = {"solves_per_s": 2 * nl * ws / (msl / 1e3), "ms_per_step": msl / nl,
                   "weights": os.path.relpath(wpath, ROOT),
                   "iters_pressure": [r[0]["iters"] for r in recl], "iters_magnetic": [r[1]["iters"] for r in recl],
                   "learned_steps": [[r[0]["learned_steps"], r[1]["learned_steps"]] for r in recl],
                   "guess_energy_ratio": [[round(r[0]["guess_energy_ratio"], 4), round(r[1]["guess_energy_ratio"], 4)]
                                          for r in recl],
                   "max_rel_residual": max(max(r[0]["rel_residual"], r[1]["rel_residual"]) for r in recl)}
        if fp64:
            learned["speedup_vs_fp64"] = round(learned["solves_per_s"] / fp64["solves_per_s"], 3)

    # dominant kernel: finest-level red-black smoother, timed live with CUDA events on the library's stream in
    # a profiled pass of the same workload (opts.profile: every finest-level smoother launch bracketed by events)
    prec = []
    for _ in range(2):
        step(args.precision, profile=1, record=prec)
    sp, sm = prec[-1]
    n_launch = sp["smooth_launches"] + sm["smooth_launches"]
    ms_tot = sp["smooth_ms"] + sm["smooth_ms"]
    bytes_tot = sp["smooth_bytes"] + sm["smooth_bytes"]
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    achieved = bytes_tot / (ms_tot / 1e3) / 1e9 if ms_tot > 0 else 0.0
    smoother = 3 if args.smoother is None else args.smoother
    if smoother == 1:
        kname = "k_rbgs_tma (one full red-black sweep per launch, TMA-staged)"
        prof = "k_rbgs_tma_pool_sphere_256.md"
    elif smoother == 3 and args.precision == "mixed" and args.n % 8 == 0:
        kname = "k_rbgs4s<__half> (one colour of a red-black sweep per launch, colour-split level, FP16 operator copy)"
        prof = "k_rbgs4s_f16_split_finest_pool_sphere_256.md"
    elif smoother in (2, 3) and args.precision == "mixed":
        kname = "k_rbgs4<__half> (one colour of a red-black sweep per launch, FP16 operator copy)"
        prof = "k_rbgs4_f16_finest_pool_sphere_256.md"
    else:
        kname = "k_rbgs (one colour of a red-black sweep per launch)"
        prof = "k_rbgs_f32_finest_pool_sphere_256.md" if args.precision == "mixed" else None
    split = smoother == 3 and args.precision == "mixed" and args.n % 8 == 0
    try:  # a reporting figure from the committed capture: never allowed to fail the bench
        per_solve = [(r["smooth_launches"], r["smooth_bytes"] / max(r["smooth_launches"], 1)) for r in (sp, sm)]
        traffic = profiled_traffic(prof, args.n, per_solve if split else None)
    except Exception:
        traffic = None
    roofline = {"bound": "hbm", "kernel": kname + ", finest level",
                "achieved": round(achieved, 1), "peak": peak, "peak_source": peak_src, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic,
                "bytes_per_launch": bytes_tot / max(n_launch, 1), "ms_per_launch": ms_tot / max(n_launch, 1),
                "per_solve": {k: {"bytes_per_launch": r["smooth_bytes"] / max(r["smooth_launches"], 1),
                                  "ms_per_launch": r["smooth_ms"] / max(r["smooth_launches"], 1)}
                              for k, r in (("pressure", sp), ("magnetic", sm))},
                "launches_timed": n_launch}

    # e2e: host pointers, pinned buffers
    e2e = None
    if not args.no_e2e:
        def pinned(a):
            t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
            t.numpy()[...] = a
            return t.numpy()
        phi_h = pinned(sc.phi)
        frac_h = [pinned(f) for f in sc.frac]
        vel0_h = [np.array(v) for v in sc.vel]
        vel_h = [pinned(v) for v in sc.vel]
        hext_h = [pinned(h) for h in sc.hext]
        H_h = [pinned(np.zeros(g.face_shape(a))) for a in range(3)]
        # the collider is built once per scene (Collider::Finish at initialisation) and stays on the device
        ctx.upload_collider(g, frac_h)

        def estep():
            # per substep: the level set once for both solves, the velocity and the applied field in; the
            # corrected velocity and the total field H out (what the reference's callers consume; p and psi
            # stay private in the reference's classes)
            for a in range(3):
                np.copyto(vel_h[a], vel0_h[a])
            t = time.perf_counter()
            ctx.upload_level_set(g, phi_h)
            ctx.prefetch_applied_field(g, hext_h)  # copied under the pressure solve
            sp = P.project(vel_h, None, None, opts=opts("pressure", args.precision), p_out=False)
            smm = M.solve(None, None, opts=opts("magnetic", args.precision), psi_out=False, H_out=H_h)
            return time.perf_counter() - t, sp, smm

        for _ in range(max(1, args.warmup)):
            estep()
        tot = 0.0
        h2d = d2h = 0
        esteps = max(2, args.steps // 2)
        for _ in range(esteps):
            dt, sp, smm = estep()
            tot += dt
            h2d = sp["h2d_bytes"] + smm["h2d_bytes"] + phi_h.nbytes
            d2h = sp["d2h_bytes"] + smm["d2h_bytes"]
        tot = max_over_ranks(ws, tot)
        e2e = {"value": round(2 * esteps * ws / tot, 3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "steps": esteps}

    out = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64/f32/f16" if args.precision == "mixed" else "f64",
        "data": "synthetic (seeded pool+sphere scene, no dataset)",
        "config": {"workload": f"pool_sphere {args.n}^3 chi=2 dipole field, pressure+potential per step, "
                               f"{args.precision} MGPCG to {args.tol:g} from zero",
                   "grid": [args.n] * 3, "precision": args.precision, "tol": args.tol,
                   "l2": "inputs larger than L2 (each field 134 MB at 256^3)", "parallelism": f"replicas x{ws}",
                   "solver": {k: getattr(args, k)
                              for k in ("inner_tol", "coarse_dim", "pre", "post", "coarse_pre", "coarse_post", "smoother",
                                        "coarse_tail", "coarse_sweeps")
                              if getattr(args, k) is not None}},
        "iters": {"pressure": it_p, "magnetic": it_m}, "max_rel_residual": {"pressure": res_p, "magnetic": res_m},
        "fp64_mgpcg": fp64,
        "speedup_vs_fp64": round(value / fp64["solves_per_s"], 3) if fp64 else None,
        "fp64_mgpcg_full_sweeps": fp64_full,
        "speedup_vs_fp64_full_sweeps": round(value / fp64_full["solves_per_s"], 3) if fp64_full else None,
        "mixed_learned": learned,
        "roofline": roofline, "clocks": clk, "e2e": e2e, "gpu_launches": int(launches),
        "scene_build_s": round(t_scene, 2),
    }
    ctx_bytes = ctx.device_bytes()
    out["device_bytes"] = ctx_bytes
    if rank == 0 and not args.no_accuracy:
        # errors of one step of each arm against the oracle's FP64 answer (outside every timed region)
        res = {}
        for precision in [args.precision] + (["fp64"] if fp64 else []):
            step(precision)
            torch.cuda.synchronize(dev)
            res[precision] = ([v.cpu().numpy() for v in vel], p_out.cpu().numpy(), psi.cpu().numpy())
        # the headline form at the reference's own tolerances: amgcl's default 1e-8 for the pressure
        # (core/Pressure.cpp:125-135) and 1e-6 for the potential (core/MagneticField.cpp:93)
        for a in range(3):
            vel[a].copy_(vel0[a])
        o = opts("pressure", args.precision)
        o.tol = 1e-8
        P.project(vel, phi, frac, opts=o, device=True, p_out=p_out)
        o = opts("magnetic", args.precision)
        o.tol = 1e-6
        M.solve(phi, hext, opts=o, device=True, psi_out=psi, H_out=H)
        torch.cuda.synchronize(dev)
        res[args.precision + " at tol 1e-8 / 1e-6"] = ([v.cpu().numpy() for v in vel], p_out.cpu().numpy(),
                                                        psi.cpu().numpy())
        out["accuracy"] = accuracy(sc, res)
    return out


def accuracy(sc, results, tol=1e-10):
    """Per solve: relative L2 and max|delta| of p (liquid cells) and psi, and the post-projection max|div u|
    (weighted divergence over liquid cells), against the oracle's FP64 answer -- the reference's assembly
    (pinned bit for bit to the reference's own code) solved with the restated SA-AMG to ``tol``."""
    from oracle import oracle as O
    scenes = importlib.import_module(PKG + ".scenes")
    O.build()
    og = O.Grid(*sc.grid.shape, sc.grid.spacing, tuple(sc.grid.origin))
    t = time.perf_counter()
    u_or, p_or, ip = O.pressure_project(og, sc.phi, sc.frac, sc.vel, tol=tol, maxit=100, solver="amg")
    psi_or, _, im = O.magnetic_solve(og, sc.phi, sc.chi, sc.band_width, sc.hext, tol=tol, maxit=100, solver="amg")
    liq = sc.phi <= 0
    full = liq & scenes.full_weight_cells(sc.grid, sc.frac)

    def div_max(v):
        d = np.abs(scenes.divergence(sc.grid, v, sc.frac))
        return float(d[full].max()), float(d[liq].max())

    dv = div_max(u_or)
    out = {"oracle": {"tol": tol, "relres_pressure": ip["relres"], "relres_potential": im["relres"],
                      "max_div_u": dv[0], "max_div_u_partial_faces": dv[1],
                      "seconds": round(time.perf_counter() - t, 1)},
           "note": "max_div_u over liquid cells whose faces are fully open or closed (the projection makes it "
                   "vanish there up to the residual); max_div_u_partial_faces over all liquid cells, where partly "
                   "open wall faces leave a divergence in the reference's discretisation as well"}
    for prec, (vel, p, psi) in results.items():
        dp = np.abs(p[liq] - p_or[liq])
        dpsi = np.abs(psi - psi_or)
        dv = div_max(vel)
        out[prec] = {
            "pressure": {"rel_l2": float(np.linalg.norm(p[liq] - p_or[liq]) / np.linalg.norm(p_or[liq])),
                         "max_dp": float(dp.max()), "max_dp_rel": float(dp.max() / np.abs(p_or[liq]).max()),
                         "max_div_u": dv[0], "max_div_u_partial_faces": dv[1]},
            "potential": {"rel_l2": float(np.linalg.norm(psi - psi_or) / np.linalg.norm(psi_or)),
                          "max_dpsi": float(dpsi.max()), "max_dpsi_rel": float(dpsi.max() / np.abs(psi_or).max())}}
    return out


# ------------------------------------------------------------------------------------------------ CPU arm
def _cpu_scene(n):
    """The bench scene for the CPU arm, built without the CUDA library: the scene's level set, velocity and
    field (numpy) and the oracle's collider fractions (bit-identical to the reference's Collider)."""
    from oracle import oracle as O
    O.build()
    scenes = importlib.import_module(PKG + ".scenes")
    sc = scenes.pool_sphere(n, seed=1234, with_fractions=False)
    og = O.Grid(*sc.grid.shape, sc.grid.spacing, tuple(sc.grid.origin))
    sc.frac = O.box_collider_fractions(og, 0)
    return O, sc, og


def _cpu_step(O, sc, og, tol, solver="amg"):
    """One substep on the CPU: Pressure::Project and MagneticField::Solve, each assembling its matrix (the
    reference's assembly, restated) and solving to tol from zero, with solver "amg" (the restated amgcl path:
    SA-AMG hierarchy rebuilt per solve, BiCGStab / CG) or "mgpcg" (the library's plain FP64 geometric-MG PCG on
    the host cores)."""
    t = time.perf_counter()
    _, _, ip = O.pressure_project(og, sc.phi, sc.frac, sc.vel, tol=tol, solver=solver)
    _, _, im = O.magnetic_solve(og, sc.phi, sc.chi, sc.band_width, sc.hext, tol=tol, solver=solver)
    return time.perf_counter() - t, ip["iters"], im["iters"]


def cpu_baseline(args, n=None, steps=1):
    """The oracle (CPU restatement of the reference's assembly + amgcl SA-AMG solves) on the same scene."""
    n = n or args.n
    O, sc, og = _cpu_scene(n)
    tot, its = 0.0, []
    for _ in range(steps):
        dt, ip, im = _cpu_step(O, sc, og, args.tol)
        tot += dt
        its.append((ip, im))
    return {"value": round(2 * steps / tot, 4), "unit": UNIT, "cores": O.num_threads(), "kind": "port",
            "sample": f"pool_sphere {n}^3, {steps} substep(s) = {2 * steps} solves (assembly + SA-AMG setup + "
                      f"BiCGStab/CG to {args.tol:g}), {tot:.1f} s, iterations (pressure, potential) {its}"}


def cpu_mgpcg_fp64(args, n=None):
    """The library's plain FP64 method (geometric-MG PCG, oracle/sf_mgcpu.c) on the host cores, same scene and
    tolerance: one warm-up substep, then one timed substep (assembly + face form + MGPCG + projection / H)."""
    n = n or args.n
    O, sc, og = _cpu_scene(n)
    _cpu_step(O, sc, og, args.tol, solver="mgpcg")
    dt, ip, im = _cpu_step(O, sc, og, args.tol, solver="mgpcg")
    return {"value": round(2 / dt, 4), "unit": UNIT, "cores": O.num_threads(), "kind": "port",
            "sample": f"pool_sphere {n}^3, 1 substep = 2 solves (assembly + MGPCG V(2,2) to {args.tol:g} from "
                      f"zero), {dt:.2f} s, iterations (pressure, potential) ({ip}, {im})"}


def run_reference(args, ws, rank):
    if rank != 0:
        return None
    O, sc, og = _cpu_scene(args.n)
    warm = min(args.warmup, 1)
    steps = max(1, min(args.steps, 3))
    for _ in range(warm):
        _cpu_step(O, sc, og, args.tol)
    tot, its = 0.0, []
    for _ in range(steps):
        dt, ip, im = _cpu_step(O, sc, og, args.tol)
        tot += dt
        its.append((ip, im))
    v = round(2 * steps / tot, 4)
    sample = (f"pool_sphere {args.n}^3, {steps} timed substep(s) after {warm} warm-up (requested --steps "
              f"{args.steps} --warmup {args.warmup}, capped to keep the CPU run within minutes), "
              f"iterations (pressure, potential) {its}")
    cb = {"value": v, "unit": UNIT, "cores": O.num_threads(), "kind": "port", "sample": sample}
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": steps, "warmup": warm,
            "ms_per_step": round(1000.0 * tot / steps, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded pool+sphere scene)", "impl": "reference",
            "config": {"workload": f"pool_sphere {args.n}^3 chi=2 dipole field, pressure+potential per step, "
                                   f"CPU restatement of the reference path (assembly + SA-AMG/SPAI-0 "
                                   f"BiCGStab/CG) to {args.tol:g} from zero", "grid": [args.n] * 3, "tol": args.tol},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    ws, rank, local = dist_init()
    if args.impl == "reference":
        out = run_reference(args, ws, rank)
        if rank == 0 and out is not None:
            print(json.dumps(out))
        return
    out = run_ours(args, ws, rank, local)
    if rank == 0:
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(args)
            out["cpu_mgpcg_fp64"] = cpu_mgpcg_fp64(args)
        print(json.dumps(out))


if __name__ == "__main__":
    main()
