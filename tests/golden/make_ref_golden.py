"""Generate the reference-pinned fixtures ``tests/golden/ref_*.npz`` from the reference's own code.

The reference's hot-path sources (core/Pressure.cpp, MagneticField.cpp, Collider.cpp, FastMarching.cpp,
Extrapolation.cpp, Reinitialization.cpp, CSG.cpp and the header-only Advection/TriLerp/TriCuInterp) are
compiled unmodified into ``oracle/_ref/libsfref.so`` by ``oracle/ref.mk`` (stand-in headers for Eigen, TBB,
fmt/spdlog, yaml-cpp and the amgcl solver call in ``oracle/refshim``).  This script runs them on seeded inputs
and records what they produce, so that ``tests/test_ref_pin.py`` checks the C oracle against the reference's
outputs wherever the tests run, with or without the reference's sources.

Fixtures:
* ``ref_case_a`` / ``ref_case_b`` -- the inputs of ``case_a`` / ``case_b`` (every branch of the assembly:
  partial fractions, solid velocity, jump, volume error, phi == 0, theta clamping, a non-dyadic spacing and a
  non-zero corner): Pressure::Project's matrix, rhs, unknown numbering and projected velocity for a given
  pressure, Reproject's rhs and initial guess, the tolerance handed to amgcl; MagneticField::Solve's mu,
  matrix, rhs and total field for a given potential, its tolerance, its grid corner and the warm start of a
  second solve.
* ``ref_neighbours`` -- three grids: Collider(sgrid) + Finish (node level set, fractions, normals),
  Extrapolation::Solve with the simulation's predicate, Collider::Enforce, Advection::Solve<2> of the level set
  and of the velocity, Reinitialization::Solve and MagneticField::CalculateVertexPressures.
* ``ref_scenes`` -- SHA-256 digests of the outputs on two full scenes: the reference's plane scene at -s 64
  (demo/SimBuilder.cpp:40-62: (64, 48, 64) cells, h = 0.12/60, boundary width 2, plane 0.024 above the domain
  floor, chi 0.33, H = (0, 6e4, 0)) and the 32^3 pool+sphere scene with the box collider of boundary width 0.

Run (needs the reference's sources):  python tests/golden/make_ref_golden.py
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import make_golden as MG  # noqa: E402
from oracle import ref as R  # noqa: E402


def digest(a) -> str:
    a = np.ascontiguousarray(a)
    dt = {"f": "<f8", "i": "<i8" if a.dtype.itemsize == 8 else "<i4", "u": "<u1", "b": "<u1"}[a.dtype.kind]
    return hashlib.sha256(a.astype(dt).tobytes()).hexdigest()


def case(name):
    shape, h, origin, seed = MG.CASES[name]
    g, phi, frac, u, us, jump, hext = MG.make_inputs(shape, h, origin, seed)
    rng = np.random.default_rng(seed + 100)
    vol_error = 0.0123
    S = R.Session(*shape, h, origin, bw=0)
    S.collider_set(frac=frac, solid_vel=us)
    n = int((phi <= 0).sum())
    p_sol = rng.normal(size=n)
    r = S.pressure_project(phi, u, jump=jump, vol_error=vol_error, mode=1, p_inject=p_sol)
    u2 = [0.5 * a + 0.1 for a in u]
    r2 = S.pressure_project(phi, u2, jump=jump, vol_error=0.02, mode=0, reproject=True)
    chi, bw = 1.3, 2 * h
    psi = rng.normal(size=int(np.prod(shape)))
    m = S.magnetic_solve(chi, bw, phi, hext, mode=1, psi_inject=psi)
    m2 = S.magnetic_solve(chi, bw, phi, hext, mode=0)
    S.close()
    out = dict(shape=np.array(shape), h=np.array(h), origin=np.array(origin), vol_error=np.array(vol_error),
               chi=np.array(chi), bw=np.array(bw), phi=phi, p_sol=p_sol, psi=psi,
               p_rowptr=r["rowptr"], p_col=r["col"], p_val=r["val"], p_rhs=r["rhs"], p_g2m=r["grid2mat"],
               p_tol=np.array(r["tol"]), p_x0=r["x0"],
               rp_vol_error=np.array(0.02), rp_rhs=r2["rhs"], rp_x0=r2["x0"],
               m_rowptr=m["rowptr"], m_col=m["col"], m_val=m["val"], m_rhs=m["rhs"], m_tol=np.array(m["tol"]),
               m_x0=m["x0"], m_origin=m["origin_ext"], m2_x0=m2["x0"])
    for a in range(3):
        out[f"frac{a}"] = frac[a]
        out[f"u{a}"] = u[a]
        out[f"us{a}"] = us[a]
        out[f"jump{a}"] = jump[a]
        out[f"hext{a}"] = hext[a]
        out[f"u_proj{a}"] = r["u"][a]
        out[f"mu{a}"] = m["mu"][a]
        out[f"H{a}"] = m["H"][a]
    return out


NEIGHBOUR_GRIDS = [  # shape, spacing, corner, boundary width
    ((12, 10, 14), 1.0 / 12.0, (0.0, 0.0, 0.0), 0),
    ((10, 9, 8), 0.002, (-0.01, -0.009, -0.008), 2),
    ((9, 8, 7), 1.0 / 8.0, (0.0, 0.0, 0.0), 1),
]


def neighbours():
    out = {}
    for t, (shape, h, origin, bw) in enumerate(NEIGHBOUR_GRIDS):
        rng = np.random.default_rng(40 + t)
        S = R.Session(*shape, h, origin, bw=bw)
        ls, frac, nrm = S.collider_finish()
        fs = [tuple(s + (b == a) for b, s in enumerate(shape)) for a in range(3)]
        y = (np.arange(shape[1]) + 0.5) / shape[1]
        phi = (y[None, :, None] - 0.45) * shape[1] * h + 0.3 * h * rng.uniform(-1, 1, shape)
        u = [rng.uniform(-1, 1, fs[a]) for a in range(3)]
        us = [rng.uniform(-0.2, 0.2, fs[a]) for a in range(3)]
        H = [rng.uniform(-1, 1, fs[a]) for a in range(3)]
        lo = np.array(origin)
        hi = lo + np.array(shape) * h
        pos = lo + rng.uniform(0, 1, (40, 3)) * (hi - lo)
        vn = rng.normal(size=(40, 3))
        vn /= np.linalg.norm(vn, axis=1, keepdims=True)
        dt = 0.3 * h
        ue = S.extrapolate_velocity(u, phi, 0.0, 6)
        S.collider_set(solid_vel=us)
        en = S.collider_enforce(ue)
        al = S.advect_levelset(phi, u, dt)
        av = S.advect_velocity(u, dt)
        ri = S.reinitialize(phi, 10)
        vp = S.vertex_pressures(1.3, H, pos, vn)
        S.close()
        d = dict(shape=np.array(shape), h=np.array(h), origin=np.array(origin), bw=np.array(bw), phi=phi,
                 node_ls=ls, pos=pos, vnormal=vn, dt=np.array(dt), chi=np.array(1.3), advect_ls=al, reinit=ri,
                 vertex_p=vp)
        for a in range(3):
            d.update({f"frac{a}": frac[a], f"normal{a}": nrm[a], f"u{a}": u[a], f"us{a}": us[a], f"H{a}": H[a],
                      f"extrap{a}": ue[a], f"enforce{a}": en[a], f"advect_u{a}": av[a]})
        out.update({f"g{t}_{k}": v for k, v in d.items()})
    return out


def plane_scene_inputs():
    """The reference's plane scene at -s 64 (demo/SimBuilder.cpp:40-62), solve-level inputs."""
    scale, bw, length = 64, 2, 0.12
    h = length / (scale - bw * 2)
    res = (4 * scale // 4, 3 * scale // 4, 4 * scale // 4)
    origin = tuple(-r * h / 2 for r in res)  # StaggeredGrid(2, h, res) with centre 0
    return res, h, origin, bw, length


def scenes():
    out = {}
    # --- the reference's plane scene at -s 64
    res, h, origin, bw, length = plane_scene_inputs()
    S = R.Session(*res, h, origin, bw=bw)
    dom_o, dom_l = S.domain()
    phi = S.csg_union(None, 0, dom_o + np.array([0.0, 1.0, 0.0]) * length * .2, (0.0, 1.0, 0.0))
    ls, frac, nrm = S.collider_finish()
    rng = np.random.default_rng(64)
    fs = [tuple(s + (b == a) for b, s in enumerate(res)) for a in range(3)]
    u = [rng.uniform(-1, 1, fs[a]) for a in range(3)]
    r = S.pressure_project(phi, u, mode=0)
    hext = [np.full(fs[a], (0.0, 6e4, 0.0)[a]) for a in range(3)]
    m = S.magnetic_solve(0.33, 2 * h, phi, hext, mode=0)
    S.close()
    out["plane_meta"] = np.array([res[0], res[1], res[2], bw, 64])
    out["plane_h"] = np.array(h)
    out["plane_origin"] = np.array(origin)
    out["plane_domain_origin"] = dom_o
    for k, v in [("phi", phi), ("node_ls", ls), ("p_rowptr", r["rowptr"]), ("p_col", r["col"]),
                 ("p_val", r["val"]), ("p_rhs", r["rhs"]), ("m_rowptr", m["rowptr"]), ("m_col", m["col"]),
                 ("m_val", m["val"]), ("m_rhs", m["rhs"])] + \
            [(f"frac{a}", frac[a]) for a in range(3)] + [(f"normal{a}", nrm[a]) for a in range(3)] + \
            [(f"u_in{a}", u[a]) for a in range(3)] + [(f"mu{a}", m["mu"][a]) for a in range(3)]:
        out["plane_sha_" + k] = np.array(digest(v))
    # --- pool + sphere at 32^3 (pool depth 0.2, sphere r 0.15 at (0.5, 0.55, 0.5)), box collider bw 0
    n = 32
    h = 1.0 / n
    S = R.Session(n, n, n, h, (0.0, 0.0, 0.0), bw=0)
    phi = S.csg_union(None, 0, (0.0, 0.2, 0.0), (0.0, 1.0, 0.0))
    phi = S.csg_union(phi, 1, (0.5, 0.55, 0.5), r=0.15)
    ls, frac, nrm = S.collider_finish()
    rng = np.random.default_rng(32)
    fs = [(n + (a == 0), n + (a == 1), n + (a == 2)) for a in range(3)]
    u = [rng.normal(0.0, 0.5, fs[a]) for a in range(3)]
    hext = [rng.uniform(-1, 1, fs[a]) + (1.0 if a == 1 else 0.0) for a in range(3)]
    r = S.pressure_project(phi, u, mode=0)
    m = S.magnetic_solve(2.0, 2 * h, phi, hext, mode=0)
    S.close()
    for k, v in [("phi", phi), ("p_rowptr", r["rowptr"]), ("p_col", r["col"]), ("p_val", r["val"]),
                 ("p_rhs", r["rhs"]), ("m_rowptr", m["rowptr"]), ("m_col", m["col"]), ("m_val", m["val"]),
                 ("m_rhs", m["rhs"])] + [(f"frac{a}", frac[a]) for a in range(3)] + \
            [(f"u_in{a}", u[a]) for a in range(3)] + [(f"hext{a}", hext[a]) for a in range(3)] + \
            [(f"mu{a}", m["mu"][a]) for a in range(3)]:
        out["ps32_sha_" + k] = np.array(digest(v))
    return out


def main():
    if R.build() is None:
        raise SystemExit("the reference's sources are not available; nothing generated")
    for name in ("case_a", "case_b"):
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **case(name))
        print("wrote", f"ref_{name}")
    np.savez_compressed(os.path.join(HERE, "ref_neighbours.npz"), **neighbours())
    print("wrote ref_neighbours")
    np.savez_compressed(os.path.join(HERE, "ref_scenes.npz"), **scenes())
    print("wrote ref_scenes")


if __name__ == "__main__":
    main()
