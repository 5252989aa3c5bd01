"""Generate the golden fixtures under tests/golden/ from the pure-Python restatement (restate.py).

The reference has no tests or golden vectors of its own and cannot be built here, so these fixtures pin the
C oracle to an independent restatement of the reference's code on small seeded inputs that exercise every
branch of the assembly: liquid/air/solid faces, partial face weights, phi == 0 cells, theta clamping, a
nonzero solid velocity, a jump array, a volume error, a non-zero grid origin and a spacing that is not a
power of two (so TriLerp's weights are inexact).

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import restate as R  # noqa: E402

CASES = {
    # name: (shape, spacing, origin, seed)
    "case_a": ((6, 5, 7), 1.0 / 6.0, (0.0, 0.0, 0.0), 11),
    "case_b": ((8, 6, 8), 0.12 / 60.0, (-0.064, -0.048, -0.064), 12),
}


def make_inputs(shape, h, origin, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    g = R.G(nx, ny, nz, h, origin)
    y = (np.arange(ny) + 0.5) / ny
    phi = (y[None, :, None] - 0.45) * ny * h + 0.3 * h * rng.uniform(-1, 1, shape)
    phi[rng.uniform(size=shape) < 0.05] = 0.0  # phi == 0 is liquid
    phi[1, ny - 2, 2] = -0.5 * h  # a liquid cell in the air
    frac = []
    for a in range(3):
        fs = g.fshape(a)
        f = np.where(rng.uniform(size=fs) < 0.6, 0.0, rng.uniform(0, 0.9, fs))
        f[rng.uniform(size=fs) < 0.08] = 1.0
        sl = [slice(None)] * 3
        sl[a] = 0
        f[tuple(sl)] = 1.0
        sl[a] = -1
        f[tuple(sl)] = 1.0
        frac.append(f)
    u = [rng.uniform(-1, 1, g.fshape(a)) for a in range(3)]
    us = [rng.uniform(-0.2, 0.2, g.fshape(a)) for a in range(3)]
    jump = [rng.uniform(-0.5, 0.5, g.fshape(a)) for a in range(3)]
    hext = [rng.uniform(-1, 1, g.fshape(a)) + (1.0 if a == 1 else 0.0) for a in range(3)]
    return g, phi, frac, u, us, jump, hext


def generate(name):
    shape, h, origin, seed = CASES[name]
    g, phi, frac, u, us, jump, hext = make_inputs(shape, h, origin, seed)
    rng = np.random.default_rng(seed + 100)
    vol_error = 0.0123
    fl = lambda arrs: [list(a.ravel()) for a in arrs]  # noqa: E731
    rows, rhs, g2m, m2g = R.pressure_assemble(g, list(phi.ravel()), fl(frac), fl(u), fl(us), fl(jump), vol_error)
    rowptr, col, val = R.rows_to_csr(rows)
    p = rng.normal(size=len(m2g))
    u_proj = R.pressure_apply(g, list(phi.ravel()), fl(frac), fl(jump), g2m, list(p), fl(u))
    chi, bw = 1.3, 2 * h
    mu = R.magnetic_coeff(g, list(phi.ravel()), chi, bw)
    mrows = R.magnetic_assemble(g, mu)
    mrowptr, mcol, mval = R.rows_to_csr(mrows)
    mrhs = R.magnetic_rhs(g, mu, fl(hext))
    psi = rng.normal(size=g.N)
    H = R.magnetic_total_field(g, list(psi), fl(hext))
    out = dict(shape=np.array(shape), h=np.array(h), origin=np.array(origin), vol_error=np.array(vol_error),
               chi=np.array(chi), bw=np.array(bw), phi=phi,
               p_rowptr=rowptr, p_col=col, p_val=val, p_rhs=np.array(rhs), p_g2m=np.array(g2m, np.int32),
               p_m2g=np.array(m2g, np.int64), p_sol=p,
               m_rowptr=mrowptr, m_col=mcol, m_val=mval, m_rhs=np.array(mrhs), psi=psi)
    for a in range(3):
        out[f"frac{a}"] = frac[a]
        out[f"u{a}"] = u[a]
        out[f"us{a}"] = us[a]
        out[f"jump{a}"] = jump[a]
        out[f"hext{a}"] = hext[a]
        out[f"u_proj{a}"] = np.array(u_proj[a]).reshape(g.fshape(a))
        out[f"mu{a}"] = np.array(mu[a]).reshape(g.fshape(a))
        out[f"H{a}"] = np.array(H[a]).reshape(g.fshape(a))
    return out


def main():
    for name in CASES:
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **generate(name))
        print("wrote", name)


if __name__ == "__main__":
    main()
