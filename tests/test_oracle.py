"""CPU tests of the oracle: pinned against the independent pure-Python restatement (golden fixtures) and
against the known-answer tests of the hot path.  No GPU involved."""
import os

import numpy as np
import pytest

from conftest import rel_l2, scenes

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return z


def _grid(O, z):
    return O.Grid(*[int(v) for v in z["shape"]], float(z["h"]), tuple(float(v) for v in z["origin"]))


@pytest.mark.parametrize("name", ["case_a", "case_b"])
def test_oracle_pressure_matches_golden(oracle, name):
    z = _load(name)
    g = _grid(oracle, z)
    f = lambda k: [z[f"{k}{a}"] for a in range(3)]  # noqa: E731
    A, b, g2m, m2g = oracle.pressure_assemble(g, z["phi"], f("frac"), f("u"), f("us"), f("jump"),
                                              float(z["vol_error"]))
    assert np.array_equal(g2m, z["p_g2m"]) and np.array_equal(m2g, z["p_m2g"])
    assert np.array_equal(A.rowptr, z["p_rowptr"]) and np.array_equal(A.col, z["p_col"])
    assert np.array_equal(A.val, z["p_val"])  # bit-exact
    assert np.array_equal(b, z["p_rhs"])
    up = oracle.pressure_apply(g, z["phi"], f("frac"), f("jump"), g2m, z["p_sol"], f("u"))
    for a in range(3):
        assert np.array_equal(up[a], z[f"u_proj{a}"])


@pytest.mark.parametrize("name", ["case_a", "case_b"])
def test_oracle_magnetic_matches_golden(oracle, name):
    z = _load(name)
    g = _grid(oracle, z)
    hext = [z[f"hext{a}"] for a in range(3)]
    mu = oracle.magnetic_coeff(g, z["phi"], float(z["chi"]), float(z["bw"]))
    for a in range(3):
        # sin() is the platform libm's in both: allow 1 ulp of chi in the band
        assert np.abs(mu[a] - z[f"mu{a}"]).max() <= 4e-16 * float(z["chi"])
    A = oracle.magnetic_assemble(g, [z[f"mu{a}"] for a in range(3)])
    assert np.array_equal(A.rowptr, z["m_rowptr"]) and np.array_equal(A.col, z["m_col"])
    assert np.array_equal(A.val, z["m_val"])
    b, _ = oracle.magnetic_rhs(g, [z[f"mu{a}"] for a in range(3)], hext)
    assert np.array_equal(b, z["m_rhs"])
    H = oracle.magnetic_total_field(g, z["psi"], hext)
    for a in range(3):
        assert np.array_equal(H[a], z[f"H{a}"])


def test_restatement_regenerates_fixture():
    """The committed fixture is exactly what the restatement script produces."""
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden
    out = make_golden.generate("case_a")
    z = _load("case_a")
    for k, v in out.items():
        assert np.array_equal(np.asarray(v), z[k]), k


def test_scipy_cross_check(oracle):
    """The oracle's PCG solution equals a direct sparse solve of the same CSR system."""
    sp = pytest.importorskip("scipy.sparse.linalg")
    sc = scenes().pool(12, seed=3)
    g = oracle.Grid(*sc.grid.shape, sc.grid.spacing)
    A, b, g2m, m2g = oracle.pressure_assemble(g, sc.phi, sc.frac, sc.vel)
    x, it, rr = A.solve(b, tol=1e-13)
    xd = sp.spsolve(A.to_scipy().tocsc(), b)
    assert rel_l2(x, xd) <= 1e-10
    psi, H, info = oracle.magnetic_solve(g, sc.phi, sc.chi, sc.band_width, sc.hext, tol=1e-13)
    xd = sp.spsolve(info["A"].to_scipy().tocsc(), info["b"])
    assert rel_l2(psi.ravel(), xd) <= 1e-9


def test_hydrostatic_kat_oracle(oracle):
    """u = 0, volError = 0, constant jump J -> p == J in every liquid cell, u unchanged."""
    sc = scenes().pool(10, seed=2)
    g = oracle.Grid(*sc.grid.shape, sc.grid.spacing)
    J = -1.25
    jump = [np.full(sc.grid.face_shape(a), J) for a in range(3)]
    zero = [np.zeros(sc.grid.face_shape(a)) for a in range(3)]
    u, p, info = oracle.pressure_project(g, sc.phi, sc.frac, zero, jump=jump, tol=1e-14)
    liq = sc.phi <= 0
    assert np.abs(p[liq] - J).max() <= 1e-11
    for a in range(3):
        assert np.abs(u[a]).max() <= 1e-11


def test_chi_zero_kat_oracle(oracle):
    sc = scenes().pool(8, seed=1)
    g = oracle.Grid(*sc.grid.shape, sc.grid.spacing)
    psi, H, info = oracle.magnetic_solve(g, sc.phi, 0.0, sc.band_width, sc.hext)
    assert np.all(info["b"] == 0) and np.all(psi == 0)
    for a in range(3):
        assert np.array_equal(H[a], sc.hext[a])


def test_neumann_compatibility(oracle):
    """Sum of the unpinned right-hand side is zero: the pinned system equals the Neumann system shifted so
    that psi[0] = 0 (the identity the CUDA solver relies on)."""
    sc = scenes().pool_sphere(12, seed=4)
    g = oracle.Grid(*sc.grid.shape, sc.grid.spacing)
    mu = oracle.magnetic_coeff(g, sc.phi, sc.chi, sc.band_width)
    b, b0 = oracle.magnetic_rhs(g, mu, sc.hext)
    assert abs(b.sum() + b0) <= 1e-12 * np.abs(b).sum()


def test_projection_divergence_free(oracle):
    """After the projection the weighted divergence of fully-liquid interior cells vanishes to the solver
    tolerance (the rhs is the negative weighted divergence)."""
    sc = scenes().pool(16, seed=6)
    g = oracle.Grid(*sc.grid.shape, sc.grid.spacing)
    u, p, info = oracle.pressure_project(g, sc.phi, sc.frac, sc.vel, tol=1e-13)
    A2, b2, _, m2g = oracle.pressure_assemble(g, sc.phi, sc.frac, u)
    # cells whose 6 neighbours are liquid and whose faces are open: rhs of the projected field ~ 0
    liq = (sc.phi <= 0).ravel()
    interior = []
    for r, c in enumerate(m2g):
        i, j, k = np.unravel_index(c, sc.grid.shape)
        if 0 < i < 15 and 0 < j < 15 and 0 < k < 15:
            nbs = [np.ravel_multi_index(t, sc.grid.shape) for t in
                   [(i - 1, j, k), (i + 1, j, k), (i, j - 1, k), (i, j + 1, k), (i, j, k - 1), (i, j, k + 1)]]
            if all(liq[q] for q in nbs):
                interior.append(r)
    assert len(interior) > 100
    assert np.abs(b2[interior]).max() <= 1e-9 * np.abs(info["b"]).max()


def test_slab_kat_oracle(oracle):
    n = 16
    g0 = scenes().unit_grid(n)
    g = oracle.Grid(n, n, n, g0.spacing)
    ys = scenes().cell_centres(g0, 1)
    phi = np.ascontiguousarray(np.broadcast_to((ys - 0.5)[None, :, None], g0.shape))
    chi = 1.0
    psi, H, info = oracle.magnetic_solve(g, phi, chi, 2 * g.h, scenes().uniform_field(g0), tol=1e-13)
    yf = np.arange(n + 1) / n
    inside = (yf > 0.05) & (yf < 0.5 - 3 * g.h)
    assert np.abs(H[1][:, inside, :] - 0.5).max() <= 1e-9


@pytest.mark.parametrize("shape", [(24, 20, 28), (17, 13, 9)])
def test_cpu_mgpcg_matches_pcg(oracle, shape):
    """The CPU geometric-MG PCG (the benchmark's CPU MGPCG FP64 baseline, oracle/sf_mgcpu.c) solves the same
    pressure and (pinned) potential systems as the oracle's Jacobi-PCG: to 1e-10 on a pool+sphere and on a
    ragged grid, in a handful of iterations."""
    import importlib
    S = importlib.import_module(scenes().__name__)
    sc = S.pool_sphere(max(shape), seed=8, with_fractions=False)
    # a ragged grid of the same kind: the scene's fields cropped
    sl = tuple(slice(0, n) for n in shape)
    g = oracle.Grid(*shape, sc.grid.spacing)
    phi = np.ascontiguousarray(sc.phi[sl])
    frac = oracle.box_collider_fractions(g, 0)
    rng = np.random.default_rng(3)
    vel = [rng.normal(0, 0.5, g.face_shape(a)) for a in range(3)]
    hext = [rng.uniform(-1, 1, g.face_shape(a)) + (a == 1) for a in range(3)]
    u1, p1, i1 = oracle.pressure_project(g, phi, frac, vel, tol=1e-10, solver="mgpcg")
    u0, p0, i0 = oracle.pressure_project(g, phi, frac, vel, tol=1e-13)
    liq = phi <= 0
    assert i1["relres"] <= 1e-10 and i1["iters"] <= 20
    assert rel_l2(p1[liq], p0[liq]) <= 1e-8
    psi1, H1, j1 = oracle.magnetic_solve(g, phi, 2.0, 2 * g.h, hext, tol=1e-10, solver="mgpcg")
    psi0, H0, j0 = oracle.magnetic_solve(g, phi, 2.0, 2 * g.h, hext, tol=1e-13)
    assert psi1.ravel()[0] == 0.0 and j1["iters"] <= 20
    r = np.linalg.norm(j0["b"] - j0["A"].matvec(psi1.ravel())) / np.linalg.norm(j0["b"])
    assert r <= 2e-10
    assert rel_l2(psi1, psi0) <= 1e-8
