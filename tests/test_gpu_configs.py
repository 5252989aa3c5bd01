"""The benchmark configurations on the GPU against the oracle's FP64 solution of the same discrete systems.

The oracle's assembly is the reference's own (tests/test_ref_pin.py), so its tightly solved systems are the
reference's answer up to amgcl's stopping tolerance.  Each test reports, per solve, the relative residual on
the reference's operator, the relative L2 error and max|delta| of p (liquid cells) and psi, and the
post-projection max|div u| (weighted divergence over liquid cells whose faces are fully open or closed, where
the projection makes it vanish up to the residual; and over all liquid cells) next to the oracle's own.

* 64^3 pool (dx = 1/64, depth 0.25 with a 1% seeded perturbation, chi 1, uniform vertical field, walls on the
  grid faces), both solves in FP64 and in the mixed form to 1e-8: within 1e-5 relative L2 of the oracle.
* The reference's plane scene at -s 64 (demo/SimBuilder.cpp:40-62: (64, 48, 64) cells, h = 0.12/60, boundary
  width 2, chi 0.33, H = (0, 6e4, 0)) at the reference's own tolerances (1e-8 pressure, amgcl's default;
  1e-6 potential, core/MagneticField.cpp:93): within 1e-5 relative L2.
* 192^3 (the same pool at dx = 1/192) in FP64 MGPCG and in the mixed form, to 1e-6 as the configuration asks
  (errors reported; the relative L2 is bounded by the condition number times the residual), and to the
  reference's tolerances, where both are within 1e-5 relative L2 of the oracle.
"""
import numpy as np
import pytest

from conftest import oracle_grid, pkg, rel_l2, scenes

pytestmark = pytest.mark.gpu


def _oracle_solutions(O, og, sc, frac, tol=1e-11):
    """The oracle's FP64 answer: the reference's assembly solved with the restated SA-AMG to tol."""
    u_or, p_or, ip = O.pressure_project(og, sc.phi, frac, sc.vel, tol=tol, maxit=100, solver="amg")
    psi_or, H_or, im = O.magnetic_solve(og, sc.phi, sc.chi, sc.band_width, sc.hext, tol=tol, maxit=100,
                                        solver="amg")
    assert ip["relres"] <= 10 * tol and im["relres"] <= 10 * tol
    return u_or, p_or, psi_or, H_or


def _errors(S, sc, frac, liq, P, M, vel, u_or, p_or, psi_or):
    dp = P.pressure[liq] - p_or[liq]
    dpsi = M.potential - psi_or
    full = liq & S.full_weight_cells(sc.grid, frac)
    div, div_or = S.divergence(sc.grid, vel, frac), S.divergence(sc.grid, u_or, frac)
    return dict(rel_l2_p=rel_l2(P.pressure[liq], p_or[liq]),
                max_dp=float(np.abs(dp).max()), max_dp_rel=float(np.abs(dp).max() / np.abs(p_or[liq]).max()),
                rel_l2_psi=rel_l2(M.potential, psi_or), max_dpsi=float(np.abs(dpsi).max()),
                max_dpsi_rel=float(np.abs(dpsi).max() / np.abs(psi_or).max()),
                max_div_u=float(np.abs(div[full]).max()), max_div_u_oracle=float(np.abs(div_or[full]).max()),
                max_div_u_all=float(np.abs(div[liq]).max()), max_div_u_all_oracle=float(np.abs(div_or[liq]).max()))


def _solve(sfpkg, ctx, sc, frac, precision, tol_p, tol_m):
    vel = [a.copy() for a in sc.vel]
    P = sfpkg.Pressure(sc.grid, ctx)
    sp = P.project(vel, sc.phi, frac, opts=sfpkg.options("pressure", precision=precision, tol=tol_p))
    M = sfpkg.MagneticField(sc.grid, sc.chi, sc.band_width, ctx)
    sm = M.solve(sc.phi, sc.hext, opts=sfpkg.options("magnetic", precision=precision, tol=tol_m, warm_start=0))
    assert sp["converged"] == 1 and sp["rel_residual"] <= tol_p * 1.01, sp
    assert sm["converged"] == 1 and sm["rel_residual_ref"] <= tol_m * 1.05, sm
    return P, M, vel, sp, sm


def _report(tag, prec, sp, sm, e):
    print(f"{tag} {prec}: iters {sp['iters']}/{sm['iters']} relres {sp['rel_residual']:.2e}/"
          f"{sm['rel_residual_ref']:.2e} relL2 p {e['rel_l2_p']:.2e} psi {e['rel_l2_psi']:.2e} "
          f"max|dp|/max|p| {e['max_dp_rel']:.2e} max|dpsi|/max|psi| {e['max_dpsi_rel']:.2e} "
          f"max|div u| {e['max_div_u']:.2e} (oracle {e['max_div_u_oracle']:.2e}; with partly open faces "
          f"{e['max_div_u_all']:.2e}, oracle {e['max_div_u_all_oracle']:.2e})")


@pytest.fixture(scope="module")
def pool64(oracle):
    S = scenes()
    sc = S.pool(64, seed=1, chi=1.0)
    og = oracle_grid(oracle, sc.grid)
    return sc, og, _oracle_solutions(oracle, og, sc, sc.frac)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_config_64_vs_oracle(sfpkg, oracle, gpu_ctx, pool64, precision):
    """64^3 pool, both solves to 1e-8: p and psi within 1e-5 relative L2 of the oracle's FP64 answer."""
    S = scenes()
    sc, og, (u_or, p_or, psi_or, H_or) = pool64
    liq = sc.phi <= 0
    P, M, vel, sp, sm = _solve(sfpkg, gpu_ctx, sc, sc.frac, precision, 1e-8, 1e-8)
    e = _errors(S, sc, sc.frac, liq, P, M, vel, u_or, p_or, psi_or)
    _report("64^3", precision, sp, sm, e)
    assert e["rel_l2_p"] <= 1e-5 and e["rel_l2_psi"] <= 1e-5, e
    for a in range(3):
        assert np.abs(vel[a] - u_or[a]).max() <= 1e-5 * np.abs(sc.vel[a]).max()
        assert np.abs(M.total_field[a] - H_or[a]).max() <= 1e-5 * np.abs(H_or[a]).max() + 1e-12


def _plane_scene(oracle):
    """demo/SimBuilder.cpp:40-62 at -s 64: the plane 0.024 above the domain floor, box collider of boundary
    width 2 (the oracle's, pinned to the reference's), seeded uniform[-1, 1] velocity."""
    S = scenes()
    sf = pkg()
    scale, bw, length = 64, 2, 0.12
    h = length / (scale - bw * 2)
    res = (scale, 3 * scale // 4, scale)
    g = sf.StaggeredGrid(bw, h, res)
    og = oracle_grid(oracle, g)
    y0 = g.domain_origin()[1] + 1.0 * length * .2
    ys = (g.origin[1] + h / 2) + np.arange(res[1]) * h
    phi = np.ascontiguousarray(np.broadcast_to((ys - y0)[None, :, None], res))
    frac = oracle.box_collider_fractions(og, bw)
    rng = np.random.default_rng(64)
    vel = [rng.uniform(-1, 1, g.face_shape(a)) for a in range(3)]
    hext = [np.full(g.face_shape(a), (0.0, 6e4, 0.0)[a]) for a in range(3)]
    return S.Scene("plane", g, phi, vel, frac, hext, 0.33, 2 * h), og


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reference_plane_scene_vs_oracle(sfpkg, oracle, gpu_ctx, precision):
    """The reference's plane scene at -s 64 at the reference's own tolerances (1e-8 / 1e-6)."""
    S = scenes()
    sc, og = _plane_scene(oracle)
    u_or, p_or, psi_or, H_or = _oracle_solutions(oracle, og, sc, sc.frac)
    liq = sc.phi <= 0
    P, M, vel, sp, sm = _solve(sfpkg, gpu_ctx, sc, sc.frac, precision, 1e-8, 1e-6)
    e = _errors(S, sc, sc.frac, liq, P, M, vel, u_or, p_or, psi_or)
    _report("plane -s 64", precision, sp, sm, e)
    assert e["rel_l2_p"] <= 1e-5 and e["rel_l2_psi"] <= 1e-5, e


@pytest.fixture(scope="module")
def pool192(oracle):
    sc = scenes().pool(192, seed=2, chi=1.0)
    og = oracle_grid(oracle, sc.grid)
    return sc, og, _oracle_solutions(oracle, og, sc, sc.frac)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_config_192_vs_oracle(sfpkg, oracle, gpu_ctx, pool192, precision):
    """192^3: to 1e-6 (the configuration's tolerance) the errors against the oracle are reported and bounded
    by the conditioning (1e-4); at the reference's tolerances (1e-8 pressure, 1e-6 potential) p and psi are
    within 1e-5 relative L2."""
    S = scenes()
    sc, og, (u_or, p_or, psi_or, H_or) = pool192
    liq = sc.phi <= 0
    P, M, vel, sp, sm = _solve(sfpkg, gpu_ctx, sc, sc.frac, precision, 1e-6, 1e-6)
    e = _errors(S, sc, sc.frac, liq, P, M, vel, u_or, p_or, psi_or)
    _report("192^3 tol 1e-6", precision, sp, sm, e)
    assert e["rel_l2_p"] <= 1e-4 and e["rel_l2_psi"] <= 1e-4, e
    P, M, vel, sp, sm = _solve(sfpkg, gpu_ctx, sc, sc.frac, precision, 1e-8, 1e-6)
    e = _errors(S, sc, sc.frac, liq, P, M, vel, u_or, p_or, psi_or)
    _report("192^3 tol 1e-8/1e-6", precision, sp, sm, e)
    assert e["rel_l2_p"] <= 1e-5 and e["rel_l2_psi"] <= 1e-5, e
