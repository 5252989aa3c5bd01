"""Failure paths, made on the host or with bounded waits (no GPU fault, trap or hang is provoked):

* a non-finite input (NaN velocity) ends the solve with a defined status (SF_NOT_CONVERGED) and the context
  stays usable;
* an iteration cap of one returns SF_NOT_CONVERGED with the last iterate (finite, and a smaller residual than
  the zero start);
* a liquid pocket enclosed by walls (a pure-Neumann block of the pressure system, singular but consistent) is
  solved to the tolerance with finite values;
* the bounded waits of the TMA-staged kernels give up after their limit: the self-test waits on an mbarrier that
  nothing completes, reports the timeout, and the context solves again afterwards.
The reference ignores non-convergence (core/Pressure.cpp:133-134, core/MagneticField.cpp:120-123); these status
codes are the library's own guard."""
import ctypes as C

import numpy as np
import pytest

from conftest import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nan_input_defined_status(sfpkg, gpu_ctx, precision):
    sc = scenes().pool(24, seed=8)
    v = [a.copy() for a in sc.vel]
    v[1][5, 3, 7] = np.nan
    P = sfpkg.Pressure(sc.grid, gpu_ctx)
    st = P.project(v, sc.phi, sc.frac, opts=sfpkg.options("pressure", precision=precision), raise_on_nonconv=False)
    assert P.status == sfpkg._abi.SF_NOT_CONVERGED and st["converged"] == 0
    # the context is still usable
    v = [a.copy() for a in sc.vel]
    st = P.project(v, sc.phi, sc.frac, opts=sfpkg.options("pressure", precision=precision))
    assert P.status == sfpkg._abi.SF_OK and st["converged"] == 1


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_iteration_cap(sfpkg, gpu_ctx, precision):
    sc = scenes().pool_sphere(32, seed=2)
    M = sfpkg.MagneticField(sc.grid, sc.chi, sc.band_width, gpu_ctx)
    st = M.solve(sc.phi, sc.hext, opts=sfpkg.options("magnetic", precision=precision, max_iters=1, warm_start=0,
                                                     tol=1e-10), raise_on_nonconv=False)
    assert M.status == sfpkg._abi.SF_NOT_CONVERGED and st["converged"] == 0
    assert st["iters"] == 1
    assert np.isfinite(M.potential).all() and np.any(M.potential != 0)
    assert 0 < st["rel_residual"] < 1.0
    for a in range(3):
        assert np.isfinite(M.total_field[a]).all()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_enclosed_liquid_pocket(sfpkg, gpu_ctx, precision):
    """Liquid everywhere inside the box walls, no free surface: every row is a Neumann row, the operator is
    singular, and the right-hand side (the divergence of the velocity) sums to zero, so the system is consistent."""
    sc = scenes().pool(24, seed=5)
    phi = -np.ones(sc.grid.shape)  # liquid everywhere
    v = [a.copy() for a in sc.vel]
    P = sfpkg.Pressure(sc.grid, gpu_ctx)
    st = P.project(v, phi, sc.frac, opts=sfpkg.options("pressure", precision=precision, tol=1e-8),
                   raise_on_nonconv=False)
    assert np.isfinite(P.pressure).all()
    for a in range(3):
        assert np.isfinite(v[a]).all()
    assert st["converged"] == 1 and st["rel_residual"] <= 1e-8 * 1.01
    # the projected field is divergence-free on the cells whose faces are fully open or closed
    S = scenes()
    full = S.full_weight_cells(sc.grid, sc.frac)
    div0 = np.abs(S.divergence(sc.grid, sc.vel, sc.frac)[full]).max()
    div = np.abs(S.divergence(sc.grid, v, sc.frac)[full]).max()
    assert div <= 1e-5 * div0  # max-norm: at most sqrt(N) times the L2 residual, 1e-8 of the rhs


def test_bounded_wait_gives_up(sfpkg, gpu_ctx):
    lib = gpu_ctx.lib
    out, waited = C.c_int(-1), C.c_double(-1.0)
    s = lib.sf_selftest_bounded_wait(gpu_ctx.handle, 50.0, C.byref(out), C.byref(waited))
    assert s == sfpkg._abi.SF_OK
    assert out.value == 1  # the wait gave up
    assert 50.0 <= waited.value < 5000.0
    assert lib.sf_selftest_bounded_wait(gpu_ctx.handle, 0.0, C.byref(out), None) == sfpkg._abi.SF_BAD_ARG
    # the context still solves
    sc = scenes().pool(16, seed=1)
    P = sfpkg.Pressure(sc.grid, gpu_ctx)
    st = P.project([a.copy() for a in sc.vel], sc.phi, sc.frac)
    assert st["converged"] == 1
