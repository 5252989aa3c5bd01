"""GPU tests of the allocation-free residual entry point (sf_magnetic_residual_noalloc).

It is checked against the existing entry point's output: the reference-operator residual that
sf_magnetic_solve_dev reports for its own potential (stats rel_residual_ref), on two calls in a row, and
against the oracle's pinned CSR system for a perturbed potential.  The file name sorts last so the suite
also exercises the once-per-device set-up after every other test has used the device; run alone, the first
call here does it.  Tolerances: against the solver's report, 1e-13 in units of ||b|| (plus 1e-6 relative): a
converged residual is a cancellation to ~1e-10 of ||b||, so fused multiply-adds and summation order change
its low digits at ~1e-16 of ||b|| (observed 3e-16); against the oracle, for a perturbed potential whose
residual is not a cancellation, 1e-9 relative."""
import ctypes as C

import numpy as np
import pytest

from conftest import oracle_grid, scenes

pytestmark = pytest.mark.gpu


def _noalloc(sfpkg, lib, grid, phi, chi, bw, hext, psi, result, stream):
    from importlib import import_module
    abi = import_module(sfpkg.__name__ + "._abi")
    g = grid.c_grid()
    return lib.sf_magnetic_residual_noalloc(C.c_void_p(stream), C.byref(g), C.c_void_p(phi.data_ptr()), float(chi),
                                            float(bw), abi.p3([h.data_ptr() for h in hext]),
                                            C.c_void_p(psi.data_ptr()), C.c_void_p(result.data_ptr()))


@pytest.fixture(scope="module")
def mag_case(sfpkg, gpu_ctx):
    """A solved 48^3 sphere-over-pool potential (device arrays) and the solver's reported residuals."""
    import torch
    sc = scenes().pool_sphere(48, seed=11, chi=2.0)
    dev = torch.device("cuda", 0)
    phi = torch.from_numpy(sc.phi).to(dev)
    hext = [torch.from_numpy(h).to(dev) for h in sc.hext]
    psi = torch.zeros(sc.grid.shape, dtype=torch.float64, device=dev)
    H = [torch.zeros(sc.grid.face_shape(a), dtype=torch.float64, device=dev) for a in range(3)]
    M = sfpkg.MagneticField(sc.grid, sc.chi, sc.band_width, gpu_ctx)
    st = M.solve(phi, hext, device=True, psi_out=psi, H_out=H,
                 opts=sfpkg.options("magnetic", precision="fp64", tol=1e-9, warm_start=0))
    torch.cuda.synchronize()
    return sc, phi, hext, psi, st


def test_noalloc_matches_solver_twice(sfpkg, gpu_ctx, mag_case):
    import torch
    sc, phi, hext, psi, st = mag_case
    assert st["converged"] == 1 and st["rel_residual_ref"] > 0
    result = torch.full((4,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        s = _noalloc(sfpkg, gpu_ctx.lib, sc.grid, phi, sc.chi, sc.band_width, hext, psi, result[2 * call:], stream)
        assert s == sfpkg._abi.SF_OK, gpu_ctx.lib.sf_status_string(s)
    torch.cuda.synchronize()
    r = result.cpu().numpy()
    assert r[0] == r[2] and r[1] == r[3]  # deterministic reduction: same bits on the second call
    assert abs(r[0] - st["rel_residual_ref"]) <= 1e-13 + 1e-6 * st["rel_residual_ref"]
    assert r[1] > 0


def test_noalloc_matches_oracle_pinned_system(sfpkg, gpu_ctx, oracle, mag_case):
    """A perturbed potential (psi_0 != 0 included) against ||b - A psi|| / ||b|| of the oracle's pinned CSR."""
    import torch
    sc, phi, hext, psi, _ = mag_case
    rng = np.random.default_rng(5)
    p = psi.cpu().numpy() + 1e-3 * rng.standard_normal(sc.grid.shape)
    og = oracle_grid(oracle, sc.grid)
    mu = oracle.magnetic_coeff(og, sc.phi, sc.chi, sc.band_width)
    A = oracle.magnetic_assemble(og, mu)
    b, _ = oracle.magnetic_rhs(og, mu, sc.hext)
    want = np.linalg.norm(b - A.matvec(p.ravel())) / np.linalg.norm(b)
    pd = torch.from_numpy(p).cuda()
    result = torch.zeros(2, dtype=torch.float64, device="cuda")
    s = _noalloc(sfpkg, gpu_ctx.lib, sc.grid, phi, sc.chi, sc.band_width, hext, pd, result,
                 torch.cuda.current_stream().cuda_stream)
    assert s == sfpkg._abi.SF_OK
    torch.cuda.synchronize()
    r = result.cpu().numpy()
    assert abs(r[0] - want) <= 1e-9 * want
    assert abs(r[1] - np.linalg.norm(b)) <= 1e-12 * np.linalg.norm(b)


def test_noalloc_rejects_oversized_and_host_pointers(sfpkg, gpu_ctx, mag_case):
    import torch
    sc, phi, hext, psi, _ = mag_case
    lib = gpu_ctx.lib
    result = torch.zeros(2, dtype=torch.float64, device="cuda")
    big = sfpkg.StaggeredGrid.from_origin(1.0 / 64, (2, 2056, 1056))  # 257 x 33 tiles per x-plane > 8192
    assert _noalloc(sfpkg, lib, big, phi, 1.0, 0.1, hext, psi, result, 0) == sfpkg._abi.SF_TOO_LARGE
    host_psi = psi.cpu()
    assert _noalloc(sfpkg, lib, sc.grid, phi, sc.chi, sc.band_width, hext, host_psi, result, 0) == \
        sfpkg._abi.SF_BAD_ARG
