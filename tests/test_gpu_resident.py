"""Resident inputs (sf_collider_upload, sf_levelset_upload): a projection and a potential solve that read the
uploaded collider and level set give the same bits as calls that pass them, copy fewer bytes, and calls that
pass NULL without a matching upload are refused with SF_NOT_READY."""
import ctypes as C

import numpy as np
import pytest

from conftest import scenes

pytestmark = pytest.mark.gpu


def test_resident_inputs_same_bits(sfpkg, gpu_ctx):
    sc = scenes().pool_sphere(32, seed=9)
    g = sc.grid
    o_p = sfpkg.options("pressure", precision="mixed")
    o_m = sfpkg.options("magnetic", precision="mixed", warm_start=0)
    v1 = [a.copy() for a in sc.vel]
    P = sfpkg.Pressure(g, gpu_ctx)
    s1 = P.project(v1, sc.phi, sc.frac, opts=o_p)
    p1 = P.pressure.copy()
    M = sfpkg.MagneticField(g, sc.chi, sc.band_width, gpu_ctx)
    M.solve(sc.phi, sc.hext, opts=o_m)
    psi1, H1 = M.potential.copy(), [h.copy() for h in M.total_field]

    gpu_ctx.upload_collider(g, sc.frac)
    gpu_ctx.upload_level_set(g, sc.phi)
    v2 = [a.copy() for a in sc.vel]
    s2 = P.project(v2, None, None, opts=o_p)
    M.solve(None, sc.hext, opts=o_m)
    assert np.array_equal(P.pressure, p1)
    for a in range(3):
        assert np.array_equal(v2[a], v1[a])
        assert np.array_equal(M.total_field[a], H1[a])
    assert np.array_equal(M.potential, psi1)
    nf = sum(int(np.prod(g.face_shape(a))) for a in range(3))
    assert s1["h2d_bytes"] - s2["h2d_bytes"] == 8 * (nf + g.num_cells)


def test_resident_inputs_not_ready(sfpkg):
    ctx = sfpkg.Context(0)
    try:
        sc = scenes().pool(16, seed=2)
        P = sfpkg.Pressure(sc.grid, ctx)
        v = [a.copy() for a in sc.vel]
        with pytest.raises(sfpkg.SolveError) as e:
            P.project(v, None, sc.frac)
        assert e.value.status == sfpkg._abi.SF_NOT_READY
        with pytest.raises(sfpkg.SolveError) as e:
            P.project(v, sc.phi, None)
        assert e.value.status == sfpkg._abi.SF_NOT_READY
        # an upload on a grid of other dimensions does not serve this one
        other = scenes().pool(12, seed=2)
        ctx.upload_collider(other.grid, other.frac)
        ctx.upload_level_set(other.grid, other.phi)
        with pytest.raises(sfpkg.SolveError) as e:
            P.project(v, None, None)
        assert e.value.status == sfpkg._abi.SF_NOT_READY
        M = sfpkg.MagneticField(sc.grid, sc.chi, sc.band_width, ctx)
        with pytest.raises(sfpkg.SolveError) as e:
            M.solve(None, sc.hext)
        assert e.value.status == sfpkg._abi.SF_NOT_READY
        # device arrays are accepted as well
        import torch
        dev = torch.device("cuda", 0)
        ctx.upload_level_set(sc.grid, torch.from_numpy(sc.phi).to(dev))
        ctx.upload_collider(sc.grid, [torch.from_numpy(f).to(dev) for f in sc.frac])
        P.project(v, None, None)
    finally:
        ctx.close()


def test_prefetched_applied_field_same_bits(sfpkg, gpu_ctx):
    """sf_applied_field_prefetch: the copy started under a pressure projection (pinned host arrays, side stream)
    and read by the magnetic call with hext = NULL gives the bits of the call that passes hext; a later call with
    NULL reads the same field again; the prefetched bytes are counted once."""
    import torch
    sc = scenes().pool_sphere(48, seed=10)
    g = sc.grid
    o_p = sfpkg.options("pressure", precision="mixed")
    o_m = sfpkg.options("magnetic", precision="mixed", warm_start=0)
    M = sfpkg.MagneticField(g, sc.chi, sc.band_width, gpu_ctx)
    s1 = M.solve(sc.phi, sc.hext, opts=o_m)
    psi1, H1 = M.potential.copy(), [h.copy() for h in M.total_field]

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
        t.numpy()[...] = a
        return t.numpy()

    hp = [pinned(h) for h in sc.hext]
    gpu_ctx.prefetch_applied_field(g, hp)
    P = sfpkg.Pressure(g, gpu_ctx)
    P.project([a.copy() for a in sc.vel], sc.phi, sc.frac, opts=o_p)
    s2 = M.solve(sc.phi, None, opts=o_m)
    assert np.array_equal(M.potential, psi1)
    for a in range(3):
        assert np.array_equal(M.total_field[a], H1[a])
    assert s2["h2d_bytes"] == s1["h2d_bytes"]
    s3 = M.solve(sc.phi, None, opts=o_m)  # no new prefetch: the same field, no copy
    assert np.array_equal(M.potential, psi1)
    nf = sum(int(np.prod(g.face_shape(a))) for a in range(3))
    assert s2["h2d_bytes"] - s3["h2d_bytes"] == 8 * nf
    # a prefetch not followed by a pressure call is copied by the magnetic call itself
    gpu_ctx.prefetch_applied_field(g, [2.0 * h for h in sc.hext])
    M.solve(sc.phi, None, opts=o_m)
    H2 = [h.copy() for h in M.total_field]
    M.solve(sc.phi, [2.0 * h for h in sc.hext], opts=o_m)
    for a in range(3):
        assert np.array_equal(M.total_field[a], H2[a])


def test_prefetched_applied_field_not_ready(sfpkg):
    ctx = sfpkg.Context(0)
    try:
        sc = scenes().pool(16, seed=3)
        M = sfpkg.MagneticField(sc.grid, sc.chi, sc.band_width, ctx)
        with pytest.raises(sfpkg.SolveError) as e:
            M.solve(sc.phi, None)
        assert e.value.status == sfpkg._abi.SF_NOT_READY
        other = scenes().pool(12, seed=3)
        ctx.prefetch_applied_field(other.grid, other.hext)
        with pytest.raises(sfpkg.SolveError) as e:
            M.solve(sc.phi, None)
        assert e.value.status == sfpkg._abi.SF_NOT_READY
        null_entry = sfpkg._abi.p3([0, 0, 0])
        assert ctx.lib.sf_applied_field_prefetch(ctx.handle, C.byref(sc.grid.c_grid()), null_entry) == \
            sfpkg._abi.SF_BAD_ARG
    finally:
        ctx.close()
