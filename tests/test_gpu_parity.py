"""GPU parity: the CUDA library against the oracle (CPU restatement of core/Pressure.cpp and
core/MagneticField.cpp) on the same seeded inputs, through the C ABI.

Tolerances (north-star): relative residual <= the requested tolerance on the reference's operator, and
relative L2 error <= 1e-5 in p (liquid cells) and psi against the oracle's solution of the same discrete
system solved to 1e-12.  Assembled operators are compared bit for bit where the arithmetic is exact.
"""
import numpy as np
import pytest

from conftest import oracle_grid, rel_l2, scenes

pytestmark = pytest.mark.gpu

P_TOL = 1e-5  # relative L2 of p / psi against the oracle


def _copy(v):
    return [np.array(a, copy=True) for a in v]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n,seed", [(16, 1), (32, 2), (48, 3)])
def test_pressure_pool_vs_oracle(sfpkg, oracle, gpu_ctx, precision, n, seed):
    sc = scenes().pool(n, seed=seed)
    og = oracle_grid(oracle, sc.grid)
    u_or, p_or, info = oracle.pressure_project(og, sc.phi, sc.frac, sc.vel, tol=1e-13)
    vel = _copy(sc.vel)
    P = sfpkg.Pressure(sc.grid, gpu_ctx)
    st = P.project(vel, sc.phi, sc.frac, opts=sfpkg.options("pressure", precision=precision))
    liquid = sc.phi <= 0
    assert st["converged"] == 1
    assert st["rel_residual"] <= 1e-8 * 1.01
    assert rel_l2(P.pressure[liquid], p_or[liquid]) <= P_TOL
    assert np.all(P.pressure[~liquid] == 0)
    for a in range(3):
        scale = np.abs(sc.vel[a]).max()
        assert np.abs(vel[a] - u_or[a]).max() <= 1e-5 * scale


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pressure_sphere_vs_oracle(sfpkg, oracle, gpu_ctx, precision):
    """Curved interface (pool + sphere, ghost-fluid terms on a sphere) at the reference's pressure tolerance,
    amgcl's default 1e-8 (core/Pressure.cpp:125-135): p within 1e-5 relative L2 of the oracle."""
    sc = scenes().pool_sphere(40, seed=5)
    og = oracle_grid(oracle, sc.grid)
    u_or, p_or, info = oracle.pressure_project(og, sc.phi, sc.frac, sc.vel, tol=1e-13)
    vel = _copy(sc.vel)
    P = sfpkg.Pressure(sc.grid, gpu_ctx)
    st = P.project(vel, sc.phi, sc.frac, opts=sfpkg.options("pressure", precision=precision, tol=1e-8))
    liquid = sc.phi <= 0
    assert st["rel_residual"] <= 1e-8 * 1.01
    assert rel_l2(P.pressure[liquid], p_or[liquid]) <= P_TOL
    for a in range(3):
        assert np.abs(vel[a] - u_or[a]).max() <= 1e-5 * np.abs(sc.vel[a]).max()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n,seed", [(16, 1), (32, 2)])
def test_magnetic_pool_vs_oracle(sfpkg, oracle, gpu_ctx, precision, n, seed):
    sc = scenes().pool(n, seed=seed, chi=1.0)
    og = oracle_grid(oracle, sc.grid)
    psi_or, H_or, info = oracle.magnetic_solve(og, sc.phi, sc.chi, sc.band_width, sc.hext, tol=1e-13)
    M = sfpkg.MagneticField(sc.grid, sc.chi, sc.band_width, gpu_ctx)
    st = M.solve(sc.phi, sc.hext, opts=sfpkg.options("magnetic", precision=precision, tol=1e-9))
    assert st["converged"] == 1
    assert st["rel_residual_ref"] <= 1e-9 * 1.05
    assert M.potential.ravel()[0] == 0.0
    assert rel_l2(M.potential, psi_or) <= P_TOL
    for a in range(3):
        assert np.abs(M.total_field[a] - H_or[a]).max() <= 1e-5 * np.abs(H_or[a]).max() + 1e-12


def test_magnetic_default_tol_matches(sfpkg, oracle, gpu_ctx):
    """At the reference's own tolerance (1e-6, core/MagneticField.cpp:93) psi is within 1e-5 of the oracle."""
    sc = scenes().pool(32, seed=7, chi=1.0)
    og = oracle_grid(oracle, sc.grid)
    psi_or, H_or, info = oracle.magnetic_solve(og, sc.phi, sc.chi, sc.band_width, sc.hext, tol=1e-13)
    M = sfpkg.MagneticField(sc.grid, sc.chi, sc.band_width, gpu_ctx)
    st = M.solve(sc.phi, sc.hext)
    assert st["rel_residual_ref"] <= 1e-6
    assert rel_l2(M.potential, psi_or) <= P_TOL


def test_hydrostatic_kat(sfpkg, gpu_ctx):
    """Zero velocity, zero volume error, constant jump J: p == J in the liquid and u is unchanged."""
    sc = scenes().pool(24, seed=3)
    J = 0.75
    jump = [np.full(sc.grid.face_shape(a), J) for a in range(3)]
    vel = [np.zeros(sc.grid.face_shape(a)) for a in range(3)]
    P = sfpkg.Pressure(sc.grid, gpu_ctx)
    P.set_pressure_jump(jump)
    P.project(vel, sc.phi, sc.frac, opts=sfpkg.options("pressure", tol=1e-12))
    liquid = sc.phi <= 0
    assert np.abs(P.pressure[liquid] - J).max() <= 1e-9
    for a in range(3):
        assert np.abs(vel[a]).max() <= 1e-9


def test_chi_zero_kat(sfpkg, gpu_ctx):
    """chi = 0: mu == 1, b == 0, psi == 0 and H == Hext exactly."""
    sc = scenes().pool(16, seed=4)
    M = sfpkg.MagneticField(sc.grid, 0.0, sc.band_width, gpu_ctx)
    M.solve(sc.phi, sc.hext)
    assert np.all(M.potential == 0)
    for a in range(3):
        assert np.array_equal(M.total_field[a], sc.hext[a])


def test_slab_kat(sfpkg, gpu_ctx):
    """Full-width horizontal slab in a uniform vertical field: H_y = H0/(1+chi) inside the liquid away from
    the smoothed band, H0 above it (continuity of B_y = mu H_y)."""
    n = 32
    g = scenes().unit_grid(n)
    ys = scenes().cell_centres(g, 1)
    phi = np.ascontiguousarray(np.broadcast_to((ys - 0.5)[None, :, None], g.shape))
    hext = scenes().uniform_field(g, (0.0, 1.0, 0.0))
    chi = 1.5
    M = sfpkg.MagneticField(g, chi, 2 * g.spacing, gpu_ctx)
    M.solve(phi, hext, opts=sfpkg.options("magnetic", tol=1e-10))
    Hy = M.total_field[1]
    yf = np.arange(n + 1) / n
    inside = (yf > 0.05) & (yf < 0.5 - 3 * g.spacing)
    above = (yf > 0.5 + 3 * g.spacing) & (yf < 0.95)
    assert np.abs(Hy[:, inside, :] - 1.0 / (1.0 + chi)).max() <= 1e-6
    assert np.abs(Hy[:, above, :] - 1.0).max() <= 1e-6


def test_reproject_reuses_operator(sfpkg, oracle, gpu_ctx):
    """Reproject: same unknowns and matrix as the last Project, new rhs without jump terms, warm start."""
    sc = scenes().pool(24, seed=9)
    og = oracle_grid(oracle, sc.grid)
    P = sfpkg.Pressure(sc.grid, gpu_ctx)
    vel = _copy(sc.vel)
    P.project(vel, sc.phi, sc.frac)
    vel2 = [v * 0.5 for v in sc.vel]
    ref = _copy(vel2)
    P.reproject(vel2, sc.phi, sc.frac, opts=sfpkg.options("pressure", tol=1e-10))
    A, b, g2m, m2g = oracle.pressure_assemble(og, sc.phi, sc.frac, ref)
    b2 = oracle.pressure_rhs(og, sc.frac, ref, None, 0.0, m2g)
    assert np.array_equal(b, b2)  # no jump, no solid velocity: same rhs
    p, it, rr = A.solve(b2, tol=1e-13)
    u_or = oracle.pressure_apply(og, sc.phi, sc.frac, None, g2m, p, ref)
    assert rel_l2(P.pressure.ravel()[m2g], p) <= P_TOL
    for a in range(3):
        assert np.abs(vel2[a] - u_or[a]).max() <= 1e-6 * np.abs(ref[a]).max()


def test_device_pointer_path(sfpkg, gpu_ctx):
    """_dev entry points on torch CUDA tensors give the same results as the host entry points."""
    import torch
    sc = scenes().pool(24, seed=11)
    P = sfpkg.Pressure(sc.grid, gpu_ctx)
    vel_h = _copy(sc.vel)
    P.project(vel_h, sc.phi, sc.frac)
    p_h = P.pressure.copy()
    dev = torch.device("cuda:0")
    vel_d = [torch.from_numpy(v).to(dev) for v in sc.vel]
    torch.cuda.synchronize()
    p_d = torch.zeros(sc.grid.shape, dtype=torch.float64, device=dev)
    P.project(vel_d, torch.from_numpy(sc.phi).to(dev), [torch.from_numpy(f).to(dev) for f in sc.frac],
              device=True, p_out=p_d)
    assert np.array_equal(p_d.cpu().numpy(), p_h)
    for a in range(3):
        assert np.array_equal(vel_d[a].cpu().numpy(), vel_h[a])


def test_deterministic(sfpkg, gpu_ctx):
    """Same inputs -> bit-identical outputs and iteration counts (deterministic reductions)."""
    sc = scenes().pool_sphere(32, seed=2)
    P = sfpkg.Pressure(sc.grid, gpu_ctx)
    outs = []
    for _ in range(2):
        vel = _copy(sc.vel)
        st = P.project(vel, sc.phi, sc.frac)
        outs.append((P.pressure.copy(), st["iters"]))
    assert outs[0][1] == outs[1][1]
    assert np.array_equal(outs[0][0], outs[1][0])


def test_odd_sizes_and_tiny(sfpkg, oracle, gpu_ctx):
    """Ragged grids (odd, non-cubic) and a grid smaller than the coarsest level."""
    for shape in [(13, 9, 7), (5, 3, 4), (33, 17, 20)]:
        g = sfpkg.StaggeredGrid.from_origin(1.0 / shape[0], shape)
        og = oracle_grid(oracle, g)
        rng = np.random.default_rng(sum(shape))
        ys = scenes().cell_centres(g, 1)
        phi = np.ascontiguousarray(np.broadcast_to((ys - 0.4 * ys.max())[None, :, None], g.shape)) \
            + 0.01 * rng.uniform(-1, 1, g.shape)
        frac = scenes().box_fractions(g)
        vel = [rng.uniform(-1, 1, g.face_shape(a)) for a in range(3)]
        u_or, p_or, info = oracle.pressure_project(og, phi, frac, vel, tol=1e-13)
        v2 = _copy(vel)
        P = sfpkg.Pressure(g, gpu_ctx)
        P.project(v2, phi, frac, opts=sfpkg.options("pressure", tol=1e-11))
        liq = phi <= 0
        assert rel_l2(P.pressure[liq], p_or[liq]) <= 1e-8
        hext = scenes().uniform_field(g)
        psi_or, H_or, _ = oracle.magnetic_solve(og, phi, 1.0, 2 * g.spacing, hext, tol=1e-13)
        M = sfpkg.MagneticField(g, 1.0, 2 * g.spacing, gpu_ctx)
        M.solve(phi, hext, opts=sfpkg.options("magnetic", tol=1e-11))
        assert rel_l2(M.potential, psi_or) <= 1e-7


def test_no_liquid(sfpkg, gpu_ctx):
    """No liquid cell: Project leaves the velocity untouched (core/Pressure.cpp:22)."""
    sc = scenes().pool(16, seed=1)
    phi = np.ones(sc.grid.shape)
    vel = _copy(sc.vel)
    P = sfpkg.Pressure(sc.grid, gpu_ctx)
    P.project(vel, phi, sc.frac)
    for a in range(3):
        assert np.array_equal(vel[a], sc.vel[a])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("shape", [(32, 32, 32), (37, 21, 70), (9, 130, 5), (20, 16, 76), (35, 27, 136)])
def test_fused_smoother_bit_identical(sfpkg, gpu_ctx, precision, shape):
    """The one-pass fused red-black sweep reproduces the two in-place colour kernels bit for bit.  Shapes with
    nz a multiple of 4 and at least 72 (one TMA box) take the TMA-staged kernel at the finest FP32 level; the
    others take the cp.async kernel."""
    g = sfpkg.StaggeredGrid.from_origin(1.0 / shape[0], shape)
    rng = np.random.default_rng(sum(shape))
    ys = scenes().cell_centres(g, 1)
    phi = np.ascontiguousarray(np.broadcast_to((ys - 0.45 * ys.max())[None, :, None], g.shape)) \
        + 0.02 * rng.uniform(-1, 1, g.shape)
    frac = scenes().box_fractions(g)
    vel = [rng.uniform(-1, 1, g.face_shape(a)) for a in range(3)]
    hext = scenes().uniform_field(g)
    out = []
    for smoother in (0, 1):
        P = sfpkg.Pressure(g, gpu_ctx)
        v = _copy(vel)
        st = P.project(v, phi, frac, opts=sfpkg.options("pressure", precision=precision, smoother=smoother))
        M = sfpkg.MagneticField(g, 1.5, 2 * g.spacing, gpu_ctx)
        sm = M.solve(phi, hext, opts=sfpkg.options("magnetic", precision=precision, smoother=smoother))
        out.append((P.pressure.copy(), st["iters"], M.potential.copy(), sm["iters"]))
    assert out[0][1] == out[1][1] and out[0][3] == out[1][3]
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][2], out[1][2])


@pytest.mark.parametrize("smoother", [2, 3])
@pytest.mark.parametrize("n,seed", [(32, 2), (48, 3)])
def test_fp16_smoothing_coefficients_same_answer(sfpkg, oracle, gpu_ctx, n, seed, smoother):
    """Smoothers 2 and 3 (finest-level smoothing from an FP16 copy of the operator; 3 with that level stored
    colour by colour) change only the preconditioner: the mixed solve reaches the same tolerance on the FP64
    operator and the same answer as the oracle."""
    sc = scenes().pool_sphere(n, seed=seed)
    og = oracle_grid(oracle, sc.grid)
    u_or, p_or, _ = oracle.pressure_project(og, sc.phi, sc.frac, sc.vel, tol=1e-13)
    psi_or, _, _ = oracle.magnetic_solve(og, sc.phi, sc.chi, sc.band_width, sc.hext, tol=1e-13)
    P = sfpkg.Pressure(sc.grid, gpu_ctx)
    st = P.project(_copy(sc.vel), sc.phi, sc.frac,
                   opts=sfpkg.options("pressure", precision="mixed", smoother=smoother))
    liquid = sc.phi <= 0
    assert st["converged"] == 1 and st["rel_residual"] <= 1e-8 * 1.01
    assert rel_l2(P.pressure[liquid], p_or[liquid]) <= P_TOL
    M = sfpkg.MagneticField(sc.grid, sc.chi, sc.band_width, gpu_ctx)
    sm = M.solve(sc.phi, sc.hext, opts=sfpkg.options("magnetic", precision="mixed", smoother=smoother, tol=1e-9))
    assert sm["converged"] == 1 and sm["rel_residual_ref"] <= 1e-9 * 1.05
    assert rel_l2(M.potential, psi_or) <= P_TOL


@pytest.mark.parametrize("shape", [(32, 32, 32), (20, 16, 40), (9, 13, 8), (37, 21, 70), (16, 16, 12)])
def test_split_level_matches_natural(sfpkg, gpu_ctx, shape):
    """Smoother 3 against smoother 2 in the mixed form.  Where nz is a multiple of 8 the finest level is stored
    colour by colour: every cell's smoothing and operator arithmetic is the natural kernels', the restriction
    leaves out the colour whose residual the last pre-smoothing half sweep zeroed (to rounding), and the Krylov
    dot products sum in the permuted order, so the two solves take the same number of iterations (+-1) and agree
    to the solve's accuracy (relative L2 1e-6 at tolerances 1e-9 / 1e-8).  Otherwise smoother 3 runs as
    smoother 2: bit for bit."""
    g = sfpkg.StaggeredGrid.from_origin(1.0 / shape[0], shape)
    rng = np.random.default_rng(sum(shape) + 7)
    ys = scenes().cell_centres(g, 1)
    phi = np.ascontiguousarray(np.broadcast_to((ys - 0.45 * ys.max())[None, :, None], g.shape)) \
        + 0.02 * rng.uniform(-1, 1, g.shape)
    frac = scenes().box_fractions(g)
    vel = [rng.uniform(-1, 1, g.face_shape(a)) for a in range(3)]
    hext = scenes().dipole_field(g)
    out = []
    for smoother in (2, 3):
        P = sfpkg.Pressure(g, gpu_ctx)
        st = P.project(_copy(vel), phi, frac,
                       opts=sfpkg.options("pressure", precision="mixed", smoother=smoother, tol=1e-9))
        M = sfpkg.MagneticField(g, 1.5, 2 * g.spacing, gpu_ctx)
        sm = M.solve(phi, hext, opts=sfpkg.options("magnetic", precision="mixed", smoother=smoother, tol=1e-8,
                                                     warm_start=0))
        assert st["converged"] == 1 and st["rel_residual"] <= 1e-9 * 1.01
        assert sm["converged"] == 1 and sm["rel_residual_ref"] <= 1e-8 * 1.05
        out.append((P.pressure.copy(), st["iters"], M.potential.copy(), sm["iters"]))
    liquid = phi <= 0
    if shape[2] % 8 == 0:
        assert abs(out[0][1] - out[1][1]) <= 1 and abs(out[0][3] - out[1][3]) <= 1, (out[0][1::2], out[1][1::2])
        assert rel_l2(out[1][0][liquid], out[0][0][liquid]) <= 1e-6
        assert rel_l2(out[1][2], out[0][2]) <= 1e-6
    else:
        assert out[0][1] == out[1][1] and out[0][3] == out[1][3]
        assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][2], out[1][2])


@pytest.mark.parametrize("smoother", [2, 3])
@pytest.mark.parametrize("shape", [(64, 64, 64), (50, 44, 40), (96, 80, 72), (37, 21, 70), (20, 16, 76),
                                   (80, 80, 80), (9, 13, 8), (192, 192, 192)])
def test_cluster_tail_bit_identical(sfpkg, gpu_ctx, smoother, shape):
    """The mixed V-cycle's levels of at most 65,536 cells run by default in one launch of a thread-block cluster
    (coarse_tail 0: 16 CTAs where the device runs it, else 8; 8 and 16 force the size); coarse_tail=1 runs them as
    separate kernels.  Every cell's arithmetic is the same, so all forms take the same iterations and return the
    same bits.  The shapes give tails of two to five levels: all held by CTA 0, distributed over the cluster
    then held by CTA 0, and (80^3 with smoother 2) two distributed levels; shares of unequal plane counts across
    the cluster, odd nz, and (9, 13, 8) a hierarchy too short for a tail (same launches); 192^3 with smoother 3
    has two split levels above the tail."""
    g = sfpkg.StaggeredGrid.from_origin(1.0 / shape[0], shape)
    rng = np.random.default_rng(sum(shape) + 11)
    ys = scenes().cell_centres(g, 1)
    phi = np.ascontiguousarray(np.broadcast_to((ys - 0.45 * ys.max())[None, :, None], g.shape)) \
        + 0.02 * rng.uniform(-1, 1, g.shape)
    frac = scenes().box_fractions(g)
    vel = [rng.uniform(-1, 1, g.face_shape(a)) for a in range(3)]
    hext = scenes().dipole_field(g)
    out = []
    for tail in (1, 8, 16, 0):
        P = sfpkg.Pressure(g, gpu_ctx)
        st = P.project(_copy(vel), phi, frac, opts=sfpkg.options(
            "pressure", precision="mixed", smoother=smoother, tol=1e-9, coarse_tail=tail))
        M = sfpkg.MagneticField(g, 1.5, 2 * g.spacing, gpu_ctx)
        sm = M.solve(phi, hext, opts=sfpkg.options("magnetic", precision="mixed", smoother=smoother, tol=1e-8,
                                                     warm_start=0, coarse_tail=tail))
        assert st["converged"] == 1 and sm["converged"] == 1
        out.append((P.pressure.copy(), st["iters"], M.potential.copy(), sm["iters"], st["kernel_launches"]))
    for o in out[1:]:
        assert o[1] == out[0][1] and o[3] == out[0][3], (out[0][1::2], o[1::2])
        assert np.array_equal(o[0], out[0][0]) and np.array_equal(o[2], out[0][2])
        if shape == (9, 13, 8):
            assert o[4] == out[0][4]
        else:
            assert o[4] < out[0][4], (out[0][4], o[4])
