"""The finest-level operator and right-hand side the GPU assembles (sf_system_operator) against the oracle's CSR
assembly of the reference's systems (core/Pressure.cpp:38-78, core/MagneticField.cpp:51-118).  The assembly
kernels are compiled without fused multiply-add and evaluate in the reference's order, fast paths for uniform
cells included, so the pressure system matches bit for bit everywhere and the potential's system wherever no
sin() is evaluated."""
import numpy as np
import pytest

from conftest import oracle_grid, scenes


def _offdiag(A):
    rows = np.repeat(np.arange(A.n), np.diff(A.rowptr))
    cols, vals = A.col.astype(np.int64), A.val
    diag = np.zeros(A.n)
    on = rows == cols
    diag[rows[on]] = vals[on]
    return rows[~on], cols[~on], vals[~on], diag


def _eq(got, want, what):
    """Bit equality, reporting where it fails."""
    got, want = np.ravel(got), np.ravel(want)
    bad = np.flatnonzero(got != want)
    assert bad.size == 0, (f"{what}: {bad.size} of {got.size} entries differ, first at {bad[:4]}: "
                           f"{got[bad[:4]]} vs {want[bad[:4]]}, max |diff| {np.abs(got[bad] - want[bad]).max():.3e}")


def _near(got, want, atol, what):
    d = np.abs(np.ravel(got) - np.ravel(want))
    assert d.max(initial=0.0) <= atol, f"{what}: max |diff| {d.max():.3e} at {np.argmax(d)} > {atol:.1e}"


def _check_couplings(shape, lower, cr, cn, vals, check):
    """Each off-diagonal (row cr, column cn) is minus the coupling stored on the face between the two cells."""
    nx, ny, nz = shape
    seen = 0
    for a, st in enumerate((ny * nz, nz, 1)):
        fl = lower[a].ravel()
        for m, face in ((cn == cr - st, cr), (cn == cr + st, cn)):
            check(fl[face[m]], -vals[m], f"couplings along axis {a}")
            seen += int(m.sum())
    assert seen == len(vals)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("extras", [False, True])
def test_pressure_assembly_bit_exact(sfpkg, oracle, gpu_ctx, precision, extras):
    """40^3 sphere over a pool; with extras, a solid velocity, a pressure jump, a volume-error term and partial
    solid fractions on a few percent of the faces."""
    sc = scenes().pool_sphere(40, seed=9)
    g = sc.grid
    og = oracle_grid(oracle, g)
    rng = np.random.default_rng(1)
    us = [rng.uniform(-0.3, 0.3, g.face_shape(a)) for a in range(3)] if extras else None
    jump = [rng.uniform(-0.1, 0.1, g.face_shape(a)) for a in range(3)] if extras else None
    vol = 3e-3 if extras else 0.0
    frac = [f.copy() for f in sc.frac]
    if extras:
        for f in frac:
            sel = rng.random(f.shape) < 0.04
            f[sel] = rng.uniform(0.0, 0.9, int(sel.sum()))
    A, b, g2m, m2g = oracle.pressure_assemble(og, sc.phi, frac, sc.vel, us, jump, vol)
    P = sfpkg.Pressure(g, gpu_ctx)
    P.set_pressure_jump(jump)
    P.project([v.copy() for v in sc.vel], sc.phi, frac, solid_velocity=us, vol_error=vol,
              opts=sfpkg.options("pressure", precision=precision))
    D, lower, rhs = gpu_ctx.system_operator(0, g.shape)
    m2g = np.asarray(m2g, dtype=np.int64)
    rows, cols, vals, diag = _offdiag(A)
    _eq(D.ravel()[m2g], diag, "D")
    _eq(rhs.ravel()[m2g], b, "rhs")
    air = np.ones(g.num_cells, bool)
    air[m2g] = False
    assert np.all(D.ravel()[air] == 0) and np.all(rhs.ravel()[air] == 0)
    _check_couplings(g.shape, lower, m2g[rows], m2g[cols], vals, _eq)
    # no coupling to an air cell: as many nonzero face couplings as symmetric off-diagonal pairs
    assert sum(int(np.count_nonzero(l)) for l in lower) * 2 == len(vals)


def _far_rows(phi, bw):
    """Cells whose own and six neighbours' level-set values lie outside the band |phi| <= bw (with a margin):
    every face of such a row has mu exactly 1 or 1 + chi, with no sin() evaluated."""
    far = np.abs(phi) > bw * (1 + 1e-7)
    out = far.copy()
    for a in range(3):
        for s in (1, -1):
            sh = np.roll(far, s, axis=a)
            edge = [slice(None)] * 3
            edge[a] = 0 if s == 1 else -1
            sh[tuple(edge)] = True  # no neighbour across the grid boundary
            out &= sh
    return out


def _check_magnetic(sc, mu, A, b, b0n, D, lower, rhs):
    g = sc.grid
    tol = 1e-13 * (1 + sc.chi)
    rows, cols, vals, diag = _offdiag(A)
    far = _far_rows(sc.phi, sc.band_width).ravel()
    far[0] = False  # row 0: pinned in the reference, Neumann form here (psi_0 = 0 is applied after the solve)
    assert far.sum() > 0.5 * g.num_cells
    bs = np.abs(b).max()
    Dg, bg = D.ravel(), rhs.ravel()
    _eq(Dg[far], diag[far], "D on rows away from the band")
    _eq(bg[far], b[far], "rhs on rows away from the band")
    _near(Dg[1:], diag[1:], tol, "D")
    _near(bg[1:], b[1:], 1e-13 * bs, "rhs")
    assert abs(bg[0] - b0n) <= 1e-13 * bs
    keep = rows != 0  # the reference drops column 0
    _check_couplings(g.shape, lower, rows[keep], cols[keep], vals[keep], lambda x, y, w: _near(x, y, tol, w))
    far_cell = np.abs(sc.phi) > sc.band_width * (1 + 1e-7)
    for a in range(3):
        sl = [slice(None)] * 3
        sl[a] = slice(1, g.shape[a])
        sl = tuple(sl)
        got, want = lower[a][sl], mu[a][sl]
        # every interior lower-face coupling is the reference's mu on that face (also those next to cell 0),
        # bit for bit unless the face is in the band
        _near(got, want, tol, f"mu on axis-{a} faces")
        far_face = np.roll(far_cell, 1, axis=a)[sl] & far_cell[sl]
        _eq(got[far_face], want[far_face], f"mu on axis-{a} faces away from the band")
        edge = [slice(None)] * 3
        edge[a] = 0
        assert np.all(lower[a][tuple(edge)] == 0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n", [32, 40])
def test_magnetic_assembly(sfpkg, oracle, gpu_ctx, precision, n):
    """Bit for bit on rows away from the interface.  On faces in the band, mu goes through the Heaviside's
    sin(): the device evaluates it as sinpi(phi / bw) with 1 / bw and 1 / pi formed on the host, which agrees
    with the reference's expression and the host C library's sin() to a few ulp; at h = 1/40 the reference's
    trilinear sample of phi at a face centre also differs from the two-cell mean by an ulp (weights 1/2 +- an
    ulp).  There the entries agree to 1e-13 of their scale."""
    sc = scenes().pool_sphere(n, seed=10, chi=2.0)
    g = sc.grid
    og = oracle_grid(oracle, g)
    mu = oracle.magnetic_coeff(og, sc.phi, sc.chi, sc.band_width)
    A = oracle.magnetic_assemble(og, mu)
    b, b0n = oracle.magnetic_rhs(og, mu, sc.hext)
    M = sfpkg.MagneticField(g, sc.chi, sc.band_width, gpu_ctx)
    M.solve(sc.phi, sc.hext, opts=sfpkg.options("magnetic", precision=precision, warm_start=0))
    _check_magnetic(sc, mu, A, b, b0n, *gpu_ctx.system_operator(1, g.shape))


def test_check_magnetic_accepts_the_oracle_itself(oracle):
    """The magnetic check passes on the oracle's own system laid out as the device stores it (host only)."""
    for n in (32, 40):
        sc = scenes().pool_sphere(n, seed=10, chi=2.0)
        g = sc.grid
        og = oracle_grid(oracle, g)
        mu = oracle.magnetic_coeff(og, sc.phi, sc.chi, sc.band_width)
        A = oracle.magnetic_assemble(og, mu)
        b, b0n = oracle.magnetic_rhs(og, mu, sc.hext)
        _, _, _, diag = _offdiag(A)
        lower = [np.zeros(g.shape) for _ in range(3)]
        for a in range(3):
            sl = [slice(None)] * 3
            sl[a] = slice(1, g.shape[a])
            lower[a][tuple(sl)] = mu[a][tuple(sl)]
        rhs = b.copy()
        rhs[0] = b0n
        _check_magnetic(sc, mu, A, b, b0n, diag.reshape(g.shape), lower, rhs.reshape(g.shape))
