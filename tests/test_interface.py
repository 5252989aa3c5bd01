"""Interface coupling (core/Simulation.cpp:204-235): vertex magnetic pressures (MagneticField::
CalculateVertexPressures) and the pressure-jump array built from the contour's edge marks.

The contour here is synthetic but has the reference's structure: one vertex on every cell-centre edge where the
level set changes sign (position linearly interpolated, Contour::Generate), numbered in edge order, with unit
normals and curvatures from seeded draws.  CPU: the oracle against a pure-Python restatement.  GPU: the kernels
against the oracle bit for bit, and the magnetic -> vertex pressure -> jump -> projection chain on device arrays."""
import math

import numpy as np
import pytest

from conftest import oracle_grid, rel_l2, scenes


def contour(shape, h, origin, phi, seed):
    """Edge marks (three int32 edge grids, -1 = none), vertex positions, normals and curvatures."""
    rng = np.random.default_rng(seed)
    marks, pos = [], []
    co = [origin[a] + h / 2 for a in range(3)]  # cell-centre grid
    for a in range(3):
        es = tuple(shape[b] - (b == a) for b in range(3))
        m = -np.ones(es, np.int32)
        lo = phi[tuple(slice(0, es[b]) for b in range(3))]
        hi = phi[tuple(slice(1, None) if b == a else slice(0, es[b]) for b in range(3))]
        for idx in zip(*np.nonzero((lo <= 0) != (hi <= 0))):
            t = lo[idx] / (lo[idx] - hi[idx])
            p = [co[b] + idx[b] * h for b in range(3)]
            p[a] += t * h
            m[idx] = len(pos)
            pos.append(p)
        marks.append(m)
    pos = np.array(pos, dtype=np.float64).reshape(-1, 3)
    nrm = rng.standard_normal(pos.shape)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    kappa = rng.uniform(-50, 50, pos.shape[0])
    return marks, pos, nrm, kappa


def _py_trilerp(origin, h, v, b, p):
    co = [origin[a] if a == b else origin[a] + h / 2 for a in range(3)]
    s = v.shape
    lo = [math.floor((p[a] - co[a]) * (1 / h) - 0.0) for a in range(3)]
    fr = [(p[a] - co[a] - lo[a] * h) * (1 / h) for a in range(3)]
    w = [[1.0 - fr[a] for a in range(3)], fr]
    val = 0.0
    for q in range(8):
        dx, dy, dz = q & 1, (q >> 1) & 1, (q >> 2) & 1
        ci = [min(max(lo[0] + dx, 0), s[0] - 1), min(max(lo[1] + dy, 0), s[1] - 1), min(max(lo[2] + dz, 0), s[2] - 1)]
        val += v[tuple(ci)] * (w[dx][0] * w[dy][1] * w[dz][2])
    return val


def _case(n, seed):
    O = pytest.importorskip("oracle.oracle")
    O.build()
    sc = scenes().pool_sphere(n, seed=seed)
    og = oracle_grid(O, sc.grid)
    rng = np.random.default_rng(seed)
    H = [rng.uniform(-2, 2, sc.grid.face_shape(a)) for a in range(3)]
    marks, pos, nrm, kappa = contour(sc.grid.shape, sc.grid.spacing, tuple(sc.grid.origin), sc.phi, seed)
    return O, sc, og, H, marks, pos, nrm, kappa


def test_oracle_vertex_pressures_match_python():
    O, sc, og, H, marks, pos, nrm, kappa = _case(12, 1)
    chi = 1.7
    got = O.vertex_pressures(og, chi, H, pos, nrm)
    mu0 = 4e-7 * 3.141592653589793238462643383279502884
    o = tuple(float(x) for x in sc.grid.origin)
    for v in range(0, pos.shape[0], 7):
        hv = [_py_trilerp(o, sc.grid.spacing, H[b], b, pos[v]) for b in range(3)]
        coeff = (hv[0] * hv[0] + hv[1] * hv[1]) + hv[2] * hv[2]
        hn = (hv[0] * nrm[v][0] + hv[1] * nrm[v][1]) + hv[2] * nrm[v][2]
        coeff += chi * chi / (4 * chi + 4) * hn * hn
        assert got[v] == mu0 * 0.5 * chi * coeff
    assert pos.shape[0] > 50


def test_oracle_jump_matches_python():
    O, sc, og, H, marks, pos, nrm, kappa = _case(10, 2)
    pm = np.random.default_rng(3).uniform(0, 5, pos.shape[0])
    sigma, rho, dt = 0.07, 1200.0, 1e-3
    got = O.pressure_jump(og, marks, kappa, pm, sigma, rho, dt)
    invh = 1 / sc.grid.spacing
    for a in range(3):
        fs = sc.grid.face_shape(a)
        want = np.zeros(fs)
        for idx in np.ndindex(*fs):
            e = list(idx)
            e[a] -= 1
            if min(e) < 0 or any(e[b] >= marks[a].shape[b] for b in range(3)):
                continue
            v = marks[a][tuple(e)]
            if v >= 0:
                want[idx] = 0.0 + kappa[v] * sigma / rho * invh * dt
                want[idx] -= pm[v] / rho * invh * dt
        assert np.array_equal(got[a], want)
        assert np.count_nonzero(want) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("n,seed", [(24, 4), (33, 5)])
def test_vertex_pressures_and_jump_vs_oracle(sfpkg, gpu_ctx, n, seed):
    import torch
    O, sc, og, H, marks, pos, nrm, kappa = _case(n, seed)
    chi = 2.0
    want_pm = O.vertex_pressures(og, chi, H, pos, nrm)
    M = sfpkg.MagneticField(sc.grid, chi, 2 * sc.grid.spacing, gpu_ctx)
    pm = M.calculate_vertex_pressures(pos, nrm, H=H)
    assert np.array_equal(pm, want_pm)
    want_j = O.pressure_jump(og, marks, kappa, want_pm, 0.07, 1200.0, 1e-3)
    got_j = sfpkg.pressure_jump(sc.grid, marks, kappa, pm, 0.07, 1200.0, 1e-3, ctx=gpu_ctx)
    for a in range(3):
        assert np.array_equal(got_j[a], want_j[a])
    # device entry points
    dev = torch.device("cuda", 0)
    Hd = [torch.from_numpy(x).to(dev) for x in H]
    pd, nd = torch.from_numpy(pos).to(dev), torch.from_numpy(nrm).to(dev)
    pmd = torch.empty(pos.shape[0], dtype=torch.float64, device=dev)
    M.calculate_vertex_pressures(pd, nd, H=Hd, device=True, out=pmd)
    md = [torch.from_numpy(m).to(dev) for m in marks]
    jd = [torch.empty(sc.grid.face_shape(a), dtype=torch.float64, device=dev) for a in range(3)]
    sfpkg.pressure_jump(sc.grid, md, None, pmd, 0.0, 1200.0, 1e-3, ctx=gpu_ctx, device=True, out=jd)
    torch.cuda.synchronize()
    assert np.array_equal(pmd.cpu().numpy(), want_pm)
    want_j2 = O.pressure_jump(og, marks, None, want_pm, 0.0, 1200.0, 1e-3)
    for a in range(3):
        assert np.array_equal(jd[a].cpu().numpy(), want_j2[a])


@pytest.mark.gpu
def test_magnetic_to_pressure_chain_on_device(sfpkg, oracle, gpu_ctx):
    """Magnetic solve -> vertex pressures -> jump -> projection with that jump, all on device arrays, against the
    oracle chain fed with the GPU's total field (the solve itself differs within its tolerance)."""
    import torch
    sc = scenes().pool_sphere(32, seed=8)
    og = oracle_grid(oracle, sc.grid)
    dev = torch.device("cuda", 0)
    phi = torch.from_numpy(sc.phi).to(dev)
    hext = [torch.from_numpy(h).to(dev) for h in sc.hext]
    H = [torch.zeros(sc.grid.face_shape(a), dtype=torch.float64, device=dev) for a in range(3)]
    psi = torch.zeros(sc.grid.shape, dtype=torch.float64, device=dev)
    M = sfpkg.MagneticField(sc.grid, sc.chi, sc.band_width, gpu_ctx)
    M.solve(phi, hext, device=True, psi_out=psi, H_out=H, opts=sfpkg.options("magnetic", tol=1e-9))
    marks, pos, nrm, _ = contour(sc.grid.shape, sc.grid.spacing, tuple(sc.grid.origin), sc.phi, 9)
    pmd = torch.empty(pos.shape[0], dtype=torch.float64, device=dev)
    M.calculate_vertex_pressures(torch.from_numpy(pos).to(dev), torch.from_numpy(nrm).to(dev), device=True, out=pmd)
    jd = [torch.empty(sc.grid.face_shape(a), dtype=torch.float64, device=dev) for a in range(3)]
    sfpkg.pressure_jump(sc.grid, [torch.from_numpy(m).to(dev) for m in marks], None, pmd, 0.0, 1.0, 1e-2,
                        ctx=gpu_ctx, device=True, out=jd)
    vel = [torch.from_numpy(v.copy()).to(dev) for v in sc.vel]
    P = sfpkg.Pressure(sc.grid, gpu_ctx)
    P.set_pressure_jump(jd)
    p_out = torch.zeros(sc.grid.shape, dtype=torch.float64, device=dev)
    P.project(vel, phi, [torch.from_numpy(f).to(dev) for f in sc.frac], device=True, p_out=p_out,
              opts=sfpkg.options("pressure", tol=1e-10))
    torch.cuda.synchronize()
    Hh = [x.cpu().numpy() for x in H]
    pm = oracle.vertex_pressures(og, sc.chi, Hh, pos, nrm)
    assert np.array_equal(pmd.cpu().numpy(), pm)
    jump = oracle.pressure_jump(og, marks, None, pm, 0.0, 1.0, 1e-2)
    for a in range(3):
        assert np.array_equal(jd[a].cpu().numpy(), jump[a])
    u_or, p_or, _ = oracle.pressure_project(og, sc.phi, sc.frac, sc.vel, jump=jump, tol=1e-13)
    liquid = sc.phi <= 0
    assert np.abs(jump[0]).max() > 0
    assert rel_l2(p_out.cpu().numpy()[liquid], p_or[liquid]) <= 1e-5
