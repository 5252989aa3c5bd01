"""Level-set neighbours of the path (core/Simulation.cpp:164-165, 265): semi-Lagrangian advection of the level
set (TVD RK2 trace, tricubic TriCuInterp) and of the velocity by itself (trilinear), and the WENO5/TVD-RK3
reinitialisation.

CPU: the oracle against plain-Python restatements on small grids (pins the C oracle).  GPU: the kernels against
the oracle bit for bit (compiled without fused multiply-add, evaluated in the reference's order), through the host
and device entry points."""
import math

import numpy as np
import pytest

from conftest import oracle_grid


def _py_trilerp_face(g, v, b, p):
    o = tuple(float(x) for x in g.origin)
    co = [o[a] if a == b else o[a] + g.h / 2 for a in range(3)]
    s = v.shape
    lo = [math.floor((p[a] - co[a]) * (1 / g.h) - 0.0) for a in range(3)]
    fr = [(p[a] - co[a] - lo[a] * g.h) * (1 / g.h) for a in range(3)]
    w = [[1.0 - fr[a] for a in range(3)], fr]
    val = 0.0
    for q in range(8):
        dx, dy, dz = q & 1, (q >> 1) & 1, (q >> 2) & 1
        ci = [min(max(lo[0] + dx, 0), s[0] - 1), min(max(lo[1] + dy, 0), s[1] - 1), min(max(lo[2] + dz, 0), s[2] - 1)]
        val += v[tuple(ci)] * (w[dx][0] * w[dy][1] * w[dz][2])
    return val


def _py_trace(g, u, p, dt):
    v0 = [_py_trilerp_face(g, u[b], b, p) for b in range(3)]
    q = [p[a] + v0[a] * dt for a in range(3)]
    v1 = [_py_trilerp_face(g, u[b], b, q) for b in range(3)]
    return [p[a] + (v0[a] + v1[a]) * dt / 2 for a in range(3)]


def _py_tricubic(g, f, p):
    o = tuple(float(x) for x in g.origin)
    co = [o[a] + g.h / 2 for a in range(3)]
    s = f.shape
    lo = [math.floor((p[a] - co[a]) * (1 / g.h) - 1.0) for a in range(3)]
    w = [[0.0] * 3 for _ in range(4)]
    for a in range(3):
        fr = (p[a] - co[a] - lo[a] * g.h) * (1 / g.h)
        w[0][a] = (fr - 1) * (fr - 2) * (fr - 3) / -6
        w[1][a] = fr * (fr - 2) * (fr - 3) / 2
        w[2][a] = fr * (fr - 1) * (fr - 3) / -2
        w[3][a] = fr * (fr - 1) * (fr - 2) / 6
    val = 0.0
    for k in range(4):
        for j in range(4):
            for i in range(4):
                ci = [min(max(lo[0] + i, 0), s[0] - 1), min(max(lo[1] + j, 0), s[1] - 1),
                      min(max(lo[2] + k, 0), s[2] - 1)]
                val += f[tuple(ci)] * (w[i][0] * w[j][1] * w[k][2])
    return val


def _py_weno(v, s, invdx):
    dev = [v[6] - v[5], v[5] - v[4], v[4] - v[3], v[3] - v[2], v[2] - v[1]] if s else \
        [v[1] - v[0], v[2] - v[1], v[3] - v[2], v[4] - v[3], v[5] - v[4]]
    eps = 0.0
    for d in dev:
        eps = max(eps, d * d)
    eps = eps * 1e-6 + 1e-99
    p1 = dev[0] / 3 - dev[1] * 7 / 6 + dev[2] * 11 / 6
    p2 = -dev[1] / 6 + dev[2] * 5 / 6 + dev[3] / 3
    p3 = dev[2] / 3 + dev[3] * 5 / 6 - dev[4] / 6
    sq = lambda x: x * x  # noqa: E731
    s1 = sq(dev[0] - 2 * dev[1] + dev[2]) * 13 / 12 + sq(dev[0] - 4 * dev[1] + 3 * dev[2]) / 4
    s2 = sq(dev[1] - 2 * dev[2] + dev[3]) * 13 / 12 + sq(dev[1] - dev[3]) / 4
    s3 = sq(dev[2] - 2 * dev[3] + dev[4]) * 13 / 12 + sq(3 * dev[2] - 4 * dev[3] + dev[4]) / 4
    a1, a2, a3 = .1 / sq(s1 + eps), .6 / sq(s2 + eps), .3 / sq(s3 + eps)
    return (a1 * p1 + a2 * p2 + a3 * p3) / (a1 + a2 + a3) * invdx


def _py_advance(g, f):
    out = np.empty_like(f)
    s = f.shape
    for idx in np.ndindex(*s):
        tot = 0.0
        for a in range(3):
            v = []
            for q in range(7):
                c = list(idx)
                c[a] = min(max(c[a] + q - 3, 0), s[a] - 1)
                v.append(f[tuple(c)])
            dm, dp = _py_weno(v, 0, 1 / g.h), _py_weno(v, 1, 1 / g.h)
            if f[idx] < 0:
                tot += min(dm, 0.0) ** 2
                tot += max(dp, 0.0) ** 2
            else:
                tot += max(dm, 0.0) ** 2
                tot += min(dp, 0.0) ** 2
        tot = math.sqrt(tot)
        fc = f[idx]
        out[idx] = fc + g.h * .5 * (fc / math.sqrt(fc * fc + (g.h * tot) ** 2)) * (1.0 - tot)
    return out


def _case(shape, seed):
    O = pytest.importorskip("oracle.oracle")
    O.build()
    g = O.Grid(*shape, 1.0 / shape[0], (0.0, 0.0, 0.0))
    rng = np.random.default_rng(seed)
    c = [(np.arange(shape[a]) + 0.5) / shape[0] for a in range(3)]
    X, Y, Z = np.meshgrid(*c, indexing="ij")
    phi = np.sqrt((X - 0.5) ** 2 + (Y - 0.4) ** 2 + (Z - 0.55) ** 2) * 1.7 - 0.3 + 0.02 * rng.uniform(-1, 1, shape)
    u = [rng.uniform(-1, 1, g.face_shape(a)) for a in range(3)]
    return O, g, np.ascontiguousarray(phi), u


def test_oracle_advection_matches_python():
    O, g, phi, u = _case((7, 6, 8), 1)
    dt = 0.09
    got = O.advect_levelset(g, phi, u, dt)
    gu = O.advect_velocity(g, u, dt)
    o = tuple(float(x) for x in g.origin)
    for idx in [(0, 0, 0), (3, 2, 4), (6, 5, 7), (1, 4, 2)]:
        p = [o[a] + g.h / 2 + idx[a] * g.h for a in range(3)]
        assert got[idx] == _py_tricubic(g, phi, _py_trace(g, u, p, -dt))
    for a in range(3):
        for idx in [(0, 0, 0), (2, 3, 4), tuple(s - 1 for s in g.face_shape(a))]:
            p = [(o[b] if b == a else o[b] + g.h / 2) + idx[b] * g.h for b in range(3)]
            assert gu[a][idx] == _py_trilerp_face(g, u[a], a, _py_trace(g, u, p, -dt))


def test_oracle_reinitialization_matches_python():
    O, g, phi, u = _case((6, 5, 7), 2)
    # one TVD-RK3 step restated in Python
    p1 = _py_advance(g, phi)
    p2 = _py_advance(g, p1)
    p1 = (phi * 3 + p2) / 4
    p2 = _py_advance(g, p1)
    want = (phi + p2 * 2) / 3
    assert np.array_equal(O.reinitialize(g, phi, 1), want)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(24, 24, 24), (13, 9, 17)])
def test_levelset_ops_vs_oracle(sfpkg, oracle, gpu_ctx, shape):
    import torch
    O, og0, phi, u = _case(shape, sum(shape))
    g = sfpkg.StaggeredGrid.from_origin(1.0 / shape[0], shape)
    og = oracle_grid(oracle, g)
    dt = 0.7 / shape[0]
    want_phi = oracle.advect_levelset(og, phi, u, dt)
    p = phi.copy()
    sfpkg.Advection(g, gpu_ctx).solve_levelset(p, u, dt)
    assert np.array_equal(p, want_phi)
    want_u = oracle.advect_velocity(og, u, dt)
    v = [a.copy() for a in u]
    sfpkg.Advection(g, gpu_ctx).solve_velocity(v, dt)
    for a in range(3):
        assert np.array_equal(v[a], want_u[a])
    want_r = oracle.reinitialize(og, want_phi, 3)
    sfpkg.Reinitialization(g, gpu_ctx).solve(p, 3)
    assert np.array_equal(p, want_r)
    # device entry points, chained as a substep does: advect phi, advect u, reinitialise phi
    dev = torch.device("cuda", 0)
    pd = torch.from_numpy(phi.copy()).to(dev)
    ud = [torch.from_numpy(a.copy()).to(dev) for a in u]
    sfpkg.Advection(g, gpu_ctx).solve_levelset(pd, ud, dt, device=True)
    sfpkg.Advection(g, gpu_ctx).solve_velocity(ud, dt, device=True)
    sfpkg.Reinitialization(g, gpu_ctx).solve(pd, 3, device=True)
    torch.cuda.synchronize()
    assert np.array_equal(pd.cpu().numpy(), want_r)
    for a in range(3):
        assert np.array_equal(ud[a].cpu().numpy(), want_u[a])


@pytest.mark.gpu
def test_reinitialization_restores_distance(sfpkg, gpu_ctx):
    """A property at a larger size: reinitialising a stretched sphere level set brings |grad phi| near 1 close to
    the interface without moving the interface by more than a fraction of a cell."""
    n = 64
    g = sfpkg.StaggeredGrid.from_origin(1.0 / n, (n, n, n))
    c = (np.arange(n) + 0.5) / n
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    r = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2)
    phi = np.ascontiguousarray(3.0 * (r - 0.3))  # |grad| = 3
    sfpkg.Reinitialization(g, gpu_ctx).solve(phi, 10)
    band = np.abs(r - 0.3) < 2.5 / n
    gx, gy, gz = np.gradient(phi, 1.0 / n)
    gn = np.sqrt(gx * gx + gy * gy + gz * gz)[band]
    assert abs(np.median(gn) - 1.0) < 0.05
    assert np.abs(phi[band] - (r[band] - 0.3)).max() < 0.5 / n
