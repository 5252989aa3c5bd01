"""The velocity pipeline after the projection (core/Simulation.cpp:236-241): Extrapolation::Solve and
Collider::Enforce.

CPU: the library's collider face normals against the oracle (bit for bit), and the oracle's extrapolation and
enforce against an independent pure-Python restatement on small grids (pins the C oracle).
GPU: both kernels against the oracle bit for bit (the kernels are compiled without fused multiply-add and
evaluate in the reference's order), through the host and device entry points, and chained after a projection."""
import math

import numpy as np
import pytest

from conftest import oracle_grid, pkg, scenes


# ------------------------------------------------------------------------------------------ pure-Python checks
def _py_extrapolate(u, valid, clear, steps):
    """Extrapolation::Solve on one face grid (core/Extrapolation.cpp:4-30), in plain loops."""
    u = u.copy()
    valid = valid.copy()
    valid1 = valid.copy()
    s = u.shape
    for _ in range(steps):
        for i in range(s[0]):
            for j in range(s[1]):
                for k in range(s[2]):
                    if not valid[i, j, k]:
                        cnt, tot = 0, 0.0
                        for d in ((-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)):
                            q = (i + d[0], j + d[1], k + d[2])
                            if all(0 <= q[a] < s[a] for a in range(3)) and valid[q]:
                                tot += u[q]
                                cnt += 1
                        if cnt:
                            u[i, j, k] = tot / cnt
                            valid1[i, j, k] = True
                        else:
                            u[i, j, k] = clear
                    else:
                        valid1[i, j, k] = True
        valid, valid1 = valid1, valid
    return u


def _py_valid(g, phi, frac, a):
    fs = g.face_shape(a)
    v = np.zeros(fs, bool)
    n = (g.nx, g.ny, g.nz)
    for i in range(fs[0]):
        for j in range(fs[1]):
            for k in range(fs[2]):
                if not frac[a][i, j, k] < 1:
                    continue
                c1 = (i, j, k)
                c0 = list(c1)
                c0[a] -= 1
                liq = lambda c: all(0 <= c[b] < n[b] for b in range(3)) and phi[tuple(c)] <= 0
                v[i, j, k] = liq(c0) or liq(c1)
    return v


def _py_trilerp(g, v, b, p):
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


def _py_enforce(g, u, frac, normal):
    new = [a.copy() for a in u]
    o = tuple(float(x) for x in g.origin)
    for a in range(3):
        for idx in zip(*np.nonzero(frac[a] == 1.0)):
            p = [(o[b] if b == a else o[b] + g.h / 2) + idx[b] * g.h for b in range(3)]
            vel = [_py_trilerp(g, u[b], b, p) for b in range(3)]
            n = [_py_trilerp(g, normal[b], b, p) for b in range(3)]
            nn = math.sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2])
            if nn > 0:
                n = [x / nn for x in n]
            dn = (vel[0] * n[0] + vel[1] * n[1]) + vel[2] * n[2]
            new[a][idx] = vel[a] - dn * n[a]
    return new


def _small_case(shape, seed):
    O = pytest.importorskip("oracle.oracle")
    O.build()
    g = O.Grid(*shape, 1.0 / shape[0], (0.0, 0.0, 0.0))
    rng = np.random.default_rng(seed)
    ys = (np.arange(shape[1]) + 0.5) / shape[0]
    phi = np.broadcast_to((ys - 0.4 * ys.max())[None, :, None], shape) + 0.03 * rng.uniform(-1, 1, shape)
    phi = np.ascontiguousarray(phi)
    ls, frac, normal = O.box_collider(g)
    u = [rng.uniform(-1, 1, g.face_shape(a)) for a in range(3)]
    return O, g, phi, ls, frac, normal, u


def test_oracle_extrapolation_matches_python():
    O, g, phi, ls, frac, normal, u = _small_case((7, 6, 9), 1)
    got = O.extrapolate_velocity(g, u, phi, frac, 0.0, 6)
    for a in range(3):
        want = _py_extrapolate(u[a], _py_valid(g, phi, frac, a), 0.0, 6)
        assert np.array_equal(got[a], want)


def test_oracle_enforce_matches_python():
    O, g, phi, ls, frac, normal, u = _small_case((6, 5, 7), 2)
    got = O.collider_enforce(g, u, frac, normal)
    want = _py_enforce(g, u, frac, normal)
    for a in range(3):
        assert np.array_equal(got[a], want[a])
        assert np.any(got[a] != u[a])  # the walls were touched


def test_library_normals_match_oracle():
    O, g, phi, ls, frac, normal, u = _small_case((9, 7, 11), 3)
    sf = pkg()
    sg = sf.StaggeredGrid.from_origin(g.h, (g.nx, g.ny, g.nz))
    got = sf.collider_face_normals(sg, ls)
    for a in range(3):
        assert np.array_equal(got[a], normal[a])


# ------------------------------------------------------------------------------------------------ GPU parity
@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(24, 24, 24), (13, 9, 17)])
def test_extrapolate_and_enforce_vs_oracle(sfpkg, oracle, gpu_ctx, shape):
    rng = np.random.default_rng(sum(shape))
    g = sfpkg.StaggeredGrid.from_origin(1.0 / shape[0], shape)
    og = oracle_grid(oracle, g)
    ys = scenes().cell_centres(g, 1)
    phi = np.ascontiguousarray(np.broadcast_to((ys - 0.45 * ys.max())[None, :, None], g.shape)) \
        + 0.05 * rng.uniform(-1, 1, g.shape)
    ls, frac, normal = oracle.box_collider(og)
    u = [rng.uniform(-1, 1, g.face_shape(a)) for a in range(3)]
    want = oracle.extrapolate_velocity(og, u, phi, frac, 0.0, 6)
    v = [a.copy() for a in u]
    sfpkg.Extrapolation(g, gpu_ctx).solve(v, phi, frac, 0.0, 6)
    for a in range(3):
        assert np.array_equal(v[a], want[a])
    want2 = oracle.collider_enforce(og, want, frac, normal)
    sfpkg.ColliderEnforce(g, frac, normal, ctx=gpu_ctx).enforce(v)
    for a in range(3):
        assert np.array_equal(v[a], want2[a])


@pytest.mark.gpu
def test_post_pipeline_on_device_after_projection(sfpkg, oracle, gpu_ctx):
    """Project -> Extrapolation::Solve -> Collider::Enforce on device arrays (the velocity stays resident), against
    the oracle chain: bit for bit after the projection's own (solver-tolerance) differences are taken out by
    feeding both pipelines the GPU's projected velocity."""
    import torch
    sc = scenes().pool(32, seed=6)
    og = oracle_grid(oracle, sc.grid)
    ls, frac, normal = oracle.box_collider(og)
    dev = torch.device("cuda", 0)
    vel = [torch.from_numpy(v.copy()).to(dev) for v in sc.vel]
    phi = torch.from_numpy(sc.phi).to(dev)
    fr = [torch.from_numpy(f).to(dev) for f in frac]
    nm = [torch.from_numpy(n).to(dev) for n in normal]
    sfpkg.Pressure(sc.grid, gpu_ctx).project(vel, phi, fr, device=True)
    torch.cuda.synchronize()
    projected = [v.cpu().numpy() for v in vel]
    sfpkg.Extrapolation(sc.grid, gpu_ctx).solve(vel, phi, fr, device=True)
    sfpkg.ColliderEnforce(sc.grid, fr, nm, ctx=gpu_ctx).enforce(vel, device=True)
    torch.cuda.synchronize()
    want = oracle.collider_enforce(og, oracle.extrapolate_velocity(og, projected, sc.phi, frac), frac, normal)
    for a in range(3):
        assert np.array_equal(vel[a].cpu().numpy(), want[a])
