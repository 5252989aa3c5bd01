"""Independent pure-Python restatement of the reference's hot-path assembly, for small grids only.

TEST INFRASTRUCTURE: a second witness for the C oracle (oracle/sf_oracle.c), written separately from it,
loop for loop from the reference sources:
  * Pressure::SetUnKnowns / BuildProjectionMatrix / SetRightHandSide / ApplyProjection
    (core/Pressure.cpp:38-166)
  * MagneticField BuildMatrix (mu with TriLerp::Interpolate, core/TriLerp.h:22-67) / AssembleRHS /
    AssignTotalField (core/MagneticField.cpp:50-143), Heaviside (core/MagneticField.h:44-54)
Python floats are IEEE doubles and Python never fuses a*b+c, so with the reference's evaluation order the
results are bit-identical to the reference's x86 build.
"""
from __future__ import annotations

import math

NB = [(-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)]


class G:
    def __init__(self, nx, ny, nz, h, origin=(0.0, 0.0, 0.0)):
        self.n = (nx, ny, nz)
        self.h = h
        self.o = tuple(origin)

    def idx(self, c):
        return c[2] + self.n[2] * (c[1] + self.n[1] * c[0])

    def coord(self, r):
        nx, ny, nz = self.n
        return (r // nz // ny, r // nz % ny, r % nz)

    def valid(self, c):
        return all(0 <= c[a] < self.n[a] for a in range(3))

    def fshape(self, a):
        return tuple(self.n[b] + (1 if b == a else 0) for b in range(3))

    def fidx(self, a, f):
        s = self.fshape(a)
        return f[2] + s[2] * (f[1] + s[1] * f[0])

    @property
    def N(self):
        return self.n[0] * self.n[1] * self.n[2]


def _face_of_cell(c, ord_):
    a = ord_ >> 1
    f = list(c)
    f[a] += ord_ & 1
    return a, tuple(f)


def _nb(c, ord_):
    d = NB[ord_]
    return (c[0] + d[0], c[1] + d[1], c[2] + d[2])


def _side(ord_):
    return 1 if ord_ & 1 else -1


def _weight(g, frac, c, ord_):
    a, f = _face_of_cell(c, ord_)
    if not g.valid(_nb(c, ord_)):
        return a, f, 0.0  # closed outer wall (see the C ABI documentation)
    return a, f, 1 - frac[a][g.fidx(a, f)]


def pressure_assemble(g, phi, frac, u, us=None, jump=None, vol_error=0.0):
    """Returns (rows: list of dict col->val, rhs list, grid2mat, mat2grid)."""
    g2m = [-1] * g.N
    m2g = []
    for r in range(g.N):  # ForEach is x, y, z lexicographic == flat index order
        if phi[r] <= 0:
            g2m[r] = len(m2g)
            m2g.append(r)
    rows, rhs = [], []
    for r, cell_idx in enumerate(m2g):
        cell = g.coord(cell_idx)
        diag = 0.0
        div = 0.0
        row = {}
        for i in range(6):
            nbc = _nb(cell, i)
            a, f, w = _weight(g, frac, cell, i)
            side = _side(i)
            fi = g.fidx(a, f)
            if w > 0:
                cn = g2m[g.idx(nbc)]
                if cn >= 0:
                    diag += w
                    row[cn] = -w
                else:
                    theta = phi[cell_idx] / (phi[cell_idx] - phi[g.idx(nbc)])
                    ic = 1.0 / max(theta, 0.001)
                    diag += w * ic
                    if jump is not None:
                        div += jump[a][fi] * w * ic
                div -= side * w * u[a][fi]
            if w < 1:
                usv = 0.0 if us is None else us[a][fi]
                div -= side * (1 - w) * usv
        div += vol_error
        rhs.append(div)
        row[r] = diag if diag else 1.0
        rows.append(row)
    return rows, rhs, g2m, m2g


def pressure_apply(g, phi, frac, jump, g2m, p, u):
    out = [list(x) for x in u]
    for a in range(3):
        s = g.fshape(a)
        for i in range(s[0]):
            for j in range(s[1]):
                for k in range(s[2]):
                    f = (i, j, k)
                    c0 = list(f)
                    c0[a] -= 1
                    c0 = tuple(c0)
                    if not g.valid(c0) or not g.valid(f):
                        continue
                    fi = g.fidx(a, f)
                    w = 1.0 - frac[a][fi]
                    if w == 0.0:
                        continue
                    id0, id1 = g2m[g.idx(c0)], g2m[g.idx(f)]
                    if id0 < 0 and id1 < 0:
                        continue
                    if id0 >= 0 and id1 >= 0:
                        out[a][fi] -= (p[id1] - p[id0]) * w
                    else:
                        phi0, phi1 = phi[g.idx(c0)], phi[g.idx(f)]
                        theta = phi0 / (phi0 - phi1)
                        pin = p[id0] if id0 >= 0 else p[id1]
                        pj = jump[a][fi] if jump is not None else 0.0
                        ic = 1.0 / max(theta if id0 >= 0 else 1 - theta, 0.001)
                        out[a][fi] -= (1 if id0 >= 0 else -1) * (pj - pin) * ic * w
    return out


def heaviside(phi, bw):
    if phi < -bw:
        return 0.0
    if phi > bw:
        return 1.0
    return 0.5 * (1.0 + phi / bw + math.sin(math.pi * phi / bw) / math.pi)


def trilerp(g, phi, pos):
    co = tuple(g.o[a] + g.h / 2 for a in range(3))
    invh = 1 / g.h
    lo = [math.floor((pos[a] - co[a]) * invh - 0.0) for a in range(3)]
    fr = [(pos[a] - co[a] - lo[a] * g.h) * invh for a in range(3)]
    w = [[1.0 - fr[a] for a in range(3)], fr]
    val = 0.0
    for q in range(8):
        d = (q & 1, (q >> 1) & 1, (q >> 2) & 1)
        c = [min(max(lo[a] + d[a], 0), g.n[a] - 1) for a in range(3)]
        wt = w[d[0]][0] * w[d[1]][1] * w[d[2]][2]
        val += phi[g.idx(c)] * wt
    return val


def magnetic_origin(g):
    out = []
    for a in range(3):
        half = g.n[a] * g.h / 2.0
        center = g.o[a] + half
        out.append(center - g.n[a] * g.h / 2)
    return tuple(out)


def magnetic_coeff(g, phi, chi, bw):
    eo = magnetic_origin(g)
    mu = []
    for a in range(3):
        s = g.fshape(a)
        fo = tuple(eo[b] + (0 if b == a else 1) * g.h / 2 for b in range(3))
        arr = [0.0] * (s[0] * s[1] * s[2])
        for i in range(s[0]):
            for j in range(s[1]):
                for k in range(s[2]):
                    f = (i, j, k)
                    if f[a] <= 0 or f[a] >= g.n[a]:
                        v = 1.0
                    else:
                        pos = tuple(fo[b] + f[b] * g.h for b in range(3))
                        v = 1.0 + (1.0 - heaviside(trilerp(g, phi, pos), bw)) * chi
                    arr[g.fidx(a, f)] = v
        mu.append(arr)
    return mu


def magnetic_assemble(g, mu):
    rows = []
    for r in range(g.N):
        if r == 0:
            rows.append({0: 1.0})
            continue
        cell = g.coord(r)
        diag = 0.0
        row = {}
        for i in range(6):
            nbc = _nb(cell, i)
            if not g.valid(nbc):
                continue
            a, f = _face_of_cell(cell, i)
            w = mu[a][g.fidx(a, f)]
            col = g.idx(nbc)
            if col != 0:
                row[col] = -w
            diag += w
        row[r] = diag
        rows.append(row)
    return rows


def magnetic_rhs(g, mu, hext):
    rhs = [0.0] * g.N
    for r in range(1, g.N):
        cell = g.coord(r)
        for i in range(6):
            nbc = _nb(cell, i)
            if not g.valid(nbc):
                continue
            a, f = _face_of_cell(cell, i)
            side = _side(i)
            w = mu[a][g.fidx(a, f)]
            rhs[r] += (w - 1.0) * hext[a][g.fidx(a, f)] * (-side) * g.h
    return rhs


def magnetic_total_field(g, psi, hext):
    invh = 1 / g.h
    H = []
    for a in range(3):
        s = g.fshape(a)
        arr = [0.0] * (s[0] * s[1] * s[2])
        for i in range(s[0]):
            for j in range(s[1]):
                for k in range(s[2]):
                    f = (i, j, k)
                    c0 = list(f)
                    c0[a] -= 1
                    c0 = tuple(c0)
                    fi = g.fidx(a, f)
                    v = 0.0
                    if g.valid(c0) and g.valid(f):
                        v = (psi[g.idx(c0)] - psi[g.idx(f)]) * invh
                    v += hext[a][fi]
                    arr[fi] = v
        H.append(arr)
    return H


def rows_to_csr(rows):
    import numpy as np
    rowptr = [0]
    col, val = [], []
    for row in rows:
        for c in sorted(row):
            col.append(c)
            val.append(row[c])
        rowptr.append(len(col))
    return np.array(rowptr, np.int64), np.array(col, np.int32), np.array(val)
