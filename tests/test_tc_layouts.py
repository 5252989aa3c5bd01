"""CPU emulation of the shared-memory layouts of the tcgen05 U-Net kernels (simferrofluid-cuda_gb300/csrc/sf_conv_tc.cuh):
where each TMA box lands, and which bytes each MMA's shared-memory descriptor reads.  The emulation places the data
as the TMA unit does (out-of-grid elements zero), reads the A and B operands through the descriptor addressing of
the K-major layouts (no swizzle: core matrices of 8 rows x 16 B, LBO between K halves, SBO = 128 B; 32-byte swizzle:
rows of 32 B whose 16-byte halves swap in rows 4-7 of every 256-byte atom, SBO = 256 B), multiplies them as the
MMA does, and compares the result with a direct convolution.  It also checks that every byte a descriptor reads
lies inside the buffer it addresses.  No GPU is needed; the kernel's constants are read from the header."""
import os
import re

import numpy as np
import pytest

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "simferrofluid-cuda_gb300", "csrc",
                   "sf_conv_tc.cuh")


def _const(name):
    m = re.search(r"\b%s\s*=\s*(\d+)" % name, open(HDR).read())
    assert m, name
    return int(m.group(1))


LZ, LY, SLACK = _const("kLineZ"), _const("kLineY"), _const("kWgSlack")


def _direct_forward(X, W):
    """Y[v][co] = sum_t W[t][co][ci] X[v + off(t)][ci], off(t) = (t/9 - 1, (t/3)%3 - 1, t%3 - 1), zero padding."""
    nx, ny, nz, _ = X.shape
    Xp = np.pad(X, ((1, 1), (1, 1), (1, 1), (0, 0)))
    Y = np.zeros((nx, ny, nz, W.shape[1]))
    for t in range(27):
        dx, dy, dz = t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1
        Y += np.einsum("xyzi,oi->xyzo", Xp[1 + dx:1 + dx + nx, 1 + dy:1 + dy + ny, 1 + dz:1 + dz + nz], W[t])
    return Y


def _swz32(byte):
    return byte ^ (((byte >> 7) & 1) << 4)


def _write_sw32(buf, base, rows):
    """TMA with CU_TENSOR_MAP_SWIZZLE_32B: row r (16 BF16) at base + 32 r, 16-byte halves swizzled."""
    r = np.arange(rows.shape[0])[:, None]
    e = np.arange(16)[None, :]
    buf[_swz32(base + r * 32 + (e // 8) * 16 + (e % 8) * 2) // 2] = rows


def _read_sw32(buf, start, m_rows):
    m = np.arange(m_rows)[:, None]
    k = np.arange(16)[None, :]
    byte = _swz32(start + (m // 8) * 256 + (m % 8) * 32 + (k // 8) * 16 + (k % 8) * 2)
    return buf[byte // 2], int(byte.max())


def _read_plain(buf, start, lbo, sbo, m_rows):
    m = np.arange(m_rows)[:, None]
    k = np.arange(16)[None, :]
    byte = start + (m // 8) * sbo + (m % 8) * 16 + (k // 8) * lbo + (k % 8) * 2
    return buf[byte // 2], int(byte.max())


@pytest.mark.parametrize("shape,ci,co", [((4, 6, 128), 16, 16), ((3, 7, 130), 16, 32), ((3, 6, 128), 32, 16),
                                         ((3, 6, 150), 32, 32)])
def test_line_kernel_layout(shape, ci, co):
    """k_conv_tc_line: bricks of 128 z x 4 y x LX x; a stage per (dz, 16 channels) is one box (16 ch, 128 z, 6 y,
    LX + 2 x) at (z0 + dz - 1, y0 - 1, x0 - 1) in the 32-byte swizzled layout; tile (yy, xx) of tap (dx, dy) starts
    4 KB x ((yy + 1 + dy) + 6 (xx + 1 + dx)) into it; the 27 taps' weights are resident, rows (tap, co) per
    16-channel group."""
    nx, ny, nz = shape
    lx = 2 if ci == 16 else 1
    kp = ci // 16
    rng = np.random.default_rng(1)
    X = rng.standard_normal(shape + (ci,))
    W = rng.standard_normal((27, co, ci))
    stage_bytes = LZ * (LY + 2) * (lx + 2) * 32
    wch = (27 * co * 32 + 1023) // 1024 * 1024
    wbuf = np.zeros(kp * wch // 2)
    for c in range(kp):
        _write_sw32(wbuf, c * wch, W[:, :, 16 * c:16 * c + 16].reshape(-1, 16))
    out = np.zeros((nx, ny, nz, co))
    bz_n, by_n, bx_n = -(-nz // LZ), -(-ny // LY), -(-nx // lx)
    Xp = np.zeros((nx + 2 + lx, ny + 2 + LY, nz + 2 + LZ, ci))  # zero outside the grid
    Xp[1:1 + nx, 1:1 + ny, 1:1 + nz] = X
    for br in range(bz_n * by_n * bx_n):
        z0, y0, x0 = LZ * (br % bz_n), LY * ((br // bz_n) % by_n), lx * (br // (bz_n * by_n))
        acc = np.zeros((LY * lx, 128, co))
        for st in range(3 * kp):
            dz, jp = st // kp, st % kp  # dz index 0..2 = shift dz - 1
            box = Xp[x0:x0 + lx + 2, y0:y0 + LY + 2, z0 + dz:z0 + dz + LZ, 16 * jp:16 * jp + 16]  # [x][y][z][16]
            stage = np.zeros(stage_bytes // 2)
            _write_sw32(stage, 0, box.reshape(-1, 16))
            for pr in range(9):
                dx, dy = pr // 3 - 1, pr % 3 - 1
                B, mb = _read_sw32(wbuf, jp * wch + (9 * (dx + 1) + 3 * (dy + 1) + dz) * co * 32, co)
                assert mb < kp * wch
                for tile in range(LY * lx):
                    yy, xx = tile % LY, tile // LY
                    A, ma = _read_sw32(stage, 4096 * ((yy + 1 + dy) + (LY + 2) * (xx + 1 + dx)), 128)
                    assert ma < stage_bytes
                    acc[tile] += A @ B.T
        for tile in range(LY * lx):
            yy, xx = y0 + tile % LY, x0 + tile // LY
            if yy < ny and xx < nx:
                zz = min(LZ, nz - z0)
                out[xx, yy, z0:z0 + zz] = acc[tile, :zz]
    ref = _direct_forward(X, W)
    assert np.abs(out - ref).max() <= 1e-9 * np.abs(ref).max()


@pytest.mark.parametrize("shape,ci,co", [((4, 4, 32), 16, 16), ((3, 5, 40), 16, 32), ((3, 5, 26), 32, 16),
                                         ((2, 4, 32), 64, 64)])
def test_weight_gradient_layout(shape, ci, co):
    """k_wgrad_tc: channel-major z-row copies dYT[zh][x][y][co][zl] and XT[zh][x][y][s][ci][zl] (three z shifts
    interleaved); a job is one (dx, dy) pair over a 32 z x 4 y x BX x brick, boxes (8, C, 4, BX, 4) landing as rows
    c + C k; MMA p reads A rows from 2p Cout 16 B (LBO Cout 16 B, SBO 128 B; rows past Cout land in unused lanes and
    may read the slack after the buffer) and B rows from 2p 3Cin 16 B; N = 3 Cin = three dz taps."""
    nx, ny, nz = shape
    bx = 2 if ci == 16 else 1
    N = 3 * ci
    rng = np.random.default_rng(2)
    X = rng.standard_normal(shape + (ci,))
    dY = rng.standard_normal(shape + (co,))
    nzh = (nz + 7) // 8

    def chmajor(src, C, ns, shift0):
        out = np.zeros((nzh, nx, ny, ns, C, 8))
        for s in range(ns):
            for zh in range(nzh):
                for zl in range(8):
                    z = 8 * zh + zl
                    zs = z + s + shift0
                    if z < nz and 0 <= zs < nz:
                        out[zh, :, :, s, :, zl] = src[:, :, zs, :]
        return out.reshape(nzh, nx, ny, ns * C, 8)

    def box(T, y, x, zh0):  # (8, C, 4, bx, 4) at (0, 0, y, x, zh0), lands [zh][x][y][c][8]
        C = T.shape[3]
        b = np.zeros((4, bx, 4, C, 8))
        for a in range(4):
            for xx in range(bx):
                for yy in range(4):
                    zh, xv, yv = zh0 + a, x + xx, y + yy
                    if 0 <= zh < nzh and 0 <= xv < nx and 0 <= yv < ny:
                        b[a, xx, yy] = T[zh, xv, yv]
        return b.reshape(-1)

    dYT, XT = chmajor(dY, co, 1, 0), chmajor(X, ci, 3, -1)
    a_bytes = 256 * co * bx
    acc = np.zeros((9, 128, N))
    bz_n, by_n, bx_n = -(-nz // 32), -(-ny // 4), -(-nx // bx)
    for br in range(bz_n * by_n * bx_n):
        z0, y0, x0 = 32 * (br % bz_n), 4 * ((br // bz_n) % by_n), bx * (br // (bz_n * by_n))
        abuf = np.concatenate([box(dYT, y0, x0, z0 // 8), np.zeros(SLACK // 2)])
        for pr in range(9):
            dx, dy = pr // 3 - 1, pr % 3 - 1
            bbuf = box(XT, y0 + dy, x0 + dx, z0 // 8)
            for p in range(8 * bx):
                A, ma = _read_plain(abuf, 2 * p * co * 16, co * 16, 128, 128)
                B, mb = _read_plain(bbuf, 2 * p * N * 16, N * 16, 128, N)
                assert ma < a_bytes + SLACK and mb < bbuf.size * 2
                acc[pr] += A @ B.T
    got = np.zeros((27, co, ci))
    for pr in range(9):
        for sz in range(3):
            got[3 * pr + sz] = acc[pr, :co, sz * ci:(sz + 1) * ci]
    Xp = np.pad(X, ((1, 1), (1, 1), (1, 1), (0, 0)))
    ref = np.zeros((27, co, ci))
    for t in range(27):
        dx, dy, dz = t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1
        ref[t] = np.einsum("xyzo,xyzi->oi", dY, Xp[1 + dx:1 + dx + nx, 1 + dy:1 + dy + ny, 1 + dz:1 + dz + nz])
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()


@pytest.mark.parametrize("shape,ci,co", [((4, 6, 64), 64, 64), ((5, 7, 70), 32, 64), ((4, 6, 64), 16, 32),
                                         ((4, 9, 64), 64, 16)])
def test_line64_kernel_layout(shape, ci, co):
    """k_conv_tc_line64: bricks of 64 z x 4 y x 2 x, four tiles of 64 z x 2 y; a stage per (dz, 16 channels) holds
    the box (16 ch, 64 z, 6 y, 4 x) at (z0 + dz - 1, y0 - 1, x0 - 1) and the weights of the nine taps of that z
    shift, rows (pr, co) of a copy whose taps are ordered 9 dz + pr; tile (ty, xx) of tap (dx, dy) starts
    2 KB x ((2 ty + 1 + dy) + 6 (xx + 1 + dx)) into the box."""
    z64, y4, x2 = _const("kL64Z"), _const("kL64Y"), _const("kL64X")
    nx, ny, nz = shape
    kp = ci // 16
    rng = np.random.default_rng(3)
    X = rng.standard_normal(shape + (ci,))
    W = rng.standard_normal((27, co, ci))
    Wp = np.stack([W[3 * (tp % 9) + tp // 9] for tp in range(27)])  # k_taps_dz_major
    a_bytes = z64 * (y4 + 2) * (x2 + 2) * 32
    w_raw = 9 * co * 32
    out = np.zeros((nx, ny, nz, co))
    bz_n, by_n, bx_n = -(-nz // z64), -(-ny // y4), -(-nx // x2)
    Xp = np.zeros((nx + 2 + x2, ny + 2 + y4, nz + 2 + z64, ci))
    Xp[1:1 + nx, 1:1 + ny, 1:1 + nz] = X
    tiles = (y4 // 2) * x2
    for br in range(bz_n * by_n * bx_n):
        z0, y0, x0 = z64 * (br % bz_n), y4 * ((br // bz_n) % by_n), x2 * (br // (bz_n * by_n))
        acc = np.zeros((tiles, 128, co))
        for st in range(3 * kp):
            dz, jp = st // kp, st % kp
            stage = np.zeros((a_bytes + (w_raw + 1023) // 1024 * 1024) // 2)
            _write_sw32(stage, 0, Xp[x0:x0 + x2 + 2, y0:y0 + y4 + 2, z0 + dz:z0 + dz + z64,
                                     16 * jp:16 * jp + 16].reshape(-1, 16))
            _write_sw32(stage, a_bytes, Wp[9 * dz:9 * dz + 9, :, 16 * jp:16 * jp + 16].reshape(-1, 16))
            for pr in range(9):
                dx, dy = pr // 3 - 1, pr % 3 - 1
                B, mb = _read_sw32(stage, a_bytes + pr * co * 32, co)
                assert a_bytes <= mb < a_bytes + w_raw
                for tile in range(tiles):
                    ty, xx = tile % (y4 // 2), tile // (y4 // 2)
                    A, ma = _read_sw32(stage, 2048 * ((2 * ty + 1 + dy) + (y4 + 2) * (xx + 1 + dx)), 128)
                    assert ma < a_bytes
                    acc[tile] += A @ B.T
        for tile in range(tiles):
            ty, xx = tile % (y4 // 2), tile // (y4 // 2)
            for m in range(128):
                z, yy, xv = z0 + m % z64, y0 + 2 * ty + m // z64, x0 + xx
                if z < nz and yy < ny and xv < nx:
                    out[xv, yy, z] = acc[tile, m]
    ref = _direct_forward(X, W)
    assert np.abs(out - ref).max() <= 1e-9 * np.abs(ref).max()


@pytest.mark.parametrize("shape,ci,co,mt", [((3, 8, 32), 16, 16, 4), ((2, 5, 40), 32, 16, 1), ((2, 8, 32), 64, 32, 2)])
def test_27_box_kernel_layout(shape, ci, co, mt):
    """k_conv_tc: a CTA takes MT tiles of 32 z x 4 y (one x plane); per tap and 8-channel chunk one box (8 ch,
    32 z, 4 MT y, 1 x) at (z0 + dz, y0 + dy, x0 + dx) lands as 128 MT rows of 16 B (no swizzle) and the tap's
    weights (8 ch, Cout) as Cout rows; MMA j (K = 16, chunks 2j and 2j + 1) of tile m reads A from
    2 j chunk + 2 KB m (LBO one chunk, SBO 128 B) and B from 2 j Cout 16 B (LBO Cout 16 B)."""
    nx, ny, nz = shape
    chunks = ci // 8
    rng = np.random.default_rng(4)
    X = rng.standard_normal(shape + (ci,))
    W = rng.standard_normal((27, co, ci))
    chunk_bytes = 128 * 16 * mt
    a_bytes, b_bytes = chunk_bytes * chunks, co * 16 * chunks
    Xp = np.zeros((nx + 2, ny + 2 + 4 * mt, nz + 2 + 32, ci))
    Xp[1:1 + nx, 1:1 + ny, 1:1 + nz] = X
    out = np.zeros((nx, ny, nz, co))
    tz, ty = -(-nz // 32), -(-ny // (4 * mt))
    for blk in range(tz * ty * nx):
        z0, y0, x0 = 32 * (blk % tz), 4 * mt * ((blk // tz) % ty), blk // (tz * ty)
        acc = np.zeros((mt, 128, co))
        for t in range(27):
            dx, dy, dz = t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1
            a = np.zeros(a_bytes // 2)
            b = np.zeros(b_bytes // 2)
            for c in range(chunks):  # box lands [y][z][8]
                box = Xp[1 + x0 + dx, 1 + y0 + dy:1 + y0 + dy + 4 * mt, 1 + z0 + dz:1 + z0 + dz + 32, 8 * c:8 * c + 8]
                a[c * chunk_bytes // 2:(c + 1) * chunk_bytes // 2] = box.reshape(-1)
                b[c * co * 8:(c + 1) * co * 8] = W[t, :, 8 * c:8 * c + 8].reshape(-1)
            for j in range(ci // 16):
                B, mb = _read_plain(b, j * 2 * co * 16, co * 16, 128, co)
                assert mb < b_bytes
                for m in range(mt):
                    A, ma = _read_plain(a, j * 2 * chunk_bytes + m * 2048, chunk_bytes, 128, 128)
                    assert ma < a_bytes
                    acc[m] += A @ B.T
        for m in range(mt):
            for r in range(128):  # TMEM lane = tile row: z = r % 32, y = 4 m + r / 32
                z, y = z0 + r % 32, y0 + 4 * m + r // 32
                if z < nz and y < ny:
                    out[x0, y, z] = acc[m, r]
    ref = _direct_forward(X, W)
    assert np.abs(out - ref).max() <= 1e-9 * np.abs(ref).max()
