// sf_rbgs_tma.cuh -- one-pass red-black Gauss-Seidel sweep of the finest FP32 level with TMA-staged planes.
//
// Same sweep as k_rbgs_fused (colour A on the tile plus a one-cell ring, then colour B on the tile, marching
// along x, out of place xin -> xout, bit-identical to the two in-place half sweeps of k_rbgs), with the global
// loads done by the tensor-memory accelerator: one elected thread issues, per x-plane, a 3-D box
// (z0-4 .. z0+TZ+3) x (y0-2 .. y0+TY+1) x 1 of each input array into a ring of shared-memory planes; an mbarrier
// per ring slot counts the bytes in.  Boxes that stick out of the grid are zero-filled by the TMA unit and
// never read.  Two groups with their own rings and barriers:
//   X: x_in and ax, needed from two steps before the plane's own step (5 slots: 3 live + 2 in flight)
//   C: ay, az, dex and b, needed from one step before (4 slots: 2 live + 2 in flight)
// Each array crosses HBM once per sweep (x in, x out, five operator arrays) instead of twice.  Every mbarrier
// wait is bounded (kWaitNs); after a timeout the block stops waiting, records the error in sc[err_slot], waits
// (bounded) for its loads in flight and returns; blocks that start after the error was recorded return at once.
#pragma once
#include "sf_internal.cuh"
#include "sf_tma.cuh"

namespace sf {
namespace rbt {

constexpr int TY = 8, TZ = 64;                    // tile of (y, z) per block; 256 threads = 32 (z pairs) x 8 (y)
constexpr int BY = TY + 4, BZ = TZ + 8;           // TMA box rows (y0-2 ..) and columns (z0-4 .., 16-byte aligned)
constexpr int PLANE = BY * BZ;                    // floats per staged plane
constexpr uint32_t kPlaneBytes = PLANE * 4;       // 3456 = 27 x 128
constexpr int RX = 5, RC = 4;                     // ring depths of the X and C groups
constexpr int RY = TY + 2, RZ = TZ + 2;           // colour-A values: tile + one-cell ring
constexpr uint64_t kWaitNs = 20000000;            // 20 ms per wait (a plane normally lands in microseconds)
constexpr size_t kSmemBytes = (size_t)kPlaneBytes * (2 * RX + 4 * RC) + sizeof(float) * 3 * RY * RZ +
                              8 * (RX + RC) + 128;  // + barriers + alignment slack

struct Maps {
    CUtensorMap x, ax, ay, az, dex, b;  // 3-D FP32 maps (nz, ny, nx), box (BZ, BY, 1)
};

__device__ __forceinline__ int ring3(int q) { return ((q % 3) + 3) % 3; }

// MODE 0: pre-smoothing from x = 0 (xin unused), A = red; MODE 1: pre-smoothing, A = red, B = black;
// MODE 2: post-smoothing, A = black, B = red.
template <int MODE>
__global__ void __launch_bounds__(256, 2) k_rbgs_tma(const __grid_constant__ Maps maps, Dims d, float *__restrict__ xout,
                                                     int xchunk, double *sc, int err_slot) {
    extern __shared__ __align__(128) uint8_t smem_raw[];
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    float *ringX = reinterpret_cast<float *>(base);                // [2 arrays][RX][PLANE]: x, ax
    float *ringC = ringX + 2 * RX * PLANE;                         // [4 arrays][RC][PLANE]: ay, az, dex, b
    float(*sa)[RY][RZ] = reinterpret_cast<float(*)[RY][RZ]>(ringC + 4 * RC * PLANE);
    uint64_t *bars = reinterpret_cast<uint64_t *>(reinterpret_cast<float *>(sa) + 3 * RY * RZ);  // RX + RC
    __shared__ int s_abort;

    const int colA = (MODE == 2) ? 1 : 0;
    // x-chunks vary fastest, then z-tiles: blocks running at the same time share their halo planes and rows
    // through L2
    const int x0 = blockIdx.x * xchunk, z0 = blockIdx.y * TZ, y0 = blockIdx.z * TY;
    const int x1 = min(x0 + xchunk, d.nx);
    const int tid = threadIdx.x + 32 * threadIdx.y;
    // plane ranges of the two groups (clipped to the grid)
    const int loX = max(x0 - 2, 0), hiX = min(x1 + 1, d.nx - 1);
    const int loC = max(x0 - 1, 0), hiC = min(x1, d.nx - 1);
    const uint32_t bytesX = (MODE == 0 ? 1u : 2u) * kPlaneBytes, bytesC = 4u * kPlaneBytes;
    const uint32_t barX0 = tc::smem_u32(bars), barC0 = barX0 + 8 * RX;

    auto slotX = [&](int q) { return (q - loX) % RX; };
    auto slotC = [&](int q) { return (q - loC) % RC; };
    // ring plane base pointers: slot arithmetic once per plane and step, not per cell
    auto xin_plane = [&](int q) { return ringX + slotX(q) * PLANE; };
    auto ax_plane = [&](int q) { return ringX + (RX + slotX(q)) * PLANE; };
    auto c_plane = [&](int arr, int q) { return ringC + (arr * RC + slotC(q)) * PLANE; };  // ay, az, dex, b

    int issuedX = loX - 1, issuedC = loC - 1;  // last plane issued (thread 0 only)
    int waitedX = loX - 1, waitedC = loC - 1;  // last plane waited for (thread 0 only)
    auto issue_to = [&](int qx, int qc) {       // thread 0: issue loads up to planes qx (X) and qc (C)
        qx = min(qx, hiX);
        qc = min(qc, hiC);
        for (int q = issuedX + 1; q <= qx; q++) {
            const uint32_t bar = barX0 + 8 * slotX(q);
            tc::mbar_expect_tx(bar, bytesX);
            float *dst = ringX + slotX(q) * PLANE;
            if (MODE != 0) tc::tma_load_3d(tc::smem_u32(dst), &maps.x, bar, z0 - 4, y0 - 2, q);
            tc::tma_load_3d(tc::smem_u32(dst + RX * PLANE), &maps.ax, bar, z0 - 4, y0 - 2, q);
        }
        if (qx > issuedX) issuedX = qx;
        for (int q = issuedC + 1; q <= qc; q++) {
            const uint32_t bar = barC0 + 8 * slotC(q);
            tc::mbar_expect_tx(bar, bytesC);
            float *dst = ringC + slotC(q) * PLANE;
            tc::tma_load_3d(tc::smem_u32(dst), &maps.ay, bar, z0 - 4, y0 - 2, q);
            tc::tma_load_3d(tc::smem_u32(dst + RC * PLANE), &maps.az, bar, z0 - 4, y0 - 2, q);
            tc::tma_load_3d(tc::smem_u32(dst + 2 * RC * PLANE), &maps.dex, bar, z0 - 4, y0 - 2, q);
            tc::tma_load_3d(tc::smem_u32(dst + 3 * RC * PLANE), &maps.b, bar, z0 - 4, y0 - 2, q);
        }
        if (qc > issuedC) issuedC = qc;
    };
    bool ok = true;
    auto wait_to = [&](int qx, int qc) {  // thread 0: planes up to qx (X) and qc (C) are in shared memory
        qx = min(qx, hiX);
        qc = min(qc, hiC);
        for (int q = waitedX + 1; q <= qx && ok; q++) {
            if (!tc::mbar_wait_ns(barX0 + 8 * slotX(q), (uint32_t)((q - loX) / RX) & 1u, kWaitNs)) ok = false;
            else waitedX = q;
        }
        for (int q = waitedC + 1; q <= qc && ok; q++) {
            if (!tc::mbar_wait_ns(barC0 + 8 * slotC(q), (uint32_t)((q - loC) / RC) & 1u, kWaitNs)) ok = false;
            else waitedC = q;
        }
    };

    // colour-A update of plane q on the tile + 1 ring (colour-B cells of the ring are not needed)
    auto compute_A = [&](int q) {
        float(*dst)[RZ] = sa[ring3(q)];
        if (q < 0 || q >= d.nx) {
            for (int e = tid; e < RY * RZ; e += 256) dst[e / RZ][e % RZ] = 0.f;
            return;
        }
        const int qm = max(q - 1, loX), qp = min(q + 1, hiX);
        const float *xm = xin_plane(qm), *xc = xin_plane(q), *xp = xin_plane(qp);
        const float *axq = ax_plane(q), *axp = ax_plane(qp);
        const float *ayq = c_plane(0, q), *azq = c_plane(1, q), *dq = c_plane(2, q), *bq = c_plane(3, q);
        for (int e = tid; e < RY * (RZ / 2); e += 256) {
            const int yy = e / (RZ / 2), pz = e - yy * (RZ / 2);
            const int y = y0 - 1 + yy;
            const int zz = 2 * pz + ((colA - q - y - z0 + 1) & 1);
            const int z = z0 - 1 + zz;
            float v = 0.f;
            if (y >= 0 && y < d.ny && z >= 0 && z < d.nz) {
                const int o = (yy + 1) * BZ + (zz + 3);  // box offset of (y, z)
                float s = 0.f, sum = 0.f;
                // y and z neighbours without guards: the stored lower-face couplings are 0 on the grid boundary
                // and the TMA boxes are zero-filled beyond it, so a missing face adds an exact zero (x guards
                // are uniform across the block and stay)
                if (MODE != 0) {
                    if (q > 0) {
                        const float a = axq[o];
                        s += a * xm[o];
                        sum += a;
                    }
                    if (q < d.nx - 1) {
                        const float a = axp[o];
                        s += a * xp[o];
                        sum += a;
                    }
                    float a = ayq[o];
                    s += a * xc[o - BZ];
                    sum += a;
                    a = ayq[o + BZ];
                    s += a * xc[o + BZ];
                    sum += a;
                    a = azq[o];
                    s += a * xc[o - 1];
                    sum += a;
                    a = azq[o + 1];
                    s += a * xc[o + 1];
                    sum += a;
                } else {
                    if (q > 0) sum += axq[o];
                    if (q < d.nx - 1) sum += axp[o];
                    sum += ayq[o];
                    sum += ayq[o + BZ];
                    sum += azq[o];
                    sum += azq[o + 1];
                }
                const float D = sum + dq[o];
                const float inv = D > 0.f ? 1.f / D : 0.f;
                v = (bq[o] + s) * inv;
            }
            dst[yy][zz] = v;
        }
    };
    // colour-B update of plane p on the tile; writes both colours of plane p (two cells per thread)
    auto update_B = [&](int p) {
        const int ty = threadIdx.y, y = y0 + ty;
        const int tz0 = 2 * threadIdx.x, z = z0 + tz0;
        if (y >= d.ny || z >= d.nz) return;
        const float(*am)[RZ] = sa[ring3(p - 1)];
        const float(*a0)[RZ] = sa[ring3(p)];
        const float(*ap)[RZ] = sa[ring3(p + 1)];
        const float *axq = ax_plane(p), *axp = ax_plane(min(p + 1, hiX));
        const float *ayq = c_plane(0, p), *azq = c_plane(1, p), *dq = c_plane(2, p), *bq = c_plane(3, p);
        float out[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int tz = tz0 + h, zc = z + h;
            const int ry = ty + 1, rz = tz + 1;
            if (((p + y + zc) & 1) == colA) {
                out[h] = a0[ry][rz];
                continue;
            }
            const int o = (ty + 2) * BZ + (tz + 4);
            float s = 0.f, sum = 0.f;
            if (p > 0) {
                const float a = axq[o];
                s += a * am[ry][rz];
                sum += a;
            }
            if (p < d.nx - 1) {
                const float a = axp[o];
                s += a * ap[ry][rz];
                sum += a;
            }
            float a = ayq[o];  // y and z faces unguarded, as in compute_A
            s += a * a0[ry - 1][rz];
            sum += a;
            a = ayq[o + BZ];
            s += a * a0[ry + 1][rz];
            sum += a;
            a = azq[o];
            s += a * a0[ry][rz - 1];
            sum += a;
            a = azq[o + 1];
            s += a * a0[ry][rz + 1];
            sum += a;
            const float D = sum + dq[o];
            const float inv = D > 0.f ? 1.f / D : 0.f;
            out[h] = (bq[o] + s) * inv;
        }
        // nz is a multiple of 4 and z even: both cells are in the grid, 8-byte aligned
        *reinterpret_cast<float2 *>(xout + cid(d, p, y, z)) = make_float2(out[0], out[1]);
    };

    if (tid == 0) {
        // another block already timed out: the sweep's result is void, return without loading anything
        s_abort = *reinterpret_cast<volatile double *>(sc + err_slot) != 0.0 ? 1 : 0;
        for (int i = 0; i < RX + RC; i++) tc::mbar_init(barX0 + 8 * i, 1);
        tc::mbar_fence_init();
        // prologue: X planes x0-2 .. x0+2 and C planes x0-1 .. x0+2 fill both rings
        if (!s_abort) issue_to(x0 + 2, x0 + 2);
    }
    __syncthreads();
    if (s_abort) return;
    // Thread 0 alone waits on the mbarriers; the CTA barrier after its wait makes the landed planes (and the
    // abort decision) visible to every thread.
    if (tid == 0) {
        wait_to(x0 + 1, x0);
        if (!ok) s_abort = 1;
    }
    __syncthreads();
    if (!s_abort) {
        compute_A(x0 - 1);  // x_in x0-2 .. x0, C x0-1
        compute_A(x0);      // x_in x0-1 .. x0+1, C x0
        for (int p = x0; p < x1; p++) {
            __syncthreads();  // step p-1 complete: X and C planes <= p-1 are dead, colour-A plane p-2 too
            if (tid == 0) {
                issue_to(p + 4, p + 3);
                wait_to(p + 2, p + 1);
                if (!ok) s_abort = 1;
            }
            __syncthreads();
            if (s_abort) break;
            compute_A(p + 1);  // x_in p .. p+2, ax p+1 .. p+2, C p+1; overwrites colour-A plane p-2
            __syncthreads();
            update_B(p);  // ax p .. p+1, C p, colour A p-1 .. p+1
        }
    }
    if (s_abort) {
        if (tid == 0) {
            sc[err_slot] = 1.0;  // a TMA load did not arrive in time
            // let the loads still in flight land before the block's shared memory is released
            for (int q = waitedX + 1; q <= issuedX; q++)
                tc::mbar_wait_ns(barX0 + 8 * slotX(q), (uint32_t)((q - loX) / RX) & 1u, kWaitNs);
            for (int q = waitedC + 1; q <= issuedC; q++)
                tc::mbar_wait_ns(barC0 + 8 * slotC(q), (uint32_t)((q - loC) / RC) & 1u, kWaitNs);
        }
    }
}

}  // namespace rbt
}  // namespace sf
