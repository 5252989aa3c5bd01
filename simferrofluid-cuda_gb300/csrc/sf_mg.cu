// sf_mg.cu -- matrix-free geometric multigrid and (flexible) PCG for the 7-point variable-coefficient
// operators of the pressure projection and the magnetic potential, for sm_103a.
//
// Multigrid design (own, from published methods):
//   * cell-centred 2x2x2 aggregation: coarse dims = ceil(n/2), piecewise-constant prolongation P,
//     restriction R = P^T (sum of the 8 children's residuals);
//   * coarse operator = (1/2) P^T A P, which keeps the 7-point face-coefficient form: a coarse face gets half
//     the sum of its 4 fine faces, a coarse cell half the diagonal excess of its 8 children.  The 1/2 is the
//     over-correction that compensates piecewise-constant interpolation of smooth errors (Braess 1995,
//     "Towards algebraic multigrid for elliptic problems of second order"; also used by aggregation AMG with
//     over-correction);
//   * red-black Gauss-Seidel smoothing, red-black before restriction and black-red after, a palindromic
//     red-black sequence on the coarsest grid, so the V-cycle is a fixed symmetric operator and plain PCG
//     applies (Tatebe 1993, "The multigrid preconditioned conjugate gradient method").
// The FP64 form keeps everything in double.  The mixed form runs the V-cycle in FP32 with FP32 level-0 and
// FP16 coarse coefficients inside an FP32 flexible CG, wrapped in FP64 iterative refinement: only the outer
// residual r = b - A x, the update x += d and the dot products stay FP64.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>

#include "sf_rbgs_tma.cuh"
#include "sf_solver.h"

namespace sf {

// ------------------------------------------------------------------------------------------------ buffers
DevBuf::~DevBuf() { release(); }
cudaError_t DevBuf::ensure(size_t bytes) {
    if (bytes <= n_ && p_) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&p_, bytes ? bytes : 256);
    if (e != cudaSuccess) {
        p_ = nullptr;
        n_ = 0;
        return e;
    }
    n_ = bytes;
    return cudaSuccess;
}
void DevBuf::release() {
    if (p_) cudaFree(p_);
    p_ = nullptr;
    n_ = 0;
}

// Grid of the stencil reductions: work items of one 32 (z) x 8 (y) tile and `xpb` consecutive x planes, at most
// max_blocks blocks looping over the items.  Memory-bound kernels take one item per block (kApplyBlocks); the
// FP64-bound residual takes a persistent grid of 8 blocks per SM (kStencilBlocks), which shortens its tail.
// 3-D grid of one block per work item (z-tile, y-tile, x-chunk), for kernels using TILE_BLOCK: at most
// kApplyBlocks blocks (the reduction partials), with x-chunks lengthened when the grid would exceed it.
dim3 tile_grid3(const Dims &d, int &xpb) {
    const long long tiles = (long long)((d.nz + 31) / 32) * ((d.ny + 7) / 8);
    const long long zmax = tiles < kApplyBlocks ? kApplyBlocks / tiles : 1;
    xpb = (int)((d.nx + zmax - 1) / zmax);
    if (xpb < kStencilPlanes) xpb = kStencilPlanes;
    return dim3((d.nz + 31) / 32, (d.ny + 7) / 8, (d.nx + xpb - 1) / xpb);
}

dim3 tile_grid(const Dims &d, int &xpb, int max_blocks) {
    xpb = kStencilPlanes;
    const long long items =
        (long long)((d.nz + 31) / 32) * ((d.ny + 7) / 8) * ((d.nx + kStencilPlanes - 1) / kStencilPlanes);
    return dim3((unsigned)(items < max_blocks ? items : max_blocks), 1, 1);
}

void Tracker::before(cudaStream_t st, bool fine) {
    launches++;
    if (!prof || !fine) return;
    if (used + 2 > ev.size())
        for (int q = 0; q < 64; q++) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            ev.push_back(e);
        }
    cudaEventRecord(ev[used++], st);
}
void Tracker::after(cudaStream_t st, bool fine, double algo_bytes) {
    if (!prof || !fine) return;
    cudaEventRecord(ev[used++], st);
    bytes += algo_bytes;
}
void Tracker::collect(double &ms, int &n, double &b) {
    ms = 0;
    n = 0;
    for (size_t q = 0; q + 1 < used; q += 2) {
        float t = 0;
        cudaEventElapsedTime(&t, ev[q], ev[q + 1]);
        ms += t;
        n++;
    }
    b = bytes;
    bytes = 0;
    used = 0;
}
Tracker::~Tracker() {
    for (auto e : ev) cudaEventDestroy(e);
}

// ------------------------------------------------------------------------------------------------ launch shapes
// Stencil kernels: block (32, 8) over (z, y), grid.z = x.  Red-black kernels cover cell pairs along z.
static inline dim3 blk2() { return dim3(32, 8, 1); }
static inline dim3 grid_cells(const Dims &d) { return dim3((d.nz + 31) / 32, (d.ny + 7) / 8, d.nx); }
constexpr int kRbRows = 1;  // rows per thread of the half sweep (block rows 8 apart); 2 measured slower
static inline dim3 grid_pairs(const Dims &d) {
    return dim3(((d.nz + 1) / 2 + 31) / 32, (d.ny + 8 * kRbRows - 1) / (8 * kRbRows), d.nx);
}

// Programmatic dependent launch.  The kernels of a solver iteration are launched with programmatic stream
// serialisation allowed (launch_pdl) and begin with pdl_entry(): each lets its successor be scheduled once all of
// its own blocks are running (launch_dependents), then waits for its predecessor to complete and its writes to be
// visible (wait) before touching memory.  A successor's blocks thus fill free SM slots during the predecessor's
// last wave instead of after it; a kernel launched without the attribute passes wait at once.
__device__ __forceinline__ void pdl_entry() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}
template <class... KArgs, class... Args>
static void launch_pdl(void (*k)(KArgs...), dim3 g, dim3 b, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = g;
    cfg.blockDim = b;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}

// Row activity: rows[(i * ny + j)] == 0 marks a row (i, j) of the level whose cells are all inactive (D = 0:
// air in the pressure system).  Kernels given flags skip such rows entirely; every vector of the level is zero
// there (cleared when the hierarchy is built, never written afterwards), which is what processing them would
// produce.  nullptr: all rows active.
__device__ __forceinline__ bool row_on(const uint8_t *rows, const Dims &d, int i, int j) {
    return !rows || rows[(long long)i * d.ny + j];
}

// ------------------------------------------------------------------------------------------------ smoothers
template <class C>
__device__ __forceinline__ typename Acc<C>::T inv_diag(const Coef<C> &cf, long long c, typename Acc<C>::T suma) {
    using R = typename Acc<C>::T;
    if (sizeof(C) == 8) return (R)cf.invd[c];
    R D = diag_of(cf, c, suma);
    return D > R(0) ? R(1) / D : R(0);
}

template <class T, class C>
__device__ __forceinline__ T couplings_sum(const Dims &d, const Coef<C> &cf, int i, int j, int k, long long c) {
    using R = typename Acc<C>::T;
    const long long sx = (long long)d.ny * d.nz, sy = d.nz;
    R sa = 0;
    if (i > 0) sa += ldv(cf.ax, c);
    if (i < d.nx - 1) sa += ldv(cf.ax, c + sx);
    if (j > 0) sa += ldv(cf.ay, c);
    if (j < d.ny - 1) sa += ldv(cf.ay, c + sy);
    if (k > 0) sa += ldv(cf.az, c);
    if (k < d.nz - 1) sa += ldv(cf.az, c + 1);
    if (sizeof(C) == 2) sa *= (R)cf.unscale;
    return (T)sa;
}

// Red-black Gauss-Seidel half sweep.  Thread (kp, j, i) owns cells (i, j, 2kp) and (i, j, 2kp+1) of kRbRows rows
// j (8 apart) and updates the one of each pair whose colour (i + j + k) & 1 equals `color`.  Inactive cells
// (D = 0) are written 0.  All rows are loaded before any is stored (more loads in flight per thread); the cells
// written are of one colour and read only the other, so the order does not change the result.
// ZERO: first half sweep of a V-cycle from x = 0; the other cell of each pair is zeroed, so x needs no clearing
// beforehand and never carries stale values into the sweep.
template <class T, class C, bool ZERO>
__global__ void __launch_bounds__(256) k_rbgs(Dims d, Coef<C> cf, T *__restrict__ x, const T *__restrict__ b,
                                              int color, const uint8_t *__restrict__ rows = nullptr) {
    pdl_entry();
    const int kp = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.z;
    const int j0 = blockIdx.y * (8 * kRbRows) + threadIdx.y;
    T res[kRbRows];
    long long cc[kRbRows];
    bool act[kRbRows];
#pragma unroll
    for (int r = 0; r < kRbRows; r++) {
        const int j = j0 + 8 * r;
        const int k = 2 * kp + ((i + j + color) & 1);
        act[r] = j < d.ny && k < d.nz && row_on(rows, d, i, j);
        cc[r] = 0;
        res[r] = T(0);
        if (!act[r]) continue;
        const long long c = cid(d, i, j, k);
        T s, sa;
        if (ZERO) {
            s = T(0);
            sa = (sizeof(C) == 8) ? T(0) : couplings_sum<T, C>(d, cf, i, j, k, c);
        } else {
            s = nbsum<T, C, sizeof(C) != 8>(d, cf, x, i, j, k, c, sa);
        }
        const T inv = (T)inv_diag<C>(cf, c, (typename Acc<C>::T)sa);
        res[r] = (b[c] + s) * inv;
        cc[r] = c;
    }
#pragma unroll
    for (int r = 0; r < kRbRows; r++) {
        const int j = j0 + 8 * r;
        if (ZERO && j < d.ny && row_on(rows, d, i, j)) {
            const int ko = 2 * kp + (((i + j + color) & 1) ^ 1);
            if (ko < d.nz) x[cid(d, i, j, ko)] = T(0);
        }
        if (act[r]) x[cc[r]] = res[r];
    }
}

// z-vectorised half sweep (FP32 vectors, FP32 or FP16 operator; nz a multiple of 4): thread (q, j, i) owns
// cells k0 = 4q .. 4q+3 of row (i, j) and updates the two of them whose colour equals `color`.  x rows are read
// as float4 (the z-neighbours inside the group come from the same vector), FP32 arrays as float4 and FP16 arrays
// as 4 halves in 8 bytes; the group is written back whole, the two other cells with the values just read (no
// other thread writes them during this half sweep).  Same arithmetic, in the same order, as k_rbgs.
__device__ __forceinline__ void ld4(const float *p, float (&v)[4]) {
    const float4 t = *reinterpret_cast<const float4 *>(p);
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
    v[3] = t.w;
}
__device__ __forceinline__ void ld4(const __half *p, float (&v)[4]) {
    const uint2 t = *reinterpret_cast<const uint2 *>(p);
    const __half2 lo = *reinterpret_cast<const __half2 *>(&t.x), hi = *reinterpret_cast<const __half2 *>(&t.y);
    v[0] = __low2float(lo);
    v[1] = __high2float(lo);
    v[2] = __low2float(hi);
    v[3] = __high2float(hi);
}

template <class C, bool ZERO>
__global__ void __launch_bounds__(256) k_rbgs4(Dims d, Coef<C> cf, float *__restrict__ x, const float *__restrict__ b,
                                               int color, const uint8_t *__restrict__ rows = nullptr) {
    pdl_entry();
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    const int k0 = 4 * q;
    if (j >= d.ny || k0 >= d.nz || !row_on(rows, d, i, j)) return;
    const long long c0 = cid(d, i, j, k0);
    const long long sx = (long long)d.ny * d.nz, sy = d.nz;
    const bool xl = i > 0, xu = i < d.nx - 1, yl = j > 0, yu = j < d.ny - 1, zr_in = k0 + 4 < d.nz;
    float xc[4] = {0, 0, 0, 0}, xm[4] = {0, 0, 0, 0}, xp[4] = {0, 0, 0, 0}, ym[4] = {0, 0, 0, 0},
          yp[4] = {0, 0, 0, 0};
    float zl = 0.f, zr = 0.f;
    if (!ZERO) {
        ld4(x + c0, xc);
        if (xl) ld4(x + c0 - sx, xm);
        if (xu) ld4(x + c0 + sx, xp);
        if (yl) ld4(x + c0 - sy, ym);
        if (yu) ld4(x + c0 + sy, yp);
        if (k0 > 0) zl = x[c0 - 1];
        if (zr_in) zr = x[c0 + 4];
    }
    float axl[4], axu[4] = {0, 0, 0, 0}, ayl[4], ayu[4] = {0, 0, 0, 0}, azl[4], dx[4], bv[4];
    ld4(cf.ax + c0, axl);
    if (xu) ld4(cf.ax + c0 + sx, axu);
    ld4(cf.ay + c0, ayl);
    if (yu) ld4(cf.ay + c0 + sy, ayu);
    ld4(cf.az + c0, azl);
    const float azr = zr_in ? ldv(cf.az, c0 + 4) : 0.f;
    ld4(cf.dex + c0, dx);
    ld4(b + c0, bv);
    float out[4] = {xc[0], xc[1], xc[2], xc[3]};  // ZERO: the other colour is cleared
    // cell t of the group (compile-time index: the four values stay in registers)
    auto upd = [&](auto tc) {
        constexpr int t = decltype(tc)::value;
        const int k = k0 + t;
        float s = 0.f, sa = 0.f;
        if (xl) {
            const float a = axl[t];
            if (!ZERO) s += a * xm[t];
            sa += a;
        }
        if (xu) {
            const float a = axu[t];
            if (!ZERO) s += a * xp[t];
            sa += a;
        }
        if (yl) {
            const float a = ayl[t];
            if (!ZERO) s += a * ym[t];
            sa += a;
        }
        if (yu) {
            const float a = ayu[t];
            if (!ZERO) s += a * yp[t];
            sa += a;
        }
        if (k > 0) {
            const float a = azl[t];
            if (!ZERO) s += a * (t == 0 ? zl : xc[t == 0 ? 0 : t - 1]);
            sa += a;
        }
        if (k < d.nz - 1) {
            const float a = t == 3 ? azr : azl[t == 3 ? 3 : t + 1];
            if (!ZERO) s += a * (t == 3 ? zr : xc[t == 3 ? 3 : t + 1]);
            sa += a;
        }
        if (sizeof(C) == 2) {
            if (!ZERO) s *= cf.unscale;
            sa *= cf.unscale;
        }
        float e = dx[t];
        if (sizeof(C) == 2) e *= cf.unscale;
        const float D = sa + e;
        const float inv = D > 0.f ? 1.f / D : 0.f;
        out[t] = (bv[t] + s) * inv;
    };
    // the colour's cells are t = 0, 2 or t = 1, 3; k0 is even, so the choice is uniform across a warp (one j)
    if (((color - i - j) & 1) == 0) {
        upd(std::integral_constant<int, 0>{});
        upd(std::integral_constant<int, 2>{});
    } else {
        upd(std::integral_constant<int, 1>{});
        upd(std::integral_constant<int, 3>{});
    }
    *reinterpret_cast<float4 *>(x + c0) = make_float4(out[0], out[1], out[2], out[3]);
}

// ------------------------------------------------------------------------------------------------ fused sweep
// One full red-black Gauss-Seidel sweep in a single pass, out of place (xin -> xout), colour A then colour B.
// A block owns a TY x TZ tile of (y, z) and marches along x over `xchunk` planes.  Colour-A values are
// computed on the tile plus a one-cell ring in y and z, so the colour-B update needs no other block's
// results: no inter-block dependency, no race, deterministic, and each array crosses HBM once per sweep
// (x in, x out, b, couplings, diagonal) instead of twice.  Arithmetic order equals k_rbgs, so the result is
// bit-identical to the two half sweeps.
//   MODE 0: pre-smoothing from x = 0 (xin unused), A = red
//   MODE 1: pre-smoothing, A = red, B = black
//   MODE 2: post-smoothing, A = black, B = red
constexpr int FTZ = 64, FTY = 8;

__device__ __forceinline__ int mod3(int q) { return ((q % 3) + 3) % 3; }

template <class T, class C, int MODE>
__global__ void __launch_bounds__(256) k_rbgs_fused(Dims d, Coef<C> cf, const T *__restrict__ xin,
                                                    T *__restrict__ xout, const T *__restrict__ b, int xchunk) {
    constexpr int EZ = FTZ + 4, EY = FTY + 4, RZ = FTZ + 2, RY = FTY + 2;
    using R = typename Acc<C>::T;
    __shared__ T sx[3][EY][EZ];  // x_in planes (ring of 3), tile + 2 halo (unused from zero)
    __shared__ T sa[3][RY][RZ];                  // colour-A values after the A update, tile + 1 halo
    const int colA = (MODE == 2) ? 1 : 0;
    const int z0 = blockIdx.x * FTZ, y0 = blockIdx.y * FTY;
    const int x0 = blockIdx.z * xchunk;
    const int x1 = min(x0 + xchunk, d.nx);
    const int tid = threadIdx.x + 32 * threadIdx.y;
    const long long sxs = (long long)d.ny * d.nz, sys = d.nz;

    auto load_x = [&](int q) {
        if constexpr (MODE == 0) return;
        T(*dst)[EZ] = sx[mod3(q)];
        const bool qin = q >= 0 && q < d.nx;
        for (int e = tid; e < EY * EZ; e += 256) {
            const int yy = e / EZ, zz = e - yy * EZ;
            const int y = y0 - 2 + yy, z = z0 - 2 + zz;
            T v = T(0);
            if (qin && y >= 0 && y < d.ny && z >= 0 && z < d.nz) v = xin[cid(d, q, y, z)];
            dst[yy][zz] = v;
        }
    };
    // colour-A update of plane q on the tile + 1 ring; colour-B cells of the ring are not needed
    auto compute_A = [&](int q) {
        T(*dst)[RZ] = sa[mod3(q)];
        const bool qin = q >= 0 && q < d.nx;
        for (int e = tid; e < RY * (RZ / 2); e += 256) {
            const int yy = e / (RZ / 2), pz = e - yy * (RZ / 2);
            const int y = y0 - 1 + yy;
            // zz parity so that (q + y + z) & 1 == colA with z = z0 - 1 + zz
            const int par = (colA - q - y - z0 + 1) & 1;
            const int zz = 2 * pz + par;
            const int z = z0 - 1 + zz;
            T v = T(0);
            if (qin && y >= 0 && y < d.ny && z >= 0 && z < d.nz) {
                const long long c = cid(d, q, y, z);
                R s = 0, sum = 0;
                if constexpr (MODE != 0) {
                    const T(*xm)[EZ] = sx[mod3(q - 1)];
                    const T(*x0p)[EZ] = sx[mod3(q)];
                    const T(*xp)[EZ] = sx[mod3(q + 1)];
                    const int sy_ = yy + 1, sz_ = zz + 1;
                    if (q > 0) {
                        R a = ldv(cf.ax, c);
                        s += a * (R)xm[sy_][sz_];
                        sum += a;
                    }
                    if (q < d.nx - 1) {
                        R a = ldv(cf.ax, c + sxs);
                        s += a * (R)xp[sy_][sz_];
                        sum += a;
                    }
                    if (y > 0) {
                        R a = ldv(cf.ay, c);
                        s += a * (R)x0p[sy_ - 1][sz_];
                        sum += a;
                    }
                    if (y < d.ny - 1) {
                        R a = ldv(cf.ay, c + sys);
                        s += a * (R)x0p[sy_ + 1][sz_];
                        sum += a;
                    }
                    if (z > 0) {
                        R a = ldv(cf.az, c);
                        s += a * (R)x0p[sy_][sz_ - 1];
                        sum += a;
                    }
                    if (z < d.nz - 1) {
                        R a = ldv(cf.az, c + 1);
                        s += a * (R)x0p[sy_][sz_ + 1];
                        sum += a;
                    }
                    if (sizeof(C) == 2) {
                        s *= (R)cf.unscale;
                        sum *= (R)cf.unscale;
                    }
                } else {
                    if (sizeof(C) != 8) sum = (R)couplings_sum<R, C>(d, cf, q, y, z, c);
                }
                const R inv = inv_diag<C>(cf, c, sum);
                v = (T)(((R)b[c] + s) * inv);
            }
            dst[yy][zz] = v;
        }
    };
    // colour-B update of plane p on the tile; writes both colours of plane p to xout
    auto update_B = [&](int p) {
        const int ty = threadIdx.y, y = y0 + ty;
        if (y >= d.ny) return;
        const T(*am)[RZ] = sa[mod3(p - 1)];
        const T(*a0)[RZ] = sa[mod3(p)];
        const T(*ap)[RZ] = sa[mod3(p + 1)];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int tz = 2 * threadIdx.x + h, z = z0 + tz;
            if (z >= d.nz) continue;
            const long long c = cid(d, p, y, z);
            const int ry = ty + 1, rz = tz + 1;
            if (((p + y + z) & 1) == colA) {
                xout[c] = a0[ry][rz];
                continue;
            }
            R s = 0, sum = 0;
            if (p > 0) {
                R a = ldv(cf.ax, c);
                s += a * (R)am[ry][rz];
                sum += a;
            }
            if (p < d.nx - 1) {
                R a = ldv(cf.ax, c + sxs);
                s += a * (R)ap[ry][rz];
                sum += a;
            }
            if (y > 0) {
                R a = ldv(cf.ay, c);
                s += a * (R)a0[ry - 1][rz];
                sum += a;
            }
            if (y < d.ny - 1) {
                R a = ldv(cf.ay, c + sys);
                s += a * (R)a0[ry + 1][rz];
                sum += a;
            }
            if (z > 0) {
                R a = ldv(cf.az, c);
                s += a * (R)a0[ry][rz - 1];
                sum += a;
            }
            if (z < d.nz - 1) {
                R a = ldv(cf.az, c + 1);
                s += a * (R)a0[ry][rz + 1];
                sum += a;
            }
            if (sizeof(C) == 2) {
                s *= (R)cf.unscale;
                sum *= (R)cf.unscale;
            }
            const R inv = inv_diag<C>(cf, c, sum);
            xout[c] = (T)(((R)b[c] + s) * inv);
        }
    };

    // pipeline: plane q needs x_in planes q-1..q+1 for its colour-A update; plane q-1's colour-B update needs
    // colour-A planes q-2..q.  Barriers separate every reuse of a ring slot from its last reader.
    load_x(x0 - 2);
    load_x(x0 - 1);
    load_x(x0);
    __syncthreads();
    compute_A(x0 - 1);  // reads x_in x0-2 .. x0
    __syncthreads();
    load_x(x0 + 1);     // overwrites the slot of x0-2
    __syncthreads();
    compute_A(x0);
    for (int q = x0 + 1; q <= x1; q++) {
        __syncthreads();  // compute_A(q-1) and update_B(q-2) are complete
        load_x(q + 1);    // slot of plane q-2, last read by compute_A(q-1)
        __syncthreads();
        compute_A(q);     // slot of colour-A plane q-3, last read by update_B(q-2)
        __syncthreads();
        update_B(q - 1);
    }
}

// ------------------------------------------------------------------------------------------------ pipelined sweep
// Finest-level variant of the one-pass red-black sweep with every global load issued asynchronously two planes
// ahead (cp.async, zero-fill outside the grid) into a ring of four planes of x and of the five operator arrays
// over the tile plus a two-cell halo.  Compute phases read shared memory only, so the march along x is not
// exposed to global-memory latency.  Same arithmetic order as k_rbgs: bit-identical results.
// T = C = double (1/D stored) or float (D = sum of couplings + dex).
constexpr int PEZ = FTZ + 4, PEY = FTY + 4, PRING = 4;

__device__ __forceinline__ void cp_async_elem(void *dst, const void *src, bool valid, int bytes) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    if (bytes == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(s), "l"(src), "r"(valid ? 8 : 0) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(s), "l"(src), "r"(valid ? 4 : 0) : "memory");
}

template <class T>
constexpr size_t pipe_smem_bytes() {
    return sizeof(T) * (size_t)(6 * PRING * PEY * PEZ + 3 * (FTY + 2) * (FTZ + 2));
}

template <class T, int MODE>
__global__ void __launch_bounds__(256) k_rbgs_pipe(Dims d, Coef<T> cf, const T *__restrict__ xin, T *__restrict__ xout,
                                                   const T *__restrict__ b, int xchunk) {
    static_assert(sizeof(T) == 4 || sizeof(T) == 8, "FP32 or FP64 finest level");
    constexpr int RZ = FTZ + 2, RY = FTY + 2, PL = PEY * PEZ;
    extern __shared__ __align__(16) uint8_t psm[];
    T *ring = reinterpret_cast<T *>(psm);  // [array 0..5][slot][PEY][PEZ]: x, ax, ay, az, dg, b
    T(*sa)[RY][RZ] = reinterpret_cast<T(*)[RY][RZ]>(ring + 6 * PRING * PL);
    const T *dg = sizeof(T) == 8 ? reinterpret_cast<const T *>(cf.invd) : reinterpret_cast<const T *>(cf.dex);
    const int colA = (MODE == 2) ? 1 : 0;
    const int z0 = blockIdx.x * FTZ, y0 = blockIdx.y * FTY;
    const int x0 = blockIdx.z * xchunk;
    const int x1 = min(x0 + xchunk, d.nx);
    const int tid = threadIdx.x + 32 * threadIdx.y;
    auto slot = [](int q) { return ((q % PRING) + PRING) % PRING; };
    auto E = [&](int arr, int q, int yy, int zz) -> T & { return ring[(arr * PRING + slot(q)) * PL + yy * PEZ + zz]; };

    auto issue = [&](int q) {
        const bool qin = q >= 0 && q < d.nx;
        for (int e = tid; e < PL; e += 256) {
            const int yy = e / PEZ, zz = e - yy * PEZ;
            const int y = y0 - 2 + yy, z = z0 - 2 + zz;
            const bool v = qin && y >= 0 && y < d.ny && z >= 0 && z < d.nz;
            const long long c = v ? cid(d, q, y, z) : 0;
            if (MODE != 0) cp_async_elem(&E(0, q, yy, zz), xin + c, v, sizeof(T));
            cp_async_elem(&E(1, q, yy, zz), cf.ax + c, v, sizeof(T));
            cp_async_elem(&E(2, q, yy, zz), cf.ay + c, v, sizeof(T));
            cp_async_elem(&E(3, q, yy, zz), cf.az + c, v, sizeof(T));
            cp_async_elem(&E(4, q, yy, zz), dg + c, v, sizeof(T));
            cp_async_elem(&E(5, q, yy, zz), b + c, v, sizeof(T));
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    auto wait1 = []() { asm volatile("cp.async.wait_group 1;" ::: "memory"); };

    // one cell update from the staged planes: neighbours `xv(dx, dy, dz)`, couplings at E-index (ey, ez)
    auto update = [&](int q, int y, int z, int ey, int ez, auto xv) -> T {
        T s = 0, sum = 0;
        if (MODE != 0 || true) {
            if (q > 0) {
                const T a = E(1, q, ey, ez);
                s += a * xv(-1, 0, 0);
                sum += a;
            }
            if (q < d.nx - 1) {
                const T a = E(1, q + 1, ey, ez);
                s += a * xv(1, 0, 0);
                sum += a;
            }
            if (y > 0) {
                const T a = E(2, q, ey, ez);
                s += a * xv(0, -1, 0);
                sum += a;
            }
            if (y < d.ny - 1) {
                const T a = E(2, q, ey + 1, ez);
                s += a * xv(0, 1, 0);
                sum += a;
            }
            if (z > 0) {
                const T a = E(3, q, ey, ez);
                s += a * xv(0, 0, -1);
                sum += a;
            }
            if (z < d.nz - 1) {
                const T a = E(3, q, ey, ez + 1);
                s += a * xv(0, 0, 1);
                sum += a;
            }
        }
        T inv;
        if (sizeof(T) == 8) {
            inv = E(4, q, ey, ez);
        } else {
            const T D = sum + E(4, q, ey, ez);
            inv = D > T(0) ? T(1) / D : T(0);
        }
        return (E(5, q, ey, ez) + s) * inv;
    };

    auto compute_A = [&](int q) {
        T(*dst)[RZ] = sa[mod3(q)];
        const bool qin = q >= 0 && q < d.nx;
        for (int e = tid; e < RY * (RZ / 2); e += 256) {
            const int yy = e / (RZ / 2), pz = e - yy * (RZ / 2);
            const int y = y0 - 1 + yy;
            const int zz = 2 * pz + ((colA - q - y - z0 + 1) & 1);
            const int z = z0 - 1 + zz;
            T v = T(0);
            if (qin && y >= 0 && y < d.ny && z >= 0 && z < d.nz) {
                const int ey = yy + 1, ez = zz + 1;
                if (MODE == 0) {
                    T sum = 0;
                    if (sizeof(T) != 8) {
                        if (q > 0) sum += E(1, q, ey, ez);
                        if (q < d.nx - 1) sum += E(1, q + 1, ey, ez);
                        if (y > 0) sum += E(2, q, ey, ez);
                        if (y < d.ny - 1) sum += E(2, q, ey + 1, ez);
                        if (z > 0) sum += E(3, q, ey, ez);
                        if (z < d.nz - 1) sum += E(3, q, ey, ez + 1);
                    }
                    T inv;
                    if (sizeof(T) == 8) {
                        inv = E(4, q, ey, ez);
                    } else {
                        const T D = sum + E(4, q, ey, ez);
                        inv = D > T(0) ? T(1) / D : T(0);
                    }
                    v = (E(5, q, ey, ez) + T(0)) * inv;
                } else {
                    v = update(q, y, z, ey, ez, [&](int dx, int dy, int dz) -> T {
                        return E(0, q + dx, ey + dy, ez + dz);
                    });
                }
            }
            dst[yy][zz] = v;
        }
    };
    auto update_B = [&](int p) {
        const int ty = threadIdx.y, y = y0 + ty;
        if (y >= d.ny) return;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int tz = 2 * threadIdx.x + h, z = z0 + tz;
            if (z >= d.nz) continue;
            const long long c = cid(d, p, y, z);
            const int ry = ty + 1, rz = tz + 1;
            if (((p + y + z) & 1) == colA) {
                xout[c] = sa[mod3(p)][ry][rz];
                continue;
            }
            xout[c] = update(p, y, z, ty + 2, tz + 2, [&](int dx, int dy, int dz) -> T {
                return sa[mod3(p + dx)][ry + dy][rz + dz];
            });
        }
    };

    issue(x0 - 2);
    issue(x0 - 1);
    issue(x0);
    issue(x0 + 1);
    wait1();  // planes x0-2 .. x0 staged
    __syncthreads();
    compute_A(x0 - 1);
    __syncthreads();
    issue(x0 + 2);  // slot of x0-2, last read by compute_A(x0-1)
    wait1();        // x0+1 staged
    __syncthreads();
    compute_A(x0);
    for (int q = x0 + 1; q <= x1; q++) {
        __syncthreads();  // compute_A(q-1) and update_B(q-2) are complete
        issue(q + 2);     // slot of plane q-2
        wait1();          // plane q+1 staged
        __syncthreads();
        compute_A(q);
        __syncthreads();
        update_B(q - 1);
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// r = b - A x on the fine level, summed over each coarse cell's (up to) 8 children -> coarse rhs.
template <class T, class C>
__global__ void __launch_bounds__(256) k_resid_restrict(Dims d, Coef<C> cf, const T *__restrict__ x,
                                                        const T *__restrict__ b, Dims dc, T *__restrict__ bc,
                                                        const uint8_t *__restrict__ rows = nullptr,
                                                        const uint8_t *__restrict__ rows_c = nullptr) {
    pdl_entry();
    const int K = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int I = blockIdx.z;
    if (K >= dc.nz || J >= dc.ny || !row_on(rows_c, dc, I, J)) return;
    T acc = 0;
#pragma unroll
    for (int di = 0; di < 2; di++) {
        const int i = 2 * I + di;
        if (i >= d.nx) break;
#pragma unroll
        for (int dj = 0; dj < 2; dj++) {
            const int j = 2 * J + dj;
            if (j >= d.ny) break;
            if (!row_on(rows, d, i, j)) continue;  // residual zero
#pragma unroll
            for (int dk = 0; dk < 2; dk++) {
                const int k = 2 * K + dk;
                if (k >= d.nz) break;
                const long long c = cid(d, i, j, k);
                T sa;
                T s = nbsum<T, C, sizeof(C) != 8>(d, cf, x, i, j, k, c, sa);
                T D = (T)diag_of<C>(cf, c, (typename Acc<C>::T)sa);
                acc += (b[c] - D * x[c]) + s;
            }
        }
    }
    bc[cid(dc, I, J, K)] = acc;
}

// x += P xc (piecewise constant).
template <class T>
__global__ void __launch_bounds__(256) k_prolong(Dims d, T *__restrict__ x, Dims dc, const T *__restrict__ xc,
                                                 const uint8_t *__restrict__ rows = nullptr) {
    pdl_entry();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= d.nz || j >= d.ny || !row_on(rows, d, i, j)) return;
    x[cid(d, i, j, k)] += xc[cid(dc, i >> 1, j >> 1, k >> 1)];
}

// Coarsest level: one block, x = 0 then the palindromic sequence red, (black, red) x pairs.  Grids of at most
// kCoarseMax cells first make b consistent on a pure-Neumann level (coarse_consistent).
// Grids of at most kCoarseMax cells keep x in shared memory and each thread's couplings, inverse diagonal and
// right-hand side in registers, so the sweeps touch no global memory; larger grids sweep in global memory.
constexpr int kCoarseMax = 1024, kCoarseThreads = 1024;

// A coarsest level without any diagonal excess (a pure-Neumann system: the operator annihilates the constant) is
// solvable only for a right-hand side of zero sum over its active cells.  The restricted right-hand side misses
// that by rounding, and Gauss-Seidel sweeps then drift along the constant, the further the more sweeps run (which
// degrades the preconditioner).  coarse_consistent subtracts the mean of b over the active cells (D > 0) on such
// a level and returns b unchanged on any other.  Every thread of the block calls it, one cell each; the sums run
// in a fixed order (warp shuffles, then the warps in order), so equal inputs give equal bits.
template <class R>
__device__ __forceinline__ R coarse_consistent(R bc, bool active, bool excess) {
    __shared__ R s_sum[32];
    __shared__ int s_cnt[32];
    if (__syncthreads_or(excess ? 1 : 0)) return bc;
    R s = active ? bc : R(0);
    int m = active ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        m += __shfl_down_sync(0xffffffffu, m, o);
    }
    if ((threadIdx.x & 31) == 0) {
        s_sum[threadIdx.x >> 5] = s;
        s_cnt[threadIdx.x >> 5] = m;
    }
    __syncthreads();
    R tot = 0;
    int cnt = 0;
    for (int w = 0; w < (int)((blockDim.x + 31) >> 5); w++) {
        tot += s_sum[w];
        cnt += s_cnt[w];
    }
    return active && cnt > 0 ? bc - tot / R(cnt) : bc;
}

template <class T, class C>
__global__ void __launch_bounds__(kCoarseThreads) k_coarse_smem(Dims d, Coef<C> cf, T *__restrict__ x,
                                                                const T *__restrict__ b, int pairs) {
    pdl_entry();
    using R = typename Acc<C>::T;
    __shared__ T xs[kCoarseMax];
    const int sx = d.ny * d.nz, sy = d.nz;
    const int c = threadIdx.x;
    R a[6], inv = 0, bc = 0;
    int has = 0, col = -1;
    if (c < d.n) {
        const int k = c % d.nz, j = (c / d.nz) % d.ny, i = c / (d.nz * d.ny);
        col = (i + j + k) & 1;
        // neighbour order and guards of nbsum: -x, +x, -y, +y, -z, +z
        has = (i > 0) | ((i < d.nx - 1) << 1) | ((j > 0) << 2) | ((j < d.ny - 1) << 3) | ((k > 0) << 4) |
              ((k < d.nz - 1) << 5);
        R sum = 0;
#pragma unroll
        for (int f = 0; f < 6; f++) {
            const C *arr = f < 2 ? cf.ax : (f < 4 ? cf.ay : cf.az);
            const int st = f < 2 ? sx : (f < 4 ? sy : 1);
            R av = 0;
            if (has & (1 << f)) {
                av = (R)ldv(arr, (f & 1) ? c + st : c);  // lower faces stored at c, upper at the neighbour
                if (sizeof(C) == 2) av *= (R)cf.unscale;
                sum += av;
            }
            a[f] = av;
        }
        inv = inv_diag<C>(cf, c, sum);
        bc = (R)b[c];
        xs[c] = T(0);
    }
    bc = coarse_consistent<R>(bc, c < d.n && inv > R(0), c < d.n && ldv(cf.dex, c) != R(0));
    __syncthreads();
    const int nh = 1 + 2 * pairs;
    for (int h = 0; h < nh; h++) {
        if (col == (h & 1)) {
            R s = 0;
#pragma unroll
            for (int f = 0; f < 6; f++) {
                const int st = f < 2 ? sx : (f < 4 ? sy : 1);
                if (has & (1 << f)) s += a[f] * (R)xs[(f & 1) ? c + st : c - st];
            }
            xs[c] = (T)((bc + s) * inv);
        }
        __syncthreads();
    }
    if (c < d.n) x[c] = xs[c];
}

template <class T, class C>
__global__ void __launch_bounds__(1024) k_coarse(Dims d, Coef<C> cf, T *__restrict__ x, const T *__restrict__ b,
                                                 int pairs) {
    pdl_entry();
    for (long long c = threadIdx.x; c < d.n; c += blockDim.x) x[c] = T(0);
    __syncthreads();
    const int nh = 1 + 2 * pairs;
    for (int h = 0; h < nh; h++) {
        const int color = h & 1;
        for (long long c = threadIdx.x; c < d.n; c += blockDim.x) {
            const int k = (int)(c % d.nz), j = (int)((c / d.nz) % d.ny), i = (int)(c / ((long long)d.nz * d.ny));
            if (((i + j + k) & 1) != color) continue;
            T sa;
            T s = nbsum<T, C, sizeof(C) != 8>(d, cf, x, i, j, k, c, sa);
            const T inv = (T)inv_diag<C>(cf, c, (typename Acc<C>::T)sa);
            x[c] = (b[c] + s) * inv;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------------------ coarsening
template <class C>
__device__ __forceinline__ double ldu(const Coef<C> &cf, const C *p, long long i) {
    double v = (double)ldv(p, i);
    if (sizeof(C) == 2) v *= (double)cf.unscale;
    return v;
}

// Coarse operator (1/2) P^T A P in face-coefficient form.
template <class CF, class CC>
__global__ void __launch_bounds__(256) k_coarsen(Dims d, Coef<CF> f, Dims dc, Coef<CC> cc) {
    const int K = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int I = blockIdx.z;
    if (K >= dc.nz || J >= dc.ny) return;
    // half the sum of the fine faces on the coarse face at coarse index (Ic, Jc, Kc) along `axis`
    auto face = [&](int axis, int Ic, int Jc, int Kc) -> double {
        int C3[3] = {Ic, Jc, Kc};
        int dn[3] = {dc.nx, dc.ny, dc.nz};
        if (C3[axis] <= 0 || C3[axis] >= dn[axis]) return 0.0;
        const CF *arr = axis == 0 ? f.ax : (axis == 1 ? f.ay : f.az);
        double s = 0;
        for (int u = 0; u < 2; u++)
            for (int v = 0; v < 2; v++) {
                int fi[3];
                fi[axis] = 2 * C3[axis];
                int o1 = (axis + 1) % 3, o2 = (axis + 2) % 3;
                fi[o1] = 2 * C3[o1] + u;
                fi[o2] = 2 * C3[o2] + v;
                if (fi[0] >= d.nx || fi[1] >= d.ny || fi[2] >= d.nz) continue;
                s += ldu(f, arr, cid(d, fi[0], fi[1], fi[2]));
            }
        return 0.5 * s;
    };
    double dex = 0;
    for (int di = 0; di < 2; di++)
        for (int dj = 0; dj < 2; dj++)
            for (int dk = 0; dk < 2; dk++) {
                int i = 2 * I + di, j = 2 * J + dj, k = 2 * K + dk;
                if (i >= d.nx || j >= d.ny || k >= d.nz) continue;
                dex += ldu(f, f.dex, cid(d, i, j, k));
            }
    dex *= 0.5;
    const long long c = cid(dc, I, J, K);
    const double fx = face(0, I, J, K), fy = face(1, I, J, K), fz = face(2, I, J, K);
    if (sizeof(CC) == 8) {
        const double D = fx + face(0, I + 1, J, K) + fy + face(1, I, J + 1, K) + fz + face(2, I, J, K + 1) + dex;
        stv(cc.ax, c, fx);
        stv(cc.ay, c, fy);
        stv(cc.az, c, fz);
        stv(cc.dex, c, dex);
        cc.D[c] = D;
        cc.invd[c] = D > 0 ? 1.0 / D : 0.0;
    } else {
        const double sc = sizeof(CC) == 2 ? (double)cc.scale : 1.0;
        stv(cc.ax, c, (float)(fx * sc));
        stv(cc.ay, c, (float)(fy * sc));
        stv(cc.az, c, (float)(fz * sc));
        stv(cc.dex, c, (float)(dex * sc));
    }
}

// FP64 level 0 -> FP32 copy (mixed form).
__global__ void k_to32(long long n, Coef<double> f, Coef<float> o) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        o.ax[c] = f64_to_f32(f.ax[c]);
        o.ay[c] = f64_to_f32(f.ay[c]);
        o.az[c] = f64_to_f32(f.az[c]);
        o.dex[c] = f64_to_f32(f.dex[c]);
    }
}

// FP64 level 0 -> FP16 copy read only by the finest-level smoother (smoother 2); scale 1 (ghost-fluid excesses
// stay below 6000, couplings in [0, 1 + chi]).
__global__ void k_to16(long long n, Coef<double> f, Coef<__half> o) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        o.ax[c] = __float2half_rn(f64_to_f32(f.ax[c]));
        o.ay[c] = __float2half_rn(f64_to_f32(f.ay[c]));
        o.az[c] = __float2half_rn(f64_to_f32(f.az[c]));
        o.dex[c] = __float2half_rn(f64_to_f32(f.dex[c]));
    }
}

// ------------------------------------------------------------------------------------------------ Krylov kernels
// Stencil kernels with a reduction: block (32, 8) looping over work items (tile_grid).  Item w = (z-tile
// fastest, y-tile, x-chunk of `xpb` planes); consecutive blocks take neighbouring tiles of the same planes.
// Threads outside the grid skip their cells but stay in the loop, so that every thread reaches the reduction.
#define TILE_LOOP(d, xpb)                                                                          \
    const unsigned tz_n = ((d).nz + 31) / 32, ty_n = ((d).ny + 7) / 8;                             \
    const unsigned items = tz_n * ty_n * (((d).nx + (xpb)-1) / (xpb));                             \
    for (unsigned w = blockIdx.x; w < items; w += gridDim.x) {                                     \
        const unsigned tzi = w % tz_n, rest = w / tz_n, tyi = rest % ty_n, chunk = rest / ty_n;   \
        const int k = (int)tzi * 32 + threadIdx.x, j = (int)tyi * 8 + threadIdx.y;                  \
        if (k >= (d).nz || j >= (d).ny) continue;                                                  \
        const int i_end = min((d).nx, (int)(chunk + 1) * (xpb));                                   \
        for (int i = (int)chunk * (xpb); i < i_end; i++) {                                         \
            const long long c = cid((d), i, j, k);

// One work item per block of a 3-D grid (tile_grid3): block (z-tile, y-tile), `xpb` planes from blockIdx.z.
#define TILE_BLOCK(d, xpb)                                                                    \
    {                                                                                         \
        const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;       \
        const bool inb = k < (d).nz && j < (d).ny;                                            \
        const int i_end = min((d).nx, (int)(blockIdx.z + 1) * (xpb));                         \
        for (int i = blockIdx.z * (xpb); i < i_end; i++) {                                    \
            if (!inb) continue;                                                               \
            const long long c = cid((d), i, j, k);

#define TILE_LOOP_END \
    }                 \
    }

// q = A p ; slot PQ = (p, q) ; alpha = rho / pq (0 and breakdown flag if pq <= 0)
// Per-thread partial sums are accumulated in the vector type (FP32 for FP32 vectors: FP64 arithmetic and
// conversions are scarce on GB300); FP32 partials are summed across a warp as a float pair (warp_sum_df) and in
// FP64 from there on.
template <class T, class C>
__global__ void __launch_bounds__(256) k_apply_dot(Dims d, int xpb, Coef<C> cf, const T *__restrict__ p,
                                                   T *__restrict__ q, double *sc, double *part, unsigned *ticket,
                                                   const uint8_t *__restrict__ rows) {
    pdl_entry();
    T acc = 0;
    TILE_BLOCK(d, xpb)
    if (!row_on(rows, d, i, j)) continue;  // q stays zero there
    T sa;
    T s = nbsum<T, C, sizeof(C) != 8>(d, cf, p, i, j, k, c, sa);
    T D = (T)diag_of<C>(cf, c, (typename Acc<C>::T)sa);
    T pc = p[c];
    T qc = D * pc - s;
    q[c] = qc;
    acc += pc * qc;
    TILE_LOOP_END
    T v[1] = {acc};
    double tot[1];
    if (grid_reduce<1>(v, part, ticket, tot)) {
        sc[S_PQ] = tot[0];
        if (tot[0] > 0 && isfinite(tot[0])) {
            sc[S_ALPHA] = sc[S_RHO] / tot[0];
        } else {
            sc[S_ALPHA] = 0;
            sc[S_AUX0] = 1;  // breakdown
        }
    }
}

// FP32 q = A p with (p, q), z-vectorised (nz a multiple of 4): thread (q4, j) of a 3-D grid block owns cells
// k0 = 4 q4 .. 4 q4 + 3 of row j over `xpb` x planes; float4 loads of p and of the operator arrays, the z-neighbours
// inside the group from the same vector.  Each cell's q is computed as in k_apply_dot.
__global__ void __launch_bounds__(256) k_apply_dot4(Dims d, int xpb, Coef<float> cf, const float *__restrict__ p,
                                                    float *__restrict__ q, double *sc, double *part,
                                                    unsigned *ticket) {
    pdl_entry();
    float acc = 0.f;
    const int k0 = 4 * (blockIdx.x * 32 + threadIdx.x), j = blockIdx.y * 8 + threadIdx.y;
    if (k0 < d.nz && j < d.ny) {
        const long long sx = (long long)d.ny * d.nz, sy = d.nz;
        const bool yl = j > 0, yu = j < d.ny - 1, zl = k0 > 0, zu = k0 + 4 < d.nz;
        const int i_end = min(d.nx, (int)(blockIdx.z + 1) * xpb);
        for (int i = blockIdx.z * xpb; i < i_end; i++) {
            const long long c0 = cid(d, i, j, k0);
            const bool xl = i > 0, xu = i < d.nx - 1;
            float pc[4], pxm[4] = {0, 0, 0, 0}, pxp[4] = {0, 0, 0, 0}, pym[4] = {0, 0, 0, 0}, pyp[4] = {0, 0, 0, 0};
            float axl[4], axu[4] = {0, 0, 0, 0}, ayl[4], ayu[4] = {0, 0, 0, 0}, azl[4], dx[4];
            ld4(p + c0, pc);
            if (xl) ld4(p + c0 - sx, pxm);
            if (xu) ld4(p + c0 + sx, pxp);
            if (yl) ld4(p + c0 - sy, pym);
            if (yu) ld4(p + c0 + sy, pyp);
            const float pzl = zl ? p[c0 - 1] : 0.f, pzr = zu ? p[c0 + 4] : 0.f;
            ld4(cf.ax + c0, axl);
            if (xu) ld4(cf.ax + c0 + sx, axu);
            ld4(cf.ay + c0, ayl);
            if (yu) ld4(cf.ay + c0 + sy, ayu);
            ld4(cf.az + c0, azl);
            const float azr = zu ? cf.az[c0 + 4] : 0.f;
            ld4(cf.dex + c0, dx);
            float out[4];
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const int k = k0 + t;
                float s = 0.f, sa = 0.f;
                if (xl) {
                    s += axl[t] * pxm[t];
                    sa += axl[t];
                }
                if (xu) {
                    s += axu[t] * pxp[t];
                    sa += axu[t];
                }
                if (yl) {
                    s += ayl[t] * pym[t];
                    sa += ayl[t];
                }
                if (yu) {
                    s += ayu[t] * pyp[t];
                    sa += ayu[t];
                }
                if (k > 0) {
                    const float a = azl[t];
                    s += a * (t == 0 ? pzl : pc[t == 0 ? 0 : t - 1]);
                    sa += a;
                }
                if (k < d.nz - 1) {
                    const float a = t == 3 ? azr : azl[t == 3 ? 3 : t + 1];
                    s += a * (t == 3 ? pzr : pc[t == 3 ? 3 : t + 1]);
                    sa += a;
                }
                const float D = sa + dx[t];
                out[t] = D * pc[t] - s;
                acc += pc[t] * out[t];
            }
            *reinterpret_cast<float4 *>(q + c0) = make_float4(out[0], out[1], out[2], out[3]);
        }
    }
    float v[1] = {acc};
    double tot[1];
    if (grid_reduce<1>(v, part, ticket, tot)) {
        sc[S_PQ] = tot[0];
        if (tot[0] > 0 && isfinite(tot[0])) {
            sc[S_ALPHA] = sc[S_RHO] / tot[0];
        } else {
            sc[S_ALPHA] = 0;
            sc[S_AUX0] = 1;  // breakdown
        }
    }
}

// Launch q = A p, (p, q) on the FP32 level-0 operator: z-vectorised when rows are 16-byte aligned.
static void apply_dot32(cudaStream_t st, const Dims &d, const Coef<float> &cf, const float *p, float *q, double *sc,
                        double *part, unsigned *ticket) {
    int xpb;
    if (d.nz % 4 == 0) {
        const long long tiles = (long long)((d.nz + 127) / 128) * ((d.ny + 7) / 8);
        const long long zmax = tiles < kApplyBlocks ? kApplyBlocks / tiles : 1;
        xpb = (int)((d.nx + zmax - 1) / zmax);
        if (xpb < 2) xpb = 2;
        const dim3 g((d.nz + 127) / 128, (d.ny + 7) / 8, (d.nx + xpb - 1) / xpb);
        launch_pdl(k_apply_dot4, g, dim3(32, 8), st, d, xpb, cf, p, q, sc, part, ticket);
        return;
    }
    const dim3 tg = tile_grid3(d, xpb);
    launch_pdl(k_apply_dot<float, float>, tg, dim3(32, 8), st, d, xpb, cf, p, q, sc, part, ticket,
               (const uint8_t *)nullptr);
}

#include "sf_split.cuh"
#include "sf_tail.cuh"

// Vector kernels of the natural layout walk rows (i, j) of nz cells, one warp per row and 8 rows per block;
// rows whose flag is 0 (no active cell; rows == nullptr: every row active) are skipped, their entries being
// zero in every vector.
#define VEC_ROWS(d, rows)                                                                                     \
    for (long long row_ = blockIdx.x * 8LL + threadIdx.y, nrows_ = (long long)(d).nx * (d).ny; row_ < nrows_; \
         row_ += (long long)gridDim.x * 8) {                                                                  \
        if ((rows) && !(rows)[row_]) continue;                                                                \
        for (int k_ = threadIdx.x; k_ < (d).nz; k_ += 32) {                                                   \
            const long long c = row_ * (d).nz + k_;
#define VEC_ROWS_END \
    }                \
    }

// rho_new = (r, z), zq = (z, q); beta = flexible ? -alpha*zq/rho : rho_new/rho; rho = rho_new
template <class T>
__global__ void __launch_bounds__(256) k_dot_rz(Dims d, const uint8_t *__restrict__ rows, const T *__restrict__ r,
                                                const T *__restrict__ z, const T *__restrict__ q, int flexible,
                                                double *sc, double *part, unsigned *ticket) {
    pdl_entry();
    T a0 = 0, a1 = 0;
    VEC_ROWS(d, rows)
    const T zc = z[c];
    a0 += r[c] * zc;
    a1 += zc * q[c];
    VEC_ROWS_END
    T v[2] = {a0, a1};
    double tot[2];
    if (grid_reduce<2>(v, part, ticket, tot)) {
        const double rho = sc[S_RHO];
        double beta = flexible ? (-sc[S_ALPHA] * tot[1] / rho) : (tot[0] / rho);
        if (!isfinite(beta)) beta = 0;
        sc[S_RHONEW] = tot[0];
        sc[S_ZQ] = tot[1];
        sc[S_BETA] = beta;
        sc[S_RHO] = tot[0];
    }
}

template <class T>
__global__ void __launch_bounds__(256) k_xpby(Dims d, const uint8_t *__restrict__ rows, const T *__restrict__ z,
                                              T *__restrict__ p, const double *sc) {
    pdl_entry();
    const T beta = (T)sc[S_BETA];
    VEC_ROWS(d, rows)
    p[c] = z[c] + beta * p[c];
    VEC_ROWS_END
}

// x += alpha p ; r -= alpha q ; slot RR = (r, r)
template <class T>
__global__ void __launch_bounds__(256) k_update(Dims d, const uint8_t *__restrict__ rows, T *__restrict__ x,
                                                T *__restrict__ r, const T *__restrict__ p, const T *__restrict__ q,
                                                double *sc, double *part, unsigned *ticket) {
    pdl_entry();
    const T alpha = (T)sc[S_ALPHA];
    T acc = 0;
    VEC_ROWS(d, rows)
    x[c] += alpha * p[c];
    T rc = r[c] - alpha * q[c];
    r[c] = rc;
    acc += rc * rc;
    VEC_ROWS_END
    T v[1] = {acc};
    double tot[1];
    if (grid_reduce<1>(v, part, ticket, tot)) sc[S_RR] = tot[0];
}

// r = b - A x (FP64 operator), written as TR (double, or float for the refinement's inner rhs, in the split
// layout when `split`); slots: rr_slot = (r, r) in FP64, bb_slot = (b, b).  skip0: leave row 0 out of both sums.
template <class TR>
__global__ void __launch_bounds__(256) k_residual64(Dims d, int xpb, Coef<double> cf, const double *__restrict__ x,
                                                    const double *__restrict__ b, TR *__restrict__ r, int skip0,
                                                    int rr_slot, int bb_slot, double *sc, double *part,
                                                    unsigned *ticket, int split = 0,
                                                    const uint8_t *__restrict__ rows = nullptr) {
    double v[2] = {0, 0};
    TILE_LOOP(d, xpb)
    if (!row_on(rows, d, i, j)) {  // residual zero
        if (r) r[split ? split_index(d, i, j, k) : c] = (TR)0;
        continue;
    }
    double sa;
    double s = nbsum<double, double, false>(d, cf, x, i, j, k, c, sa);
    const double bc = b[c];
    double rc = (bc - cf.D[c] * x[c]) + s;
    if (r) r[split ? split_index(d, i, j, k) : c] = (TR)rc;
    if (!(skip0 && c == 0)) {
        v[0] += rc * rc;
        if (bb_slot >= 0) v[1] += bc * bc;
    }
    TILE_LOOP_END
    double tot[2];
    if (grid_reduce<2>(v, part, ticket, tot)) {
        sc[rr_slot] = tot[0];
        if (bb_slot >= 0) sc[bb_slot] = tot[1];
    }
}

// r = b for x = 0 (the first refinement step): cast to the inner precision; slots rr = bb = (b, b).
template <class TR>
__global__ void __launch_bounds__(256) k_cast_rhs(long long n, const double *__restrict__ b, TR *__restrict__ r,
                                                  int rr_slot, int bb_slot, double *sc, double *part,
                                                  unsigned *ticket) {
    double v[1] = {0};
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    for (long long c = blockIdx.x * 256LL + tid; c < n; c += (long long)gridDim.x * 256) {
        const double bc = b[c];
        r[c] = to_prec<TR>(bc);
        v[0] += bc * bc;
    }
    double tot[1];
    if (grid_reduce<1>(v, part, ticket, tot)) {
        sc[rr_slot] = tot[0];
        sc[bb_slot] = tot[0];
    }
}

// Self-test of the bounded waits: one CTA arms an mbarrier for bytes that no copy will deliver (nothing is in
// flight), waits for it with the same bounded wait as the TMA kernels, and records the outcome: out[0] = 1 when the
// wait gave up, 0 if it completed; out[1] = the nanoseconds waited.
__global__ void k_selftest_bounded_wait(unsigned long long limit_ns, unsigned long long *out) {
    __shared__ __align__(8) uint64_t bar;
    const uint32_t b = tc::smem_u32(&bar);
    if (threadIdx.x == 0) {
        tc::mbar_init(b, 1);
        tc::mbar_fence_init();
        tc::mbar_expect_tx(b, 16);  // 16 bytes that never arrive
        const uint64_t t0 = tc::global_ns();
        const bool done = tc::mbar_wait_ns(b, 0, limit_ns);
        out[0] = done ? 0ull : 1ull;
        out[1] = tc::global_ns() - t0;
    }
}

cudaError_t selftest_bounded_wait(cudaStream_t st, unsigned long long limit_ns, unsigned long long *out) {
    k_selftest_bounded_wait<<<1, 32, 0, st>>>(limit_ns, out);
    return cudaGetLastError();
}

// rows[row] = 1 when a cell of row (i, j) has D > 0, else 0 (one warp per row)
__global__ void __launch_bounds__(256) k_rows_from_diag(Dims d, const double *__restrict__ D, uint8_t *__restrict__ rows) {
    for (long long row = blockIdx.x * 8LL + threadIdx.y, nr = (long long)d.nx * d.ny; row < nr;
         row += (long long)gridDim.x * 8) {
        bool on = false;
        for (int k = threadIdx.x; k < d.nz; k += 32) on |= D[row * d.nz + k] > 0;
        on = __any_sync(0xffffffffu, on);
        if (threadIdx.x == 0) rows[row] = on ? 1 : 0;
    }
}

// y = 0 on inactive cells (D = 0), where the solver's vectors are zero
__global__ void k_mask_active(long long n, const double *__restrict__ D, float *__restrict__ y) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        if (!(D[c] > 0)) y[c] = 0.f;
}

// Learned step: gamma = (r, y) / (y, A y) from the slots k_dot_rz left (RHONEW = (r, y), ZQ = (y, A y); 0 when
// not finite or (y, A y) <= 0); d = gamma y, r -= gamma A y, (r, r) -> RR; gamma, (r, y), (y, A y) -> the
// learned-step slots.
__global__ void __launch_bounds__(256) k_learned_update(long long n, float *__restrict__ dlt, float *__restrict__ r,
                                                        const float *__restrict__ y, const float *__restrict__ ay,
                                                        double *sc, double *part, unsigned *ticket) {
    const double ry = sc[S_RHONEW], yay = sc[S_ZQ];
    double g = (yay > 0 && isfinite(yay) && isfinite(ry)) ? ry / yay : 0.0;
    if (!isfinite(g)) g = 0.0;
    const float gf = (float)g;
    float acc = 0.f;
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    for (long long c = blockIdx.x * 256LL + tid; c < n; c += (long long)gridDim.x * 256) {
        // no step when gamma = 0: y and A y may hold non-finite values, and 0 times those is not zero
        const float rc = gf != 0.f ? r[c] - gf * ay[c] : r[c];
        dlt[c] = gf != 0.f ? gf * y[c] : 0.f;
        r[c] = rc;
        acc += rc * rc;
    }
    float v[1] = {acc};
    double tot[1];
    if (grid_reduce<1>(v, part, ticket, tot)) {
        sc[S_RR] = tot[0];
        sc[S_LGAMMA] = g;
        sc[S_LRY] = ry;
        sc[S_LYAY] = yay;
    }
}

// (y, b) with y FP32 and b FP64 -> slot
__global__ void __launch_bounds__(256) k_dot_fd(long long n, const float *__restrict__ y, const double *__restrict__ b,
                                                int slot, double *sc, double *part, unsigned *ticket) {
    float acc = 0.f;
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    for (long long c = blockIdx.x * 256LL + tid; c < n; c += (long long)gridDim.x * 256) acc += y[c] * (float)b[c];
    float v[1] = {acc};
    double tot[1];
    if (grid_reduce<1>(v, part, ticket, tot)) sc[slot] = tot[0];
}

__global__ void k_scale_to64(long long n, double g, const float *__restrict__ y, double *__restrict__ x) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        x[c] = g * (double)y[c];
}

// (a, b) of two FP64 vectors -> slot
__global__ void __launch_bounds__(256) k_dot_dd(long long n, const double *__restrict__ a, const double *__restrict__ b,
                                                int slot, double *sc, double *part, unsigned *ticket) {
    double v[1] = {0};
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    for (long long c = blockIdx.x * 256LL + tid; c < n; c += (long long)gridDim.x * 256) v[0] += a[c] * b[c];
    double tot[1];
    if (grid_reduce<1>(v, part, ticket, tot)) sc[slot] = tot[0];
}

// x64 += d32
__global__ void k_ir_update(long long n, double *__restrict__ x, const float *__restrict__ dlt) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        x[c] += (double)dlt[c];
}

__global__ void k_shift(long long n, double *__restrict__ x) {
    const double x0 = x[0];  // x[0] itself is not touched here (cleared by a memset afterwards)
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x + 1; c < n; c += (long long)gridDim.x * blockDim.x)
        x[c] -= x0;
}

template <class T>
__global__ void k_copy_cast(long long n, const double *__restrict__ a, T *__restrict__ o) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        o[c] = (T)a[c];
}

static inline int flat_grid(long long n) {
    long long g = (n + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    if (g < 1) g = 1;
    return (int)g;
}

// ------------------------------------------------------------------------------------------------ V-cycle
template <class T, class C>
static void rb(cudaStream_t st, Tracker &tk, bool fine, bool zero, const Dims &d, const Coef<C> &cf, T *x, const T *b,
               int color, const uint8_t *rows = nullptr) {
    const dim3 g = grid_pairs(d), bk = blk2();
    // algorithmic bytes of one colour: half of (x r/w + b + 3 couplings + diagonal term)
    const double per = (3.0 * sizeof(T) + 4.0 * sizeof(C)) / 2.0;
    const double cells = (fine && rows && tk.active0 >= 0) ? tk.active0 : (double)d.n;  // rows skipped
    tk.before(st, fine);
    if constexpr (std::is_same<T, float>::value && sizeof(C) <= 4) {
        if (d.nz % 4 == 0) {  // rows start 16-byte aligned: z-vectorised kernel
            const dim3 g4((d.nz / 4 + 31) / 32, (d.ny + 7) / 8, d.nx);
            if (zero)
                launch_pdl(k_rbgs4<C, true>, g4, bk, st, d, cf, x, b, color, rows);
            else
                launch_pdl(k_rbgs4<C, false>, g4, bk, st, d, cf, x, b, color, rows);
            tk.after(st, fine, per * cells);
            return;
        }
    }
    if (zero)
        launch_pdl(k_rbgs<T, C, true>, g, bk, st, d, cf, x, b, color, rows);
    else
        launch_pdl(k_rbgs<T, C, false>, g, bk, st, d, cf, x, b, color, rows);
    tk.after(st, fine, per * cells);
}

static inline int fused_chunk(const Dims &d) {
    // planes per block along x: enough blocks to fill 152 SMs a few times over, long runs for reuse
    const long long tiles = (long long)((d.nz + FTZ - 1) / FTZ) * ((d.ny + FTY - 1) / FTY);
    int chunk = 32;
    while (chunk > 4 && tiles * ((d.nx + chunk - 1) / chunk) < 152 * 6) chunk /= 2;
    return chunk < d.nx ? chunk : d.nx;
}

// TMA-staged one-pass sweep of the finest FP32 level (sf_rbgs_tma.cuh).  Needs nz a multiple of 4 (16-byte
// row strides for the tensor maps) and a grid at least one box wide in y and z.
static bool rbt_ok(const Dims &d) {
    return d.nz % 4 == 0 && d.nz >= rbt::BZ && d.ny >= rbt::BY && tensor_map_encoder() != nullptr;
}

// Tensor maps of finest-level arrays, encoded once per (address, dims): an address that is freed and reused with
// the same dims maps the same bytes, so entries never go stale.
static bool rbt_map(const float *p, const Dims &d, CUtensorMap &out) {
    static std::mutex mu;
    static std::map<std::tuple<const void *, int, int, int>, CUtensorMap> cache;
    const auto key = std::make_tuple(static_cast<const void *>(p), d.nx, d.ny, d.nz);
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
        out = it->second;
        return true;
    }
    auto enc = tensor_map_encoder();
    if (!enc || !p || (reinterpret_cast<uintptr_t>(p) & 15u)) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)d.nz, (cuuint64_t)d.ny, (cuuint64_t)d.nx};
    const cuuint64_t strides[2] = {(cuuint64_t)d.nz * 4, (cuuint64_t)d.ny * d.nz * 4};
    const cuuint32_t box[3] = {(cuuint32_t)rbt::BZ, (cuuint32_t)rbt::BY, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    CUtensorMap m;
    if (enc(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(p), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    cache.emplace(key, m);
    out = m;
    return true;
}

template <int MODE>
static bool launch_rbgs_tma(cudaStream_t st, Tracker &tk, const Dims &d, const Coef<float> &cf, const float *xin,
                            float *xout, const float *b) {
    if (!tk.sc) return false;
    rbt::Maps m;
    if (!rbt_map(MODE == 0 ? b : xin, d, m.x) || !rbt_map(cf.ax, d, m.ax) || !rbt_map(cf.ay, d, m.ay) ||
        !rbt_map(cf.az, d, m.az) || !rbt_map(cf.dex, d, m.dex) || !rbt_map(b, d, m.b))
        return false;
    // planes per block: 32, or fewer while the grid would not fill the 152 SMs (two blocks each) three times
    const long long tiles = (long long)((d.nz + rbt::TZ - 1) / rbt::TZ) * ((d.ny + rbt::TY - 1) / rbt::TY);
    int chunk = 32;
    while (chunk > 4 && tiles * ((d.nx + chunk - 1) / chunk) < 152 * 2 * 3) chunk /= 2;
    if (chunk > d.nx) chunk = d.nx;
    const dim3 g((d.nx + chunk - 1) / chunk, (d.nz + rbt::TZ - 1) / rbt::TZ, (d.ny + rbt::TY - 1) / rbt::TY);
    if (cudaFuncSetAttribute(rbt::k_rbgs_tma<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)rbt::kSmemBytes) != cudaSuccess)
        return false;
    // x in (not from zero) + x out + b + 3 couplings + dex
    const double per = (MODE == 0 ? 0.0 : 4.0) + 4.0 + 4.0 + 12.0 + 4.0;
    tk.before(st, true);
    rbt::k_rbgs_tma<MODE><<<g, dim3(32, 8), rbt::kSmemBytes, st>>>(m, d, xout, chunk, tk.sc, (int)S_ERR);
    tk.after(st, true, per * d.n);
    return true;
}

template <class T, class C, int MODE>
static void fused(cudaStream_t st, Tracker &tk, bool fine, const Dims &d, const Coef<C> &cf, const T *xin, T *xout,
                  const T *b) {
    if constexpr (std::is_same<T, C>::value) {
        if constexpr (std::is_same<T, float>::value) {
            if (fine && rbt_ok(d) && launch_rbgs_tma<MODE>(st, tk, d, cf, xin, xout, b)) return;
        }
        if (fine) {
            // pipelined kernel: two blocks (FP32) or one (FP64) per SM, blocks marching 32 planes
            const long long tiles = (long long)((d.nz + FTZ - 1) / FTZ) * ((d.ny + FTY - 1) / FTY);
            int chunk = 32;
            while (chunk > 4 && tiles * ((d.nx + chunk - 1) / chunk) < 152 * 6) chunk /= 2;
            if (chunk > d.nx) chunk = d.nx;
            const dim3 g((d.nz + FTZ - 1) / FTZ, (d.ny + FTY - 1) / FTY, (d.nx + chunk - 1) / chunk);
            const size_t smem = pipe_smem_bytes<T>();
            cudaFuncSetAttribute(k_rbgs_pipe<T, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            const double s = sizeof(T);
            const double per = (MODE == 0 ? 0.0 : s) + s + s + 3 * s + s;
            tk.before(st, fine);
            k_rbgs_pipe<T, MODE><<<g, dim3(32, 8), smem, st>>>(d, cf, xin, xout, b, chunk);
            tk.after(st, fine, per * d.n);
            return;
        }
    }
    const int chunk = fused_chunk(d);
    const dim3 g((d.nz + FTZ - 1) / FTZ, (d.ny + FTY - 1) / FTY, (d.nx + chunk - 1) / chunk);
    const double s = sizeof(C) == 8 ? 8.0 : 4.0;
    // x in (not from zero) + x out + b + 3 couplings + diagonal term
    const double per = (MODE == 0 ? 0.0 : s) + s + s + 3 * s + s;
    tk.before(st, fine);
    k_rbgs_fused<T, C, MODE><<<g, dim3(32, 8), 0, st>>>(d, cf, xin, xout, b, chunk);
    tk.after(st, fine, per * d.n);
}

// nu sweeps; the result always ends in x.  pre: starts from x = 0 (x's input value is ignored).
// fused (tmp != nullptr): one kernel per sweep, ping-ponging between x and tmp; else two in-place colours.
// Half sweep of the split level 0 (smoother 3); same algorithmic bytes as the natural half sweep.
template <class C>
static void rb_split(cudaStream_t st, Tracker &tk, bool fine, bool zero, const Dims &d, const Coef<C> &cf, float *x,
                     const float *b, int color, const int *list, const int *count, const float4 *rc,
                     const float *dinv) {
    const long long items = split_items((long long)d.nx * d.ny, d.nz >> 3);
    tk.before(st, fine);
    if (zero)
        launch_pdl(k_rbgs4s<C, true>, row_grid((const void *)k_rbgs4s<C, true>, items), blk2(), st, d, cf, x, b,
                   color, list, count, rc, dinv);
    else
        launch_pdl(k_rbgs4s<C, false>, row_grid((const void *)k_rbgs4s<C, false>, items), blk2(), st, d, cf, x, b,
                   color, list, count, rc, dinv);
    tk.after(st, fine, tk.bytes0 >= 0 ? tk.bytes0 : (3.0 * sizeof(float) + 4.0 * sizeof(C)) / 2.0 * d.n);
}

template <class T, class C>
static void smooth(cudaStream_t st, Tracker &tk, bool fine, const Dims &d, const Coef<C> &cf, T *x, T *tmp,
                   const T *b, int nu, bool pre, bool split = false, const uint8_t *rows = nullptr,
                   const int *list = nullptr, const int *count = nullptr, const float4 *rc = nullptr,
                   const float *dinv = nullptr) {
    if constexpr (std::is_same<T, float>::value && std::is_same<C, __half>::value) {  // split: FP16 copy only
        if (split) {
            for (int s = 0; s < nu; s++) {
                if (pre) {
                    rb_split<C>(st, tk, fine, s == 0, d, cf, x, b, 0, list, count, rc, dinv);
                    rb_split<C>(st, tk, fine, false, d, cf, x, b, 1, list, count, rc, dinv);
                } else {
                    rb_split<C>(st, tk, fine, false, d, cf, x, b, 1, list, count, rc, dinv);
                    rb_split<C>(st, tk, fine, false, d, cf, x, b, 0, list, count, rc, dinv);
                }
            }
            return;
        }
    }
    if (!tmp) {
        for (int s = 0; s < nu; s++) {
            if (pre) {
                rb<T, C>(st, tk, fine, s == 0, d, cf, x, b, 0, rows);
                rb<T, C>(st, tk, fine, false, d, cf, x, b, 1, rows);
            } else {
                rb<T, C>(st, tk, fine, false, d, cf, x, b, 1, rows);
                rb<T, C>(st, tk, fine, false, d, cf, x, b, 0, rows);
            }
        }
        return;
    }
    if (pre) {
        T *prev = nullptr;
        for (int s = 0; s < nu; s++) {
            T *out = ((nu - 1 - s) % 2 == 0) ? x : tmp;
            if (s == 0)
                fused<T, C, 0>(st, tk, fine, d, cf, (const T *)nullptr, out, b);
            else
                fused<T, C, 1>(st, tk, fine, d, cf, prev, out, b);
            prev = out;
        }
    } else {
        for (int s = 0; s < nu; s++) {
            const T *in = (s % 2 == 0) ? x : tmp;
            T *out = (s % 2 == 0) ? tmp : x;
            fused<T, C, 2>(st, tk, fine, d, cf, in, out, b);
        }
        if (nu % 2 == 1) {
            tk.launches++;
            cudaMemcpyAsync(x, tmp, sizeof(T) * d.n, cudaMemcpyDeviceToDevice, st);
        }
    }
}

template <class T, class C>
static void restrict_res(cudaStream_t st, Tracker &tk, const Dims &d, const Coef<C> &cf, const T *x, const T *b,
                         const Dims &dc, T *bc, bool split = false, const uint8_t *rows = nullptr,
                         const uint8_t *rows_c = nullptr, const int *list_c = nullptr,
                         const int *count_c = nullptr, const float *crow = nullptr, bool sout = false) {
    tk.launches++;
    if constexpr (std::is_same<T, float>::value && std::is_same<C, __half>::value) {
        if (split) {
            const long long items = split_items((long long)dc.nx * dc.ny, dc.nz >> 2);
            if (sout)
                launch_pdl(k_resid_restrict_s<C, true>, row_grid((const void *)k_resid_restrict_s<C, true>, items),
                           blk2(), st, d, cf, x, b, dc, bc, rows, crow, list_c, count_c);
            else
                launch_pdl(k_resid_restrict_s<C, false>, row_grid((const void *)k_resid_restrict_s<C, false>, items),
                           blk2(), st, d, cf, x, b, dc, bc, rows, crow, list_c, count_c);
            return;
        }
    }
    launch_pdl(k_resid_restrict<T, C>, grid_cells(dc), blk2(), st, d, cf, x, b, dc, bc, rows, rows_c);
}

template <class T, class C>
static void coarse_solve(cudaStream_t st, Tracker &tk, const Dims &d, const Coef<C> &cf, T *x, const T *b, int pairs) {
    tk.launches++;
    if (d.n <= kCoarseMax) {
        launch_pdl(k_coarse_smem<T, C>, 1, kCoarseThreads, st, d, cf, x, b, pairs);
        return;
    }
    int nt = d.n >= 1024 ? 1024 : (int)((d.n + 31) / 32 * 32);
    launch_pdl(k_coarse<T, C>, 1, nt, st, d, cf, x, b, pairs);
}

// V-cycle z = M r.  Level 0 uses coefficient type C0, coarse levels Cc (cc[l] for level l >= 1).  ts[l] is a
// scratch vector of level l for the fused smoother (nullptr entries select the in-place two-colour smoother).
// c0s: level-0 coefficients read by the level-0 smoother and the residual restriction (c0 itself, or a
// lower-precision copy, making the V-cycle a multigrid cycle for that copy); the coarsest solve of a one-level
// hierarchy uses c0.
// Row activity of a hierarchy with a split level 0: flags per level, and the ordered active rows of levels 0
// and 1 (the persistent split kernels walk those lists).
struct RowSets {
    const std::vector<uint8_t *> *flags;
    const int *list[3], *count[3];  // levels 0, 1, 2
    const float *crow[2];           // levels 0, 1: the coupling of each uniform row
    const Coef<__half> *c1s;        // split FP16 operator of level 1 when level 1 is split too, else nullptr
    const float4 *rc[2];            // levels 0, 1: the smoother's row constants (k_smooth_consts_s)
    const float *dinv[2];           // levels 0, 1: the smoother's 1 / D on general rows
};

template <class T, class C0, class Cc, class C0S>
static void vcycle(cudaStream_t st, Tracker &tk, const std::vector<Dims> &dims, const Coef<C0> &c0,
                   const Coef<C0S> &c0s, const std::vector<Coef<Cc>> &cc, T *z, const T *r,
                   const std::vector<T *> &xs, const std::vector<T *> &bs, const std::vector<T *> &ts,
                   const SolverParams &p, bool split0 = false, const RowSets *rs = nullptr, int tail_lt = -1,
                   int tail_smem = 0, int tail_nc = 8, float *const *tail_op = nullptr) {
    const int L = (int)dims.size();
    if (L == 1) {
        coarse_solve<T, C0>(st, tk, dims[0], c0, z, r, p.coarse_sweeps);
        return;
    }
    auto R = [&](int l) -> const uint8_t * { return rs ? (*rs->flags)[l] : nullptr; };
    auto LST = [&](int l) -> const int * { return rs ? rs->list[l] : nullptr; };
    auto CNT = [&](int l) -> const int * { return rs ? rs->count[l] : nullptr; };
    const float *cr = rs ? rs->crow[0] : nullptr, *cr1 = rs ? rs->crow[1] : nullptr;
    // level 1 split as well: its vectors and its FP16 operator copy *rs->c1s are stored colour by colour
    bool split1 = false;
    if constexpr (std::is_same<T, float>::value && std::is_same<Cc, __half>::value) split1 = rs && rs->c1s;
    smooth<T, C0S>(st, tk, true, dims[0], c0s, z, ts[0], r, p.pre, true, split0, R(0), LST(0), CNT(0),
                   rs ? rs->rc[0] : nullptr, rs ? rs->dinv[0] : nullptr);
    // the residual of the smoothed operator
    restrict_res<T, C0S>(st, tk, dims[0], c0s, z, r, dims[1], bs[1], split0, R(0), R(1), LST(1), CNT(1), cr, split1);
    // levels from `bottom` on are solved in one piece: the coarsest solve, or the fused tail (one cluster launch
    // for every level from tail_lt on)
    bool tail = false;
    if constexpr (std::is_same<T, float>::value && std::is_same<Cc, __half>::value)
        tail = tail_lt >= (split1 ? 2 : 1) && tail_lt < L - 1;
    const int bottom = tail ? tail_lt : L - 1;
    for (int l = 1; l < bottom; l++) {
        if constexpr (std::is_same<T, float>::value && std::is_same<Cc, __half>::value) {
            if (l == 1 && split1) {
                const Coef<__half> &c1 = *rs->c1s;
                smooth<T, Cc>(st, tk, false, dims[1], c1, xs[1], nullptr, bs[1], p.pre, true, true, R(1), LST(1),
                              CNT(1), rs->rc[1], rs->dinv[1]);
                restrict_res<T, Cc>(st, tk, dims[1], c1, xs[1], bs[1], dims[2], bs[2], true, R(1), R(2), LST(2),
                                    CNT(2), cr1);
                continue;
            }
        }
        smooth<T, Cc>(st, tk, false, dims[l], cc[l], xs[l], nullptr, bs[l], l >= 2 ? p.coarse_pre : p.pre, true, false,
                      R(l));
        restrict_res<T, Cc>(st, tk, dims[l], cc[l], xs[l], bs[l], dims[l + 1], bs[l + 1], false, R(l), R(l + 1));
    }
    if constexpr (std::is_same<T, float>::value && std::is_same<Cc, __half>::value) {
        if (tail) {
            TailParams P{};
            int smem = 0;
            tail_plan(dims, tail_lt, tail_nc, P, smem);
            for (int l = 0; l < P.nlev; l++) {
                P.lv[l].cf = cc[tail_lt + l];
                P.lv[l].unscale = cc[tail_lt + l].unscale;
                P.lv[l].op = tail_op[tail_lt + l];
                P.lv[l].pre = tail_lt + l >= 2 ? p.coarse_pre : p.pre;
                P.lv[l].post = tail_lt + l >= 2 ? p.coarse_post : p.post;
            }
            P.b0 = bs[tail_lt];
            P.x0 = xs[tail_lt];
            P.pairs = p.coarse_sweeps;
            tk.launches++;
            if (launch_tail(st, tail_nc, P, tail_smem) != cudaSuccess) {
                cudaGetLastError();
                tk.tail_failed = true;
                tail = false;  // the same levels with the separate kernels (same arithmetic, same bits)
                for (int l = bottom; l < L - 1; l++) {
                    smooth<T, Cc>(st, tk, false, dims[l], cc[l], xs[l], nullptr, bs[l],
                                  l >= 2 ? p.coarse_pre : p.pre, true, false, R(l));
                    restrict_res<T, Cc>(st, tk, dims[l], cc[l], xs[l], bs[l], dims[l + 1], bs[l + 1], false, R(l),
                                        R(l + 1));
                }
            }
        }
    }
    if (!tail) coarse_solve<T, Cc>(st, tk, dims[L - 1], cc[L - 1], xs[L - 1], bs[L - 1], p.coarse_sweeps);
    for (int l = L - 2; !tail && l >= bottom && bottom < L - 1; l--) {  // after a rejected tail launch
        tk.launches++;
        launch_pdl(k_prolong<T>, grid_cells(dims[l]), blk2(), st, dims[l], xs[l], dims[l + 1], xs[l + 1], R(l));
        smooth<T, Cc>(st, tk, false, dims[l], cc[l], xs[l], nullptr, bs[l], l >= 2 ? p.coarse_post : p.post, false,
                      false, R(l));
    }
    for (int l = bottom - 1; l >= 1; l--) {
        tk.launches++;
        if constexpr (std::is_same<T, float>::value && std::is_same<Cc, __half>::value) {
            if (l == 1 && split1) {
                const Dims &d1 = dims[1];
                const int g = row_grid((const void *)k_prolong_s, split_items((long long)d1.nx * d1.ny, d1.nz >> 3));
                launch_pdl(k_prolong_s, g, blk2(), st, d1, xs[1], dims[2], xs[2], LST(1), CNT(1));
                smooth<T, Cc>(st, tk, false, d1, *rs->c1s, xs[1], nullptr, bs[1], p.post, false, true, R(1), LST(1),
                              CNT(1), rs->rc[1], rs->dinv[1]);
                continue;
            }
        }
        launch_pdl(k_prolong<T>, grid_cells(dims[l]), blk2(), st, dims[l], xs[l], dims[l + 1], xs[l + 1], R(l));
        smooth<T, Cc>(st, tk, false, dims[l], cc[l], xs[l], nullptr, bs[l], l >= 2 ? p.coarse_post : p.post, false,
                      false, R(l));
    }
    tk.launches++;
    if constexpr (std::is_same<T, float>::value) {
        if (split0) {
            const Dims &d0 = dims[0];
            const long long items = split_items((long long)d0.nx * d0.ny, d0.nz >> 3);
            if (split1)
                launch_pdl(k_prolong_ss, row_grid((const void *)k_prolong_ss, items), blk2(), st, d0, z, dims[1], xs[1],
                           LST(0), CNT(0));
            else
                launch_pdl(k_prolong_s, row_grid((const void *)k_prolong_s, items), blk2(), st, d0, z, dims[1], xs[1],
                           LST(0), CNT(0));
            smooth<T, C0S>(st, tk, true, dims[0], c0s, z, ts[0], r, p.post, false, true, R(0), LST(0), CNT(0),
                           rs->rc[0], rs->dinv[0]);
            return;
        }
    }
    launch_pdl(k_prolong<T>, grid_cells(dims[0]), blk2(), st, dims[0], z, dims[1], xs[1], R(0));
    smooth<T, C0S>(st, tk, true, dims[0], c0s, z, ts[0], r, p.post, false, false, R(0));
}

// ------------------------------------------------------------------------------------------------ MGSolver
MGSolver::MGSolver(cudaStream_t s) : st_(s) {}
MGSolver::~MGSolver() {
    destroy_graphs();
    free_all();
}

void MGSolver::destroy_graphs() {
    if (g_iter64_) cudaGraphExecDestroy(g_iter64_);
    if (g_iter32_) cudaGraphExecDestroy(g_iter32_);
    if (g_loop32_) cudaGraphExecDestroy(g_loop32_);
    if (g_loop64_) cudaGraphExecDestroy(g_loop64_);
    g_iter64_ = g_iter32_ = g_loop32_ = g_loop64_ = nullptr;
    graph_key_ = -1;
}

bool MGSolver::drop_tail() {
    if (!tk_.tail_failed) return false;
    tk_.tail_failed = false;
    tail_lt_ = -1;
    tail_smem_ = tail_nc_ = 0;
    destroy_graphs();
    return true;
}

void MGSolver::free_all() {
    bufs_.clear();
    if (sc_host_) cudaFreeHost(sc_host_);
    sc_host_ = nullptr;
    bytes_ = 0;
    configured_ = false;
}

void *MGSolver::alloc(size_t bytes) {
    bytes = (bytes + 255) / 256 * 256;
    auto b = std::make_unique<DevBuf>();
    if (b->ensure(bytes) != cudaSuccess) return nullptr;
    void *p = b->get();
    bytes_ += bytes;
    bufs_.push_back(std::move(b));
    return p;
}

size_t MGSolver::device_bytes() const { return bytes_; }

cudaError_t MGSolver::configure(const Dims &d, const SolverParams &p) {
    if ((long long)((d.nz + 31) / 32) * ((d.ny + 7) / 8) > kApplyBlocks) {  // tile_grid3's one block per tile
        last_error = "grid cross-section above 16384 tiles of 32 (z) x 8 (y) cells";
        return cudaErrorInvalidValue;
    }
    // level dims
    std::vector<Dims> dims{d};
    const int cdim = p.coarse_dim > 0 ? p.coarse_dim : 8;
    while (true) {
        const Dims &t = dims.back();
        if (p.max_levels > 0 && (int)dims.size() >= p.max_levels) break;
        if (t.nx <= cdim && t.ny <= cdim && t.nz <= cdim) break;
        dims.push_back(make_dims((t.nx + 1) / 2, (t.ny + 1) / 2, (t.nz + 1) / 2));
    }
    // smoother 3 (split level 0) needs rows of whole 16-byte vectors per colour, a coarse level, and a split
    // Krylov operator grid within the reduction's block budget; otherwise it runs as smoother 2
    const bool split0 = p.precision == 1 && p.smoother == 3 && d.nz % 8 == 0 && dims.size() >= 2 && d.nx < 32768 &&
                        d.ny < 65536 &&
                        (long long)(((d.nz >> 1) + 127) / 128) * 2 * ((d.ny + 7) / 8) <= kApplyBlocks;
    const bool fp16copy = p.smoother == 2 || p.smoother == 3;
    // FP64 form: row flags on every level unless every row is swept (the fused one-pass sweep has none)
    const bool rows64 = p.precision == 0 && !p.full_sweeps && p.smoother != 1;
    const bool same = configured_ && cfg_dims_.nx == d.nx && cfg_dims_.ny == d.ny && cfg_dims_.nz == d.nz &&
                      cfg_prec_ == p.precision && cfg_levels_ == (int)dims.size() && cfg_cdim_ == cdim &&
                      (p.precision == 0 ? rows64_ == rows64
                                        : ((cfg_smoother_ == 2 || cfg_smoother_ == 3) == fp16copy && cfg_split_ == split0));
    prm_ = p;
    if (same) {
        plan_tail();
        return cudaSuccess;
    }
    destroy_graphs();
    free_all();
    lev_dims_ = dims;
    rows64_ = rows64;
    const int L = (int)dims.size();
    const long long n = d.n;
    auto A = [&](size_t bytes) -> void * { return alloc(bytes); };
    bool ok = true;
    auto chk = [&](void *q) {
        if (!q) ok = false;
        return q;
    };
    c64_.assign(p.precision == 0 ? L : 1, Coef<double>{});
    for (int l = 0; l < (int)c64_.size(); l++) {
        const long long m = dims[l].n;
        Coef<double> &c = c64_[l];
        c.ax = (double *)chk(A(8 * m));
        c.ay = (double *)chk(A(8 * m));
        c.az = (double *)chk(A(8 * m));
        c.dex = (double *)chk(A(8 * m));
        c.D = (double *)chk(A(8 * m));
        c.invd = (double *)chk(A(8 * m));
        c.scale = c.unscale = 1.f;
    }
    x_ = (double *)chk(A(8 * n));
    b_ = (double *)chk(A(8 * n));
    sc_ = (double *)chk(A(8 * S_NSLOTS));
    tk_.sc = sc_;
    part_ = (double *)chk(A(8 * 4 * (size_t)(kMaxRedGrid + kMaxRedGrid / kRedGroup + 1)));
    ticket_ = (unsigned *)chk(A(4 * (size_t)(2 + kMaxRedGrid / kRedGroup)));
    if (p.precision == 0) {
        x64_.assign(L, nullptr);
        b64_.assign(L, nullptr);
        t64_.assign(L, nullptr);
        for (int l = 0; l < L; l++) t64_[l] = (double *)chk(A(8 * dims[l].n));
        for (int l = 1; l < L; l++) {
            x64_[l] = (double *)chk(A(8 * dims[l].n));
            b64_[l] = (double *)chk(A(8 * dims[l].n));
        }
        r_ = (double *)chk(A(8 * n));
        z_ = (double *)chk(A(8 * n));
        p_ = (double *)chk(A(8 * n));
        q_ = (double *)chk(A(8 * n));
        rows_.assign(rows64 ? L : 0, nullptr);
        for (int l = 0; l < (int)rows_.size(); l++) rows_[l] = (uint8_t *)chk(A((size_t)dims[l].nx * dims[l].ny));
    } else {
        c32_.ax = (float *)chk(A(4 * n));
        c32_.ay = (float *)chk(A(4 * n));
        c32_.az = (float *)chk(A(4 * n));
        c32_.dex = (float *)chk(A(4 * n));
        c32_.D = c32_.invd = nullptr;
        c32_.scale = c32_.unscale = 1.f;
        c16s0_ = Coef<__half>{};
        if (fp16copy) {
            c16s0_.ax = (__half *)chk(A(2 * n));
            c16s0_.ay = (__half *)chk(A(2 * n));
            c16s0_.az = (__half *)chk(A(2 * n));
            c16s0_.dex = (__half *)chk(A(2 * n));
            c16s0_.scale = c16s0_.unscale = 1.f;
        }
        c16_.assign(L, Coef<__half>{});
        tail_op_.assign(L, nullptr);
        for (int l = 1; l < L; l++)
            if (dims[l].n <= kTailMaxCells) tail_op_[l] = (float *)chk(A(4 * (size_t)kTailOps * dims[l].n));
        x32_.assign(L, nullptr);
        b32_.assign(L, nullptr);
        t32_.assign(L, nullptr);
        for (int l = 0; l < L; l++) t32_[l] = (float *)chk(A(4 * dims[l].n));
        for (int l = 1; l < L; l++) {
            const long long m = dims[l].n;
            Coef<__half> &c = c16_[l];
            c.ax = (__half *)chk(A(2 * m));
            c.ay = (__half *)chk(A(2 * m));
            c.az = (__half *)chk(A(2 * m));
            c.dex = (__half *)chk(A(2 * m));
            c.D = c.invd = nullptr;
            // level-l couplings grow ~2^l and excesses up to 4^l: store scaled by 4^-l
            c.scale = ldexpf(1.f, -2 * l);
            c.unscale = ldexpf(1.f, 2 * l);
            x32_[l] = (float *)chk(A(4 * m));
            b32_[l] = (float *)chk(A(4 * m));
        }
        rows_.assign(split0 ? L : 0, nullptr);
        for (int l = 0; l < (int)rows_.size(); l++) rows_[l] = (uint8_t *)chk(A((size_t)dims[l].nx * dims[l].ny));
        list_[0] = list_[1] = nullptr;
        count_ = nullptr;
        crow_ = crow1_ = nullptr;
        rc_[0] = rc_[1] = nullptr;
        dinv_[0] = dinv_[1] = nullptr;
        list_[2] = nullptr;
        c16s1_ = Coef<__half>{};
        // level 1 split too when it has a coarser level and whole 16-byte rows per colour
        const bool split1 = split0 && L >= 3 && dims[1].nz % 8 == 0;
        if (split0) {
            for (int l = 0; l < (split1 ? 3 : 2); l++) list_[l] = (int *)chk(A(4 * (size_t)dims[l].nx * dims[l].ny));
            count_ = (int *)chk(A(16));
            crow_ = (float *)chk(A(4 * (size_t)dims[0].nx * dims[0].ny));
            rc_[0] = (float4 *)chk(A(16 * (size_t)dims[0].nx * dims[0].ny));
            dinv_[0] = (float *)chk(A(4 * (size_t)dims[0].n));
            list_cnt_ = (int *)chk(A(8 * (((size_t)dims[0].nx * dims[0].ny + kListRows - 1) / kListRows)));
            if (split1) {
                crow1_ = (float *)chk(A(4 * (size_t)dims[1].nx * dims[1].ny));
                rc_[1] = (float4 *)chk(A(16 * (size_t)dims[1].nx * dims[1].ny));
                dinv_[1] = (float *)chk(A(4 * (size_t)dims[1].n));
                const long long m = dims[1].n;
                c16s1_.ax = (__half *)chk(A(2 * m));
                c16s1_.ay = (__half *)chk(A(2 * m));
                c16s1_.az = (__half *)chk(A(2 * m));
                c16s1_.dex = (__half *)chk(A(2 * m));
                c16s1_.D = c16s1_.invd = nullptr;
                c16s1_.scale = ldexpf(1.f, -2);  // as level 1's natural copy
                c16s1_.unscale = ldexpf(1.f, 2);
            }
        }
        split1_ = split1;
        r32_ = (float *)chk(A(4 * n));
        d32_ = (float *)chk(A(4 * n));
        z32_ = (float *)chk(A(4 * n));
        p32_ = (float *)chk(A(4 * n));
        q32_ = (float *)chk(A(4 * n));
        ri32_ = r32_;
    }
    if (!ok) {
        free_all();
        last_error = "device allocation failed";
        return cudaErrorMemoryAllocation;
    }
    cudaError_t e = cudaMallocHost(&sc_host_, 8 * S_NSLOTS);
    if (e != cudaSuccess) return e;
    cudaMemsetAsync(ticket_, 0, 4 * (size_t)(2 + kMaxRedGrid / kRedGroup), st_);
    cudaMemsetAsync(sc_, 0, 8 * S_NSLOTS, st_);
    cudaMemsetAsync(x_, 0, 8 * n, st_);
    configured_ = true;
    cfg_dims_ = d;
    cfg_prec_ = p.precision;
    cfg_levels_ = L;
    cfg_cdim_ = cdim;
    cfg_smoother_ = p.smoother;
    cfg_split_ = split0_ = split0;
    if (split0) {  // occupancy lookups of the persistent split kernels, here rather than inside a graph capture
        const void *ks[] = {(const void *)k_rbgs4s<__half, true>, (const void *)k_rbgs4s<__half, false>,
                            (const void *)k_resid_restrict_s<__half, false>,
                            (const void *)k_resid_restrict_s<__half, true>, (const void *)k_prolong_s,
                            (const void *)k_prolong_ss, (const void *)k_apply_dot4s, (const void *)k_dot_rz_s,
                            (const void *)k_xpby_s, (const void *)k_update_s, (const void *)k_ir_update_s};
        for (const void *k : ks) resident_grid(k);
    }
    plan_tail();
    return cudaGetLastError();
}

// The fused tail (sf_tail.cuh) of the mixed V-cycle: from the first level of at most kTailMaxCells cells below
// the split levels, when its layout fits in shared memory and one cluster of it fits on the device.
void MGSolver::plan_tail() {
    tail_lt_ = -1;
    tail_smem_ = tail_nc_ = 0;
    if (prm_.precision != 1 || prm_.tail == 1) return;
    const int L = (int)lev_dims_.size();
    for (int nc : {16, 8}) {
        if (prm_.tail != 0 && prm_.tail != nc) continue;
        for (int lt = split1_ ? 2 : 1; lt < L - 1; lt++) {
            TailParams P{};
            int smem = 0;
            if (lev_dims_[lt].n > kTailMaxCells || !tail_plan(lev_dims_, lt, nc, P, smem)) continue;
            if (nc == 16 ? tail_launchable<16>(smem) : tail_launchable<8>(smem)) {
                tail_lt_ = lt;
                tail_smem_ = smem;
                tail_nc_ = nc;
                return;
            }
            break;
        }
    }
}

const SplitOut *MGSolver::split_targets() {
    if (!split0_) return nullptr;
    so_.c32 = c32_;
    so_.c16 = c16s0_;
    so_.rows = rows_[0];
    copies_written_ = true;
    return &so_;
}

cudaError_t MGSolver::build_hierarchy() {
    const int L = (int)lev_dims_.size();
    tk_.launches += prm_.precision == 0 ? (L - 1) : L;
    if (prm_.precision == 0) {
        for (int l = 1; l < L; l++)
            k_coarsen<double, double><<<grid_cells(lev_dims_[l]), blk2(), 0, st_>>>(lev_dims_[l - 1], c64_[l - 1],
                                                                                    lev_dims_[l], c64_[l]);
        if (rows64_) {
            // row flags from the fine diagonal (D > 0), coarse rows active where a fine row is; the vectors of
            // inactive rows must be zero and stay so
            const Dims &d0 = lev_dims_[0];
            const long long nr0 = (long long)d0.nx * d0.ny;
            k_rows_from_diag<<<(int)std::min<long long>((nr0 + 7) / 8, 152 * 16), dim3(32, 8), 0, st_>>>(
                d0, c64_[0].D, rows_[0]);
            cudaMemsetAsync(z_, 0, 8 * (size_t)d0.n, st_);
            for (int l = 1; l < L; l++) {
                const Dims &dl = lev_dims_[l];
                const long long nr = (long long)dl.nx * dl.ny;
                k_rows_coarsen<<<(int)std::min<long long>((nr + 255) / 256, 152 * 8), 256, 0, st_>>>(
                    lev_dims_[l - 1], rows_[l - 1], dl, rows_[l]);
                cudaMemsetAsync(x64_[l], 0, 8 * (size_t)dl.n, st_);
                cudaMemsetAsync(b64_[l], 0, 8 * (size_t)dl.n, st_);
            }
            tk_.launches += L;
            tk_.active0 = -1;
            if (prm_.profile) {  // profiled runs synchronise anyway: the smoother's bytes over active rows only
                std::vector<uint8_t> h((size_t)nr0);
                cudaMemcpyAsync(h.data(), rows_[0], h.size(), cudaMemcpyDeviceToHost, st_);
                const cudaError_t e = cudaStreamSynchronize(st_);
                if (e != cudaSuccess) return e;
                long long act = 0;
                for (uint8_t v : h) act += v != 0;
                tk_.active0 = (double)act * d0.nz;
            }
        }
    } else {
        if (split0_) {
            if (!copies_written_)
                k_to_split<<<split_rows_grid(lev_dims_[0]), dim3(32, 8), 0, st_>>>(lev_dims_[0], c64_[0], c32_,
                                                                                    c16s0_, rows_[0]);
            copies_written_ = false;
            k_rows_uniform<float><<<split_rows_grid(lev_dims_[0]), dim3(32, 8), 0, st_>>>(lev_dims_[0], c32_, rows_[0],
                                                                                          crow_);
            k_smooth_consts_s<__half><<<split_rows_grid(lev_dims_[0]), dim3(32, 8), 0, st_>>>(
                lev_dims_[0], c16s0_, rows_[0], crow_, rc_[0], dinv_[0]);
            tk_.launches += 2;
            // rows that hold no active cell are skipped by every level-l kernel; their vector entries must be
            // zero, and stay so
            cudaMemsetAsync(z32_, 0, 4 * (size_t)lev_dims_[0].n, st_);
            for (int l = 1; l < L; l++) {
                const Dims &dl = lev_dims_[l];
                const long long nr = (long long)dl.nx * dl.ny;
                k_rows_coarsen<<<(int)std::min<long long>((nr + 255) / 256, 152 * 8), 256, 0, st_>>>(
                    lev_dims_[l - 1], rows_[l - 1], dl, rows_[l]);
                cudaMemsetAsync(x32_[l], 0, 4 * (size_t)dl.n, st_);
                cudaMemsetAsync(b32_[l], 0, 4 * (size_t)dl.n, st_);
            }
            // level 1 from the split FP32 copy (half the bytes of the FP64 operator, FP32 sums), with its own split
            // copy and uniform rows when level 1 is split too
            k_coarsen_s<<<grid_cells(lev_dims_[1]), blk2(), 0, st_>>>(lev_dims_[0], c32_, lev_dims_[1], c16_[1],
                                                                       split1_ ? c16s1_ : Coef<__half>{});
            tk_.launches += L - 1;
            if (split1_) {
                k_rows_uniform<__half><<<split_rows_grid(lev_dims_[1]), dim3(32, 8), 0, st_>>>(lev_dims_[1], c16s1_,
                                                                                               rows_[1], crow1_);
                k_smooth_consts_s<__half><<<split_rows_grid(lev_dims_[1]), dim3(32, 8), 0, st_>>>(
                    lev_dims_[1], c16s1_, rows_[1], crow1_, rc_[1], dinv_[1]);
                tk_.launches += 2;
            }
            for (int l = 0; l < (split1_ ? 3 : 2); l++) {
                const long long nr = (long long)lev_dims_[l].nx * lev_dims_[l].ny;
                const int nb = (int)((nr + kListRows - 1) / kListRows);
                k_rows_count<<<nb, kListRows, 0, st_>>>(nr, rows_[l], list_cnt_);
                k_rows_scatter<<<nb, kListRows, 0, st_>>>(nr, lev_dims_[l].ny, rows_[l], list_cnt_, list_[l],
                                                          count_ + l);
                tk_.launches += 2;
            }
            tk_.bytes0 = -1;
            if (prm_.profile) {  // profiled runs synchronise anyway: count the level-0 rows by kind
                const Dims &d0 = lev_dims_[0];
                std::vector<uint8_t> h((size_t)d0.nx * d0.ny);
                cudaMemcpyAsync(h.data(), rows_[0], h.size(), cudaMemcpyDeviceToHost, st_);
                const cudaError_t e = cudaStreamSynchronize(st_);
                if (e != cudaSuccess) return e;
                long long gen = 0, uni = 0;
                for (uint8_t v : h) {
                    gen += v == 1;
                    uni += v == 2;
                }
                // algorithmic bytes of a half sweep per grid cell: 11 on a general row (x r/w, b, 3 FP16
                // couplings and the FP32 1 / D, half of each), 6 on a uniform row (x r/w and b)
                tk_.bytes0 = (11.0 * gen + 6.0 * uni) * d0.nz;
            }
        } else {
            k_to32<<<flat_grid(lev_dims_[0].n), 256, 0, st_>>>(lev_dims_[0].n, c64_[0], c32_);
            if (prm_.smoother == 2 || prm_.smoother == 3) {
                k_to16<<<flat_grid(lev_dims_[0].n), 256, 0, st_>>>(lev_dims_[0].n, c64_[0], c16s0_);
                tk_.launches++;
            }
        }
        if (!split0_ && L > 1)
            k_coarsen<double, __half><<<grid_cells(lev_dims_[1]), blk2(), 0, st_>>>(lev_dims_[0], c64_[0],
                                                                                    lev_dims_[1], c16_[1]);
        for (int l = 2; l < L; l++)
            k_coarsen<__half, __half><<<grid_cells(lev_dims_[l]), blk2(), 0, st_>>>(lev_dims_[l - 1], c16_[l - 1],
                                                                                    lev_dims_[l], c16_[l]);
        // the fused tail's FP32 operator of its levels above the coarsest
        for (int l = std::max(tail_lt_, 1); tail_lt_ >= 0 && l < L - 1; l++) {
            k_tail_op<<<grid_cells(lev_dims_[l]), blk2(), 0, st_>>>(lev_dims_[l], c16_[l], tail_op_[l]);
            tk_.launches++;
        }
    }
    return cudaGetLastError();
}

void MGSolver::enqueue_iter64(bool copy_slots) {
    const Dims &d = lev_dims_[0];
    const long long n = d.n;
    int xpb;
    const dim3 tg = tile_grid3(d, xpb);
    const long long l0 = tk_.launches;
    // with row flags (rows64_): the smoothers, transfers and vector kernels skip rows without an active cell
    const RowSets rs{&rows_, {nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}, {nullptr, nullptr}, nullptr,
                     {nullptr, nullptr}, {nullptr, nullptr}};
    const uint8_t *r0 = rows64_ ? rows_[0] : nullptr;
    vcycle<double, double, double, double>(st_, tk_, lev_dims_, c64_[0], c64_[0], c64_, z_, r_, x64_, b64_,
                                           prm_.smoother == 1 ? t64_ : std::vector<double *>(t64_.size(), nullptr),
                                           prm_, false, rows64_ ? &rs : nullptr);
    launch_pdl(k_dot_rz<double>, kMaxRedBlocks, dim3(32, 8), st_, d, r0, r_, z_, q_, prm_.flexible ? 1 : 0, sc_,
               part_, ticket_);
    launch_pdl(k_xpby<double>, kMaxRedBlocks, dim3(32, 8), st_, d, r0, z_, p_, sc_);
    launch_pdl(k_apply_dot<double, double>, tg, dim3(32, 8), st_, d, xpb, c64_[0], p_, q_, sc_, part_, ticket_, r0);
    launch_pdl(k_update<double>, kMaxRedBlocks, dim3(32, 8), st_, d, r0, x_, r_, p_, q_, sc_, part_, ticket_);
    tk_.launches += 4;
    iter_launches64_ = tk_.launches - l0;
    if (copy_slots) cudaMemcpyAsync(sc_host_, sc_, 8 * S_NSLOTS, cudaMemcpyDeviceToHost, st_);
}

void MGSolver::enqueue_iter32(bool copy_slots) {
    const Dims &d = lev_dims_[0];
    const long long n = d.n;
    const long long l0 = tk_.launches;
    const std::vector<float *> ts = prm_.smoother == 1 ? t32_ : std::vector<float *>(t32_.size(), nullptr);
    if (split0_) {
        // colour-split level 0 with row flags on every level (vectors in split rows, inactive rows skipped)
        const RowSets rs{&rows_, {list_[0], list_[1], list_[2]}, {count_, count_ + 1, count_ + 2}, {crow_, crow1_},
                         split1_ ? &c16s1_ : nullptr, {rc_[0], rc_[1]}, {dinv_[0], dinv_[1]}};
        const int *lst0 = list_[0], *cnt0 = count_;
        vcycle<float, float, __half, __half>(st_, tk_, lev_dims_, c32_, c16s0_, c16_, z32_, ri32_, x32_, b32_, ts,
                                             prm_, true, &rs, tail_lt_, tail_smem_, tail_nc_, tail_op_.data());
        const long long vitems = split_items(2LL * d.nx * d.ny, d.nz >> 3);
        launch_pdl(k_dot_rz_s, row_grid((const void *)k_dot_rz_s, vitems), dim3(32, 8), st_, d, ri32_, z32_, q32_,
                   lst0, cnt0, 1, sc_, part_, ticket_);
        launch_pdl(k_xpby_s, row_grid((const void *)k_xpby_s, vitems), dim3(32, 8), st_, d, z32_, p32_, lst0, cnt0,
                   sc_);
        apply_dot32s(st_, d, c32_, p32_, q32_, lst0, cnt0, crow_, sc_, part_, ticket_);
        launch_pdl(k_update_s, row_grid((const void *)k_update_s, vitems), dim3(32, 8), st_, d, d32_, ri32_, p32_,
                   q32_, lst0, cnt0, sc_, part_, ticket_);
        tk_.launches += 4;
        iter_launches32_ = tk_.launches - l0;
        if (copy_slots) cudaMemcpyAsync(sc_host_, sc_, 8 * S_NSLOTS, cudaMemcpyDeviceToHost, st_);
        return;
    }
    if (prm_.smoother == 2 || prm_.smoother == 3)
        vcycle<float, float, __half, __half>(st_, tk_, lev_dims_, c32_, c16s0_, c16_, z32_, ri32_, x32_, b32_, ts,
                                             prm_, false, nullptr, tail_lt_, tail_smem_, tail_nc_, tail_op_.data());
    else
        vcycle<float, float, __half, float>(st_, tk_, lev_dims_, c32_, c32_, c16_, z32_, ri32_, x32_, b32_, ts,
                                            prm_, false, nullptr, tail_lt_, tail_smem_, tail_nc_, tail_op_.data());
    const uint8_t *nr = nullptr;
    launch_pdl(k_dot_rz<float>, kMaxRedBlocks, dim3(32, 8), st_, d, nr, ri32_, z32_, q32_, 1, sc_, part_, ticket_);
    launch_pdl(k_xpby<float>, kMaxRedBlocks, dim3(32, 8), st_, d, nr, z32_, p32_, sc_);
    apply_dot32(st_, d, c32_, p32_, q32_, sc_, part_, ticket_);
    launch_pdl(k_update<float>, kMaxRedBlocks, dim3(32, 8), st_, d, nr, d32_, ri32_, p32_, q32_, sc_, part_, ticket_);
    tk_.launches += 4;
    iter_launches32_ = tk_.launches - l0;
    if (copy_slots) cudaMemcpyAsync(sc_host_, sc_, 8 * S_NSLOTS, cudaMemcpyDeviceToHost, st_);
}

// Control of the device-side inner loop (one thread, the last node of the loop body): counts the iteration and
// continues while no breakdown or timed-out wait was flagged, ||r||^2 is finite and above its target, the budget
// is not spent, and (mixed form) the iteration is not stagnating -- the host loop's tests: two consecutive
// iterations each leaving more than a quarter of ||r||^2 end the inner solve (FP32 stagnation; the refinement
// takes over).
__global__ void k_inner_ctl(double *sc, cudaGraphConditionalHandle h) {
    const double it = sc[S_IT] + 1.0;
    sc[S_IT] = it;
    const double rin = sc[S_RR];
    const double slow = (sc[S_STAG] != 0.0 && rin > 0.25 * sc[S_RPREV]) ? sc[S_SLOW] + 1.0 : 0.0;
    sc[S_SLOW] = slow;
    sc[S_RPREV] = rin;
    const bool go = sc[S_AUX0] == 0.0 && sc[S_ERR] == 0.0 && isfinite(rin) && rin > sc[S_TOL2] &&
                    it < sc[S_BUDGET] && slow < 2.0;
    cudaGraphSetConditional(h, go ? 1u : 0u);
}

cudaError_t MGSolver::build_loop(bool mixed) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) return e;
    cudaGraphConditionalHandle h;
    cudaGraphNodeParams cp = {};
    if ((e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault)) == cudaSuccess) {
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp);
    }
    if (e == cudaSuccess) {
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        const long long before = tk_.launches;
        e = cudaStreamBeginCaptureToGraph(st_, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            if (mixed)
                enqueue_iter32(false);
            else
                enqueue_iter64(false);
            k_inner_ctl<<<1, 1, 0, st_>>>(sc_, h);
            e = cudaStreamEndCapture(st_, &body);
        }
        tk_.launches = before;  // counted per iteration after each loop
    }
    cudaGraphExec_t &ge = mixed ? g_loop32_ : g_loop64_;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
    if (e != cudaSuccess) ge = nullptr;
    cudaGraphDestroy(g);
    return e;
}

// Runs inner iterations until the loop's tests stop it (at least one; budget > 0), from the recurrence state
// already on the device.  One graph launch and one read-back when the device-side loop is available, else one
// graph launch (or direct launches) and one read-back per iteration.
cudaError_t MGSolver::inner_loop(bool mixed, int budget, double tol2, double rr, int &iters) {
    cudaError_t e;
    iters = 0;
    cudaGraphExec_t *ge = nullptr;
    if (prm_.use_graph && !prm_.profile && loop_ok_) {
        // same configuration key as run_iter's graphs (it destroys these as well when the key changes)
        if ((e = run_iter_prepare()) != cudaSuccess) return e;
        ge = mixed ? &g_loop32_ : &g_loop64_;
        if (!*ge && build_loop(mixed) != cudaSuccess) {
            cudaGetLastError();
            // a rejected tail launch invalidates the capture: once more without the tail, else the host loop
            if (!(drop_tail() && run_iter_prepare() == cudaSuccess && build_loop(mixed) == cudaSuccess)) {
                cudaGetLastError();
                loop_ok_ = false;  // the host-driven loop below
                ge = nullptr;
            }
        }
    }
    if (ge && *ge) {
        // S_IT, S_TOL2, S_BUDGET, S_RPREV, S_SLOW, S_STAG
        const double st[6] = {0.0, tol2, (double)budget, rr, 0.0, mixed ? 1.0 : 0.0};
        cudaMemcpyAsync(sc_ + S_IT, st, sizeof(st), cudaMemcpyHostToDevice, st_);
        if ((e = cudaGraphLaunch(*ge, st_)) != cudaSuccess) return e;
        if ((e = read_slots()) != cudaSuccess) return e;
        iters = (int)sc_host_[S_IT];
        tk_.launches += (long long)iters * ((mixed ? iter_launches32_ : iter_launches64_) + 1);
        return cudaSuccess;
    }
    double rprev = rr;
    int slow = 0;
    const int every = prm_.check_every > 0 ? prm_.check_every : 1;
    while (iters < budget) {
        for (int s = 0; s < every && iters < budget; s++, iters++)
            if ((e = run_iter(mixed)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(st_)) != cudaSuccess) return e;
        const double rin = sc_host_[S_RR];
        if (sc_host_[S_AUX0] != 0) break;
        if (rin <= tol2 || !std::isfinite(rin)) break;
        if (!mixed) continue;
        // FP32 stagnation: two consecutive iterations reducing ||r|| by less than 2x -> refine in FP64
        slow = (rin > 0.25 * rprev) ? slow + 1 : 0;
        rprev = rin;
        if (slow >= 2) break;
    }
    return cudaSuccess;
}

// The captured graphs depend on the smoothing configuration: drop them when it changed.
cudaError_t MGSolver::run_iter_prepare() {
    const long long key = (long long)prm_.pre | ((long long)prm_.post << 8) | ((long long)prm_.coarse_sweeps << 16) |
                          ((long long)prm_.flexible << 32) | ((long long)prm_.smoother << 33) |
                          ((long long)prm_.coarse_pre << 36) | ((long long)prm_.coarse_post << 44) |
                          ((long long)tail_nc_ << 52);
    if (key != graph_key_) destroy_graphs();
    graph_key_ = key;
    return cudaSuccess;
}

cudaError_t MGSolver::run_iter(bool mixed) {
    cudaError_t e;
    tk_.prof = prm_.profile;
    if (!prm_.use_graph || prm_.profile) {
        if (mixed)
            enqueue_iter32();
        else
            enqueue_iter64();
        drop_tail();  // this iteration ran the separate kernels in its place
        return cudaGetLastError();
    }
    run_iter_prepare();
    cudaGraphExec_t &ge = mixed ? g_iter32_ : g_iter64_;
    if (!ge) {
        cudaGraph_t g;
        const long long before = tk_.launches;
        e = cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        if (mixed)
            enqueue_iter32();
        else
            enqueue_iter64();
        e = cudaStreamEndCapture(st_, &g);
        if (e != cudaSuccess) {
            tk_.launches = before;
            if (!drop_tail()) return e;
            cudaGetLastError();
            return run_iter(mixed);  // captured again without the tail
        }
        e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        tk_.launches = before;  // counted at replay
        if (e != cudaSuccess) {
            ge = nullptr;
            return e;
        }
    }
    tk_.launches += mixed ? iter_launches32_ : iter_launches64_;
    return cudaGraphLaunch(ge, st_);
}

cudaError_t MGSolver::read_slots() {
    cudaMemcpyAsync(sc_host_, sc_, 8 * S_NSLOTS, cudaMemcpyDeviceToHost, st_);
    const cudaError_t e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return e;
    if (sc_host_[S_ERR] != 0) {
        last_error = "a smoother's TMA load did not arrive within its bounded wait";
        return cudaErrorLaunchTimeout;
    }
    return cudaSuccess;
}

cudaError_t MGSolver::solve(bool x_is_zero, SolveResult &res) {
    res = SolveResult{};
    res.levels = (int)lev_dims_.size();
    tk_.prof = prm_.profile;
    cudaError_t e = prm_.precision == 0 ? solve64(x_is_zero, res) : solve_mixed(x_is_zero, res);
    if (e != cudaSuccess) return e;
    if (prm_.profile) {
        e = cudaStreamSynchronize(st_);
        if (e != cudaSuccess) return e;
        tk_.collect(res.smooth_ms, res.smooth_launches, res.smooth_bytes);
    }
    return cudaSuccess;
}

cudaError_t MGSolver::solve64(bool x_is_zero, SolveResult &res) {
    const Dims &d = lev_dims_[0];
    const long long n = d.n;
    int xpb;
    const dim3 tg = tile_grid(d, xpb, kStencilBlocks);
    cudaError_t e;
    if (x_is_zero) {
        cudaMemsetAsync(x_, 0, 8 * n, st_);
        k_cast_rhs<double><<<kMaxRedBlocks, dim3(32, 8), 0, st_>>>(n, b_, r_, S_RR, S_BB, sc_, part_, ticket_);
    } else {
        // r = b - A x, (r,r), (b,b)
        k_residual64<double><<<tg, dim3(32, 8), 0, st_>>>(d, xpb, c64_[0], x_, b_, r_, 0, S_RR, S_BB, sc_, part_,
                                                          ticket_, 0, rows64_ ? rows_[0] : nullptr);
    }
    tk_.launches++;
    cudaMemsetAsync(p_, 0, 8 * n, st_);
    cudaMemsetAsync(q_, 0, 8 * n, st_);
    {
        double init[S_NSLOTS] = {0};
        // S_RHO = 1 so that the first beta multiplies a zero p; ALPHA = 0 for the flexible form
        init[S_RHO] = 1.0;
        // keep RR/BB computed above: copy only the first 4 slots and ALPHA/BETA/AUX0
        cudaMemcpyAsync(sc_ + S_RHO, &init[S_RHO], 8 * 4, cudaMemcpyHostToDevice, st_);
        cudaMemcpyAsync(sc_ + S_ALPHA, &init[S_ALPHA], 8 * 3, cudaMemcpyHostToDevice, st_);
    }
    if ((e = read_slots()) != cudaSuccess) return e;
    const double bb = sc_host_[S_BB];
    res.bnorm = std::sqrt(bb);
    if (bb == 0.0) {  // amgcl returns x = 0 for a zero right-hand side
        cudaMemsetAsync(x_, 0, 8 * n, st_);
        res.converged = true;
        res.relres = 0;
        return cudaStreamSynchronize(st_);
    }
    const double tol2 = prm_.tol * prm_.tol * bb;
    double rr = sc_host_[S_RR];
    if (rr <= tol2) {
        res.converged = true;
        res.relres = std::sqrt(rr / bb);
        return cudaSuccess;
    }
    int it = 0;
    if ((e = inner_loop(false, prm_.max_iters, tol2, rr, it)) != cudaSuccess) return e;
    rr = sc_host_[S_RR];
    if (sc_host_[S_AUX0] != 0) res.breakdown = true;
    if (sc_host_[S_ERR] != 0) {
        last_error = "a smoother's TMA load did not arrive within its bounded wait";
        return cudaErrorLaunchTimeout;
    }
    res.iters = it;
    res.relres = std::sqrt(rr / bb);
    res.converged = rr <= tol2;
    return cudaSuccess;
}

cudaError_t MGSolver::solve_mixed(bool x_is_zero, SolveResult &res) {
    const Dims &d = lev_dims_[0];
    const long long n = d.n;
    int xpb;
    const dim3 tg = tile_grid(d, xpb, kStencilBlocks);
    cudaError_t e;
    if (x_is_zero) cudaMemsetAsync(x_, 0, 8 * n, st_);
    double bb = -1, rr = 0;
    int total_inner = 0, outer = 0;
    const int max_outer = 30;
    bool x_zero = x_is_zero, stalled = false;
    while (true) {
        // outer FP64 residual, cast to the FP32 inner right-hand side
        if (x_zero) {
            if (split0_)
                k_cast_rhs_s<<<kMaxRedBlocks, dim3(32, 8), 0, st_>>>(d, b_, r32_, S_AUX1, S_BB, sc_, part_, ticket_);
            else
                k_cast_rhs<float><<<kMaxRedBlocks, dim3(32, 8), 0, st_>>>(n, b_, r32_, S_AUX1, S_BB, sc_, part_,
                                                                           ticket_);
            x_zero = false;
        } else {
            k_residual64<float><<<tg, dim3(32, 8), 0, st_>>>(d, xpb, c64_[0], x_, b_, r32_, 0, S_AUX1,
                                                             bb < 0 ? S_BB : -1, sc_, part_, ticket_, split0_ ? 1 : 0,
                                                             split0_ ? rows_[0] : nullptr);
        }
        tk_.launches++;
        if ((e = read_slots()) != cudaSuccess) return e;
        rr = sc_host_[S_AUX1];
        if (bb < 0) {
            bb = sc_host_[S_BB];
            res.bnorm = std::sqrt(bb);
            if (bb == 0.0) {
                cudaMemsetAsync(x_, 0, 8 * n, st_);
                res.converged = true;
                return cudaStreamSynchronize(st_);
            }
        }
        const double rel = std::sqrt(rr / bb);
        if (rel <= prm_.tol || !std::isfinite(rr) || outer >= max_outer || total_inner >= prm_.max_iters) break;
        // inner FCG on A32 d = r32, d = 0
        double tau = 0.5 * prm_.tol / rel;
        if (tau < prm_.inner_tol) tau = prm_.inner_tol;
        if (tau > 0.5) tau = 0.5;
        const double in_tol2 = tau * tau * rr;
        cudaMemsetAsync(d32_, 0, 4 * n, st_);
        cudaMemsetAsync(p32_, 0, 4 * n, st_);
        cudaMemsetAsync(q32_, 0, 4 * n, st_);
        {
            double init[4] = {1.0, 0.0, 0.0, 0.0};
            cudaMemcpyAsync(sc_ + S_RHO, init, 8, cudaMemcpyHostToDevice, st_);
            cudaMemcpyAsync(sc_ + S_ALPHA, init + 1, 8 * 3, cudaMemcpyHostToDevice, st_);
        }
        if (learned_ && !stalled) {
            if ((e = learned_step(rr, outer == 0, stalled, res)) != cudaSuccess) return e;
            if (outer == 0) res.guess_relres = std::sqrt(sc_host_[S_RR] / bb);
        }
        int it = 0;
        const int budget = prm_.max_iters - total_inner;
        // the inner residual after a learned step (it is the FP64 residual otherwise)
        const double rin0 = (learned_ && res.learned_steps > 0 && !stalled) ? sc_host_[S_RR] : rr;
        if (budget > 0 && (e = inner_loop(true, budget, in_tol2, rin0, it)) != cudaSuccess) return e;
        if (sc_host_[S_ERR] != 0) {
            last_error = "a smoother's TMA load did not arrive within its bounded wait";
            return cudaErrorLaunchTimeout;
        }
        total_inner += it;
        if (split0_)
            k_ir_update_s<<<row_grid((const void *)k_ir_update_s, (long long)d.nx * d.ny * (((d.nz >> 1) + 31) / 32)),
                            dim3(32, 8), 0, st_>>>(d, x_, d32_, list_[0], count_);
        else
            k_ir_update<<<flat_grid(n), 256, 0, st_>>>(n, x_, d32_);
        tk_.launches++;
        outer++;
        if (sc_host_[S_AUX0] != 0) {
            res.breakdown = true;
            // one more residual evaluation happens at the loop head; stop after it
        }
        if (it == 0) break;
    }
    res.iters = total_inner;
    res.outer = outer;
    res.relres = std::sqrt(rr / bb);
    res.converged = res.relres <= prm_.tol;
    if (res.guess_relres >= 0 && guess_yay_ > 0 && std::isfinite(guess_yb_)) {
        // A-norm error of the guess relative to zero: 1 - (y,b)^2 / ((y,Ay) (b,x*)), x* = the solution
        k_dot_dd<<<kMaxRedBlocks, dim3(32, 8), 0, st_>>>(n, b_, x_, S_AUX2, sc_, part_, ticket_);
        tk_.launches++;
        if ((e = read_slots()) != cudaSuccess) return e;
        const double bx = sc_host_[S_AUX2];
        if (bx > 0) res.guess_energy = 1.0 - guess_yb_ * guess_yb_ / (guess_yay_ * bx);
    }
    return cudaGetLastError();
}

// One learned correction step at the start of an inner solve (d32 = 0, p32 = q32 = 0, r32 = the inner residual,
// rr its squared norm): y = N(r) on the active cells, q = A y, gamma = (y, r) / (y, q), d32 = gamma y,
// r32 -= gamma q.  p32 and q32 serve as scratch and are cleared again, with the recurrence's slots.
cudaError_t MGSolver::learned_step(double rr, bool first, bool &stalled, SolveResult &res) {
    const Dims &d = lev_dims_[0];
    const long long n = d.n;
    cudaError_t e;
    if ((e = lrn_r_.ensure(4 * (size_t)n)) != cudaSuccess) return e;
    if ((e = lrn_y_.ensure(4 * (size_t)n)) != cudaSuccess) return e;
    float *rn = (float *)lrn_r_.get(), *yn = (float *)lrn_y_.get();
    if (split0_)
        k_split_to_vec<<<split_rows_grid(d), dim3(32, 8), 0, st_>>>(d, r32_, rn);
    else
        cudaMemcpyAsync(rn, r32_, 4 * (size_t)n, cudaMemcpyDeviceToDevice, st_);
    if ((e = learned_->predict(rn, rr, yn)) != cudaSuccess) return e;
    k_mask_active<<<flat_grid(n), 256, 0, st_>>>(n, c64_[0].D, yn);
    // (r, y) and (y, A y): q32 = A y (p32 = y), then the flexible beta's dot kernel on (r, y, A y)
    if (split0_) {
        k_vec_to_split<<<split_rows_grid(d), dim3(32, 8), 0, st_>>>(d, yn, p32_);
        apply_dot32s(st_, d, c32_, p32_, q32_, list_[0], count_, crow_, sc_, part_, ticket_);
        const long long vitems = split_items(2LL * d.nx * d.ny, d.nz >> 3);
        k_dot_rz_s<<<row_grid((const void *)k_dot_rz_s, vitems), dim3(32, 8), 0, st_>>>(
            d, r32_, p32_, q32_, list_[0], count_, 1, sc_, part_, ticket_);
    } else {
        cudaMemcpyAsync(p32_, yn, 4 * (size_t)n, cudaMemcpyDeviceToDevice, st_);
        apply_dot32(st_, d, c32_, p32_, q32_, sc_, part_, ticket_);
        k_dot_rz<float><<<kMaxRedBlocks, dim3(32, 8), 0, st_>>>(d, (const uint8_t *)nullptr, r32_, p32_, q32_, 1, sc_,
                                                                 part_, ticket_);
    }
    k_learned_update<<<kMaxRedBlocks, dim3(32, 8), 0, st_>>>(n, d32_, r32_, p32_, q32_, sc_, part_, ticket_);
    tk_.launches += 6;
    cudaMemsetAsync(p32_, 0, 4 * (size_t)n, st_);
    cudaMemsetAsync(q32_, 0, 4 * (size_t)n, st_);
    {
        double init[4] = {1.0, 0.0, 0.0, 0.0};
        cudaMemcpyAsync(sc_ + S_RHO, init, 8, cudaMemcpyHostToDevice, st_);
        cudaMemcpyAsync(sc_ + S_ALPHA, init + 1, 8 * 3, cudaMemcpyHostToDevice, st_);
    }
    if ((e = read_slots()) != cudaSuccess) return e;
    const double ry = sc_host_[S_LRY], yay = sc_host_[S_LYAY], rr1 = sc_host_[S_RR];
    res.learned_steps++;
    if (first) {
        guess_yb_ = ry;  // the first step is from r = b: (y, b)
        guess_yay_ = yay;
    }
    // a step that is not finite was not taken (gamma = 0); one that removes less than 10% of ||r|| stalls
    if (!std::isfinite(rr1) || !(rr1 <= 0.81 * rr)) {
        stalled = true;
        res.fallback = true;
    }
    return cudaSuccess;
}

cudaError_t MGSolver::true_relres(bool skip0, double &relres, double &bnorm) {
    const Dims &d = lev_dims_[0];
    int xpb;
    const dim3 tg = tile_grid(d, xpb, kStencilBlocks);
    k_residual64<double><<<tg, dim3(32, 8), 0, st_>>>(d, xpb, c64_[0], x_, b_, (double *)nullptr, skip0 ? 1 : 0,
                                                      S_AUX1, S_AUX2, sc_, part_, ticket_, 0,
                                                      (split0_ || rows64_) ? rows_[0] : nullptr);
    tk_.launches++;
    cudaError_t e = read_slots();
    if (e != cudaSuccess) return e;
    const double rr = sc_host_[S_AUX1], bb = sc_host_[S_AUX2];
    bnorm = std::sqrt(bb);
    relres = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
    return cudaSuccess;
}

cudaError_t MGSolver::shift_to_zero_at_origin() {
    const long long n = lev_dims_[0].n;
    k_shift<<<flat_grid(n), 256, 0, st_>>>(n, x_);
    tk_.launches++;
    cudaMemsetAsync(x_, 0, 8, st_);
    return cudaGetLastError();
}

}  // namespace sf
