// sf_internal.cuh -- shared device-side definitions of the sm_103a solver library.
//
// Grid layout is the reference's (core/Grid.h:28): cell (i,j,k) -> k + nz*(j + ny*i), z fastest.  Every
// multigrid level stores its 7-point operator in "face-coefficient" form on a dense cell grid:
//   ax[c] = coupling across the lower x-face of cell c (between c - e_x and c); 0 on the grid boundary and
//           wherever either cell is inactive (air for the pressure solve).  Likewise ay, az.
//   (A v)_c = D_c v_c - sum over the 6 faces of (coupling * v_neighbour),  D_c = sum of the 6 couplings + dex_c
//   dex_c  = diagonal excess (ghost-fluid Dirichlet terms, the isolated-cell 1); D_c == 0 marks an inactive cell.
#pragma once
#include <type_traits>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "sf_convert.cuh"

#include <cstdint>

namespace sf {

struct Dims {
    int nx, ny, nz;
    long long n;
};

static inline Dims make_dims(int nx, int ny, int nz) { return Dims{nx, ny, nz, (long long)nx * ny * nz}; }

// An FP64 value stored at precision T: float through the integer-pipe conversion (sf_convert.cuh), double as is.
template <class T>
__device__ __forceinline__ T to_prec(double v) {
    if constexpr (std::is_same<T, float>::value)
        return f64_to_f32(v);
    else
        return (T)v;
}

__host__ __device__ __forceinline__ long long cid(const Dims &d, int i, int j, int k) {
    return (long long)k + (long long)d.nz * ((long long)j + (long long)d.ny * i);
}

// Operator storage of one level.  C = double | float | __half.
//   double: dg = D (full diagonal), invd = 1/D (0 where inactive), dex kept for coarsening.
//   float/__half: dg = dex, D is recomputed from the stored couplings so that the stored operator keeps
//   exact row sums (a Neumann row stays singular, a Dirichlet row stays dominant) whatever the rounding.
//   __half values are stored multiplied by `scale` (a power of two) and multiplied by `unscale` on load.
template <class C>
struct Coef {
    C *ax, *ay, *az;
    C *dex;
    double *D, *invd;  // double levels only
    float scale, unscale;
};

// Colour-split index of cell (i, j, k) (the mixed form's level 0 with smoother 3): colour (i + j + k) & 1 selects
// the half of the array, row (i, j) holds its nz / 2 cells of that colour in k order.
__host__ __device__ __forceinline__ long long split_index(const Dims &d, int i, int j, int k) {
    const int col = (i + j + k) & 1;
    return (long long)col * (d.n >> 1) + ((long long)i * d.ny + j) * (d.nz >> 1) + (k >> 1);
}

// Where the assembly kernels also write the split level 0's FP32 and FP16 operator copies and its row flags
// (1 on a row with an active cell; cleared by the launcher first).  rows == nullptr: not written.
struct SplitOut {
    Coef<float> c32;
    Coef<__half> c16;
    uint8_t *rows;
};

__device__ __forceinline__ double ldv(const double *p, long long i) { return p[i]; }
__device__ __forceinline__ float ldv(const float *p, long long i) { return p[i]; }
__device__ __forceinline__ float ldv(const __half *p, long long i) { return __half2float(p[i]); }

template <class C>
struct Acc;  // arithmetic type of a coefficient storage type
template <>
struct Acc<double> {
    using T = double;
};
template <>
struct Acc<float> {
    using T = float;
};
template <>
struct Acc<__half> {
    using T = float;
};

__device__ __forceinline__ void stv(double *p, long long i, double v) { p[i] = v; }
__device__ __forceinline__ void stv(float *p, long long i, float v) { p[i] = v; }
__device__ __forceinline__ void stv(__half *p, long long i, float v) { p[i] = __float2half_rn(v); }

// Sum of coupling * x over the 6 faces of cell (i,j,k) and (optionally) the sum of the couplings.
// Returned values are already unscaled.
template <class T, class C, bool SUMA>
__device__ __forceinline__ T nbsum(const Dims &d, const Coef<C> &cf, const T *__restrict__ x, int i, int j,
                                   int k, long long c, T &suma) {
    using R = typename Acc<C>::T;
    const long long sx = (long long)d.ny * d.nz, sy = d.nz;
    R s = 0, sa = 0;
    if (i > 0) {
        R a = ldv(cf.ax, c);
        s += a * (R)x[c - sx];
        if (SUMA) sa += a;
    }
    if (i < d.nx - 1) {
        R a = ldv(cf.ax, c + sx);
        s += a * (R)x[c + sx];
        if (SUMA) sa += a;
    }
    if (j > 0) {
        R a = ldv(cf.ay, c);
        s += a * (R)x[c - sy];
        if (SUMA) sa += a;
    }
    if (j < d.ny - 1) {
        R a = ldv(cf.ay, c + sy);
        s += a * (R)x[c + sy];
        if (SUMA) sa += a;
    }
    if (k > 0) {
        R a = ldv(cf.az, c);
        s += a * (R)x[c - 1];
        if (SUMA) sa += a;
    }
    if (k < d.nz - 1) {
        R a = ldv(cf.az, c + 1);
        s += a * (R)x[c + 1];
        if (SUMA) sa += a;
    }
    if (sizeof(C) == 2) {
        s *= (R)cf.unscale;
        sa *= (R)cf.unscale;
    }
    suma = (T)sa;
    return (T)s;
}

// Diagonal of cell c given the (unscaled) sum of its couplings.
template <class C>
__device__ __forceinline__ typename Acc<C>::T diag_of(const Coef<C> &cf, long long c, typename Acc<C>::T suma) {
    if (sizeof(C) == 8) return (typename Acc<C>::T)cf.D[c];
    typename Acc<C>::T e = ldv(cf.dex, c);
    if (sizeof(C) == 2) e *= cf.unscale;
    return suma + e;
}

// --------------------------------------------------------------------------------------------------------
// Deterministic reductions: each block writes its partial sums to `part`, the last block to finish (atomic
// ticket) sums the partials in block order and runs a finaliser.  Same inputs -> same bits.
// --------------------------------------------------------------------------------------------------------
constexpr int kRedThreads = 256;

template <int K>
__device__ __forceinline__ void warp_sum(double (&v)[K]) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int q = 0; q < K; q++) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
}

// Fixed-order tree sum of one value per thread over a kRedThreads block; result valid in tid 0.
template <int K>
__device__ __forceinline__ void block_sum(double (&acc)[K], int tid) {
    __shared__ double sh2[K][kRedThreads];
#pragma unroll
    for (int q = 0; q < K; q++) sh2[q][tid] = acc[q];
    __syncthreads();
    for (int s = kRedThreads / 2; s > 0; s >>= 1) {
        if (tid < s)
#pragma unroll
            for (int q = 0; q < K; q++) sh2[q][tid] += sh2[q][tid + s];
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < K; q++) acc[q] = sh2[q][0];
    __syncthreads();
}

constexpr int kRedGroup = 256;  // blocks per first-level group

// Warp sum of FP32 values as an unevaluated (hi, lo) pair of floats: each shuffle stage adds the partner's pair
// with the exact two-sum (Knuth), keeps the rounding error in lo and renormalises, so the sum carries about 48
// bits.  It runs on the FP32 pipe, which on this GPU issues 64 times as many lanes per clock as the FP64 pipe;
// lane 0 holds the warp's pair (converted to FP64 only in the block stage, by one thread).  Same fixed shuffle
// order as warp_sum, hence deterministic.
template <int K>
__device__ __forceinline__ void warp_sum_df(const float (&v)[K], float (&hi_out)[K], float (&lo_out)[K]) {
#pragma unroll
    for (int q = 0; q < K; q++) {
        float hi = v[q], lo = 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float bh = __shfl_down_sync(0xffffffffu, hi, o);
            const float bl = __shfl_down_sync(0xffffffffu, lo, o);
            const float sum = __fadd_rn(hi, bh);
            const float bb = __fsub_rn(sum, hi);
            const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(sum, bb)), __fsub_rn(bh, bb));
            const float l = __fadd_rn(__fadd_rn(lo, bl), err);
            hi = __fadd_rn(sum, l);
            lo = __fsub_rn(l, __fsub_rn(hi, sum));
        }
        hi_out[q] = hi;
        lo_out[q] = lo;
    }
}

// Deterministic grid-wide sum.  Blocks write partials; the last block of each group of kRedGroup blocks sums
// its group in block order; the last group to finish sums the group partials in group order.  Returns true in
// exactly one thread (linear thread 0 of that block) with `tot` holding the totals.  Blocks must have
// kRedThreads threads (any shape).  part: K * (nblk + ngroups) doubles; ticket: 1 + ngroups counters, zero on
// entry and re-armed on exit.  Per-thread values are doubles (warp stage in FP64) or floats (warp stage as a
// float pair, warp_sum_df); the block and grid stages are FP64.
template <int K, class V>
__device__ __forceinline__ bool grid_reduce(V (&v)[K], double *part, unsigned *ticket, double (&tot)[K]) {
    __shared__ double sh[K][kRedThreads / 32];
    __shared__ float shf[K][2][kRedThreads / 32];
    __shared__ bool last;
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nblk = gridDim.x * gridDim.y * gridDim.z;
    const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    const int ngroups = (nblk + kRedGroup - 1) / kRedGroup;
    const int grp = bid / kRedGroup;
    const int gsize = min(kRedGroup, nblk - grp * kRedGroup);
    double *gpart = part + (long long)K * nblk;
    const int lane = tid & 31, wid = tid >> 5;
    constexpr bool kFloat = std::is_same<V, float>::value;
    if constexpr (kFloat) {
        float hi[K], lo[K];
        warp_sum_df<K>(v, hi, lo);
        if (lane == 0)
#pragma unroll
            for (int q = 0; q < K; q++) {
                shf[q][0][wid] = hi[q];
                shf[q][1][wid] = lo[q];
            }
    } else {
        warp_sum<K>(v);
        if (lane == 0)
#pragma unroll
            for (int q = 0; q < K; q++) sh[q][wid] = v[q];
    }
    __syncthreads();
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < K; q++) {
            double b = 0;
            for (int w = 0; w < kRedThreads / 32; w++)
                b += kFloat ? ((double)shf[q][0][w] + (double)shf[q][1][w]) : sh[q][w];
            part[(long long)q * nblk + bid] = b;
        }
        __threadfence();
        const unsigned t = atomicAdd(&ticket[1 + grp], 1u);
        last = (t == (unsigned)gsize - 1);
    }
    __syncthreads();
    if (!last) return false;
    // last block of the group: sum the group's partials in block order
    __threadfence();
    double acc[K];
#pragma unroll
    for (int q = 0; q < K; q++)
        acc[q] = tid < gsize ? ((volatile double *)part)[(long long)q * nblk + grp * kRedGroup + tid] : 0.0;
    block_sum<K>(acc, tid);
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < K; q++) gpart[(long long)q * ngroups + grp] = acc[q];
        ticket[1 + grp] = 0u;
        __threadfence();
        const unsigned t = atomicAdd(&ticket[0], 1u);
        last = (t == (unsigned)ngroups - 1);
    }
    __syncthreads();
    if (!last) return false;
    // last group: sum the group partials in group order
    __threadfence();
#pragma unroll
    for (int q = 0; q < K; q++) acc[q] = 0;
    for (int g = tid; g < ngroups; g += kRedThreads)
#pragma unroll
        for (int q = 0; q < K; q++) acc[q] += ((volatile double *)gpart)[(long long)q * ngroups + g];
    block_sum<K>(acc, tid);
    if (tid != 0) return false;
#pragma unroll
    for (int q = 0; q < K; q++) tot[q] = acc[q];
    ticket[0] = 0u;
    return true;
}

// Scalar slots shared by the PCG kernels (device array of doubles).
enum Slot {
    S_RHO = 0,   // (r, z) of the current iteration
    S_RHONEW,    // (r, z) just computed
    S_ZQ,        // (z, q) for the flexible (Polak-Ribiere) beta
    S_PQ,        // (p, A p)
    S_RR,        // (r, r)
    S_BB,        // (b, b)
    S_ALPHA,
    S_BETA,
    S_AUX0,
    S_AUX1,
    S_AUX2,
    S_ERR,  // set to 1 by a kernel whose bounded wait timed out
    S_LGAMMA,  // learned step: gamma, (r, y), (y, A y)
    S_LRY,
    S_LYAY,
    S_IT,      // device-side inner loop: iterations run, (target residual)^2, iteration budget, last ||r||^2,
    S_TOL2,    // consecutive slow iterations
    S_BUDGET,
    S_RPREV,
    S_SLOW,
    S_STAG,    // 1: the loop ends on FP32 stagnation (mixed form), 0: no stagnation test (FP64 form)
    S_NSLOTS = 32
};

}  // namespace sf
