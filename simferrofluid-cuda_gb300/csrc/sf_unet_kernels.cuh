// sf_unet_kernels.cuh -- kernels of the learned solver's 3D U-Net (BF16 activations and weights, FP32
// accumulation), channels-last volumes [voxel][channel] on the solver's cell layout.
//
// Convolutions are implicit GEMMs: M = voxels, N = output channels, K = taps x input channels.  This file holds
// the warp-level tensor-core form (mma.sync m16n8k16): it is the training path (forward, input gradient,
// weight gradient) and the reference against which the tcgen05 forward kernel is checked.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "sf_internal.cuh"

namespace sf {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}
__device__ __forceinline__ uint32_t pack_raw(bf16 lo, bf16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// tap t of a 3x3x3 stencil: offsets (dx, dy, dz) in -1..1, t = 9 (dx+1) + 3 (dy+1) + (dz+1)
__device__ __forceinline__ void tap_off(int t, int taps, int &dx, int &dy, int &dz) {
    if (taps == 1) {
        dx = dy = dz = 0;
        return;
    }
    dx = t / 9 - 1;
    dy = (t / 3) % 3 - 1;
    dz = t % 3 - 1;
}

// --------------------------------------------------------------------------------------------------------
// y[v][co] = epi( sum_t sum_ci w[t][co][ci] x[v + off_t][ci] ), zero padding.
// Block: 4 warps, 128 voxels (each warp two m16 tiles); one tap's weights staged in shared memory.
// EPI 0: + bias, ReLU, BF16 out.  EPI 1: FP32 out, no bias (input gradient).
// --------------------------------------------------------------------------------------------------------
template <int CI, int CO, int EPI>
__global__ void __launch_bounds__(128) k_conv_mma(Dims d, const bf16 *__restrict__ x, const bf16 *__restrict__ w,
                                                  const float *__restrict__ bias, void *__restrict__ yout, int taps) {
    static_assert(CI % 16 == 0 && CO % 8 == 0, "channel counts");
    __shared__ __align__(16) bf16 ws[CO][CI + 8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, tq = lane & 3;
    const long long vbase = (long long)blockIdx.x * 128 + warp * 32;
    int ci_[4], cj_[4], ck_[4];
    bool ok[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const long long v = vbase + (r >> 1) * 16 + (r & 1) * 8 + g;
        ok[r] = v < d.n;
        const long long vv = ok[r] ? v : 0;
        ck_[r] = (int)(vv % d.nz);
        cj_[r] = (int)((vv / d.nz) % d.ny);
        ci_[r] = (int)(vv / ((long long)d.nz * d.ny));
    }
    float acc[2][CO / 8][4];
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int n = 0; n < CO / 8; n++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[m][n][q] = 0.f;

    for (int t = 0; t < taps; t++) {
        __syncthreads();
        for (int e = threadIdx.x; e < CO * CI / 8; e += 128) {
            const int co = e / (CI / 8), cc = e % (CI / 8);
            *reinterpret_cast<uint4 *>(&ws[co][cc * 8]) =
                *reinterpret_cast<const uint4 *>(w + ((long long)t * CO + co) * CI + cc * 8);
        }
        __syncthreads();
        int dx, dy, dz;
        tap_off(t, taps, dx, dy, dz);
        const uint32_t *src[4];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int ii = ci_[r] + dx, jj = cj_[r] + dy, kk = ck_[r] + dz;
            const bool in = ok[r] && ii >= 0 && ii < d.nx && jj >= 0 && jj < d.ny && kk >= 0 && kk < d.nz;
            src[r] = in ? reinterpret_cast<const uint32_t *>(x + cid(d, ii, jj, kk) * CI) : nullptr;
        }
#pragma unroll
        for (int c0 = 0; c0 < CI; c0 += 16) {
            uint32_t a[2][4];
#pragma unroll
            for (int m = 0; m < 2; m++) {
                const uint32_t *ra = src[2 * m], *rb = src[2 * m + 1];
                a[m][0] = ra ? ra[(c0 >> 1) + tq] : 0u;
                a[m][1] = rb ? rb[(c0 >> 1) + tq] : 0u;
                a[m][2] = ra ? ra[(c0 >> 1) + 4 + tq] : 0u;
                a[m][3] = rb ? rb[(c0 >> 1) + 4 + tq] : 0u;
            }
#pragma unroll
            for (int n = 0; n < CO / 8; n++) {
                const uint32_t *wr = reinterpret_cast<const uint32_t *>(&ws[n * 8 + g][c0]);
                const uint32_t b[2] = {wr[tq], wr[4 + tq]};
                mma16816(acc[0][n], a[0], b);
                mma16816(acc[1][n], a[1], b);
            }
        }
    }
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int hh = 0; hh < 2; hh++) {
            const long long v = vbase + m * 16 + hh * 8 + g;
            if (v >= d.n) continue;
#pragma unroll
            for (int n = 0; n < CO / 8; n++) {
                const int co = n * 8 + 2 * tq;
                float y0 = acc[m][n][2 * hh], y1 = acc[m][n][2 * hh + 1];
                if (EPI == 0) {
                    y0 = fmaxf(y0 + bias[co], 0.f);
                    y1 = fmaxf(y1 + bias[co + 1], 0.f);
                    reinterpret_cast<uint32_t *>(yout)[(v * CO + co) >> 1] = pack_bf16(y0, y1);
                } else {
                    reinterpret_cast<float2 *>(yout)[(v * CO + co) >> 1] = make_float2(y0, y1);
                }
            }
        }
}

// --------------------------------------------------------------------------------------------------------
// Weight gradient, partial over a voxel chunk: part[chunk][t][co][ci] = sum_{v in chunk} dy[v][co] x[v+off_t][ci]
// Block: 4 warps, one tap (blockIdx.y), one chunk of `vchunk` voxels (blockIdx.x).  M = co (m16 tiles), N = ci,
// K = voxels; warps split the m tiles and, when CO < 64, the voxels.
// --------------------------------------------------------------------------------------------------------
template <int CI, int CO>
__global__ void __launch_bounds__(128) k_wgrad_mma(Dims d, const bf16 *__restrict__ dy, const bf16 *__restrict__ x,
                                                   float *__restrict__ part, int taps, int vchunk) {
    constexpr int MT = CO / 16 > 0 ? CO / 16 : 1;  // m16 tiles (CO = 8 uses one padded tile)
    constexpr int WPM = 4 / (MT > 4 ? 4 : MT);    // warps per m tile
    static_assert(MT <= 4, "CO <= 64");
    __shared__ float red[4][CO > 16 ? 16 : CO][CI];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, tq = lane & 3;
    const int mt = warp % MT, ks = warp / MT;
    const int t = blockIdx.y;
    int dx, dy_, dz;
    tap_off(t, taps, dx, dy_, dz);
    const long long v_begin = (long long)blockIdx.x * vchunk;
    const long long v_end = min(v_begin + vchunk, d.n);
    float acc[CI / 8][4];
#pragma unroll
    for (int n = 0; n < CI / 8; n++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[n][q] = 0.f;
    const int co_a = mt * 16 + g, co_b = co_a + 8;
    const bool oka = co_a < CO, okb = co_b < CO;
    auto xs = [&](long long v, int ci) -> bf16 {  // x[v + off_t][ci], 0 outside
        if (v >= v_end) return __float2bfloat16(0.f);
        const int k = (int)(v % d.nz), j = (int)((v / d.nz) % d.ny), i = (int)(v / ((long long)d.nz * d.ny));
        const int ii = i + dx, jj = j + dy_, kk = k + dz;
        if (ii < 0 || ii >= d.nx || jj < 0 || jj >= d.ny || kk < 0 || kk >= d.nz) return __float2bfloat16(0.f);
        return x[cid(d, ii, jj, kk) * CI + ci];
    };
    auto dys = [&](long long v, int co, bool okc) -> bf16 {
        return (okc && v < v_end) ? dy[v * CO + co] : __float2bfloat16(0.f);
    };
    for (long long v0 = v_begin + 16LL * ks; v0 < v_end; v0 += 16LL * WPM) {
        const long long va = v0 + 2 * tq, vb = va + 8;
        uint32_t a[4];
        a[0] = pack_raw(dys(va, co_a, oka), dys(va + 1, co_a, oka));
        a[1] = pack_raw(dys(va, co_b, okb), dys(va + 1, co_b, okb));
        a[2] = pack_raw(dys(vb, co_a, oka), dys(vb + 1, co_a, oka));
        a[3] = pack_raw(dys(vb, co_b, okb), dys(vb + 1, co_b, okb));
#pragma unroll
        for (int n = 0; n < CI / 8; n++) {
            const int ci = n * 8 + g;
            const uint32_t b[2] = {pack_raw(xs(va, ci), xs(va + 1, ci)), pack_raw(xs(vb, ci), xs(vb + 1, ci))};
            mma16816(acc[n], a, b);
        }
    }
    // reduce the WPM warps of each m tile through shared memory (fixed order)
    for (int s = 0; s < WPM; s++) {
        if (ks == s) {
#pragma unroll
            for (int n = 0; n < CI / 8; n++)
#pragma unroll
                for (int hh = 0; hh < 2; hh++) {
                    const int row = g + 8 * hh, ci = n * 8 + 2 * tq;
                    if (mt * 16 + row >= CO) continue;
                    float *dst = &red[mt][row][ci];
                    if (s == 0) {
                        dst[0] = acc[n][2 * hh];
                        dst[1] = acc[n][2 * hh + 1];
                    } else {
                        dst[0] += acc[n][2 * hh];
                        dst[1] += acc[n][2 * hh + 1];
                    }
                }
        }
        __syncthreads();
    }
    float *out = part + ((long long)blockIdx.x * taps + t) * CO * CI;
    for (int e = threadIdx.x; e < CO * CI; e += 128) {
        const int co = e / CI, ci = e % CI;
        out[e] = red[co / 16][co % 16][ci];
    }
}

// sum over chunks (fixed order): dw[t][co][ci] = sum_c part[c][t][co][ci]
__global__ void k_reduce_chunks(const float *__restrict__ part, int chunks, long long m, float *__restrict__ out) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m; e += (long long)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int c = 0; c < chunks; c++) s += part[(long long)c * m + e];
        out[e] = s;
    }
}

// bias gradient partials: part[chunk][co] = sum_{v in chunk} dy[v][co].  256 threads per chunk: thread t sums
// channel t % C over the voxels v0 + t / C, v0 + t / C + 256 / C, ... (consecutive threads read consecutive
// channels), then the 256 / C lane sums of each channel are added in lane order: fixed order, deterministic.
template <int C>
__global__ void __launch_bounds__(256) k_bias_grad(long long n, const bf16 *__restrict__ dy, int vchunk,
                                                   float *__restrict__ part) {
    constexpr int LANES = 256 / C;
    __shared__ float red[256];
    const int c = threadIdx.x % C, l = threadIdx.x / C;
    const long long v0 = (long long)blockIdx.x * vchunk, v1 = min(v0 + vchunk, n);
    float s = 0.f;
    for (long long v = v0 + l; v < v1; v += LANES) s += __bfloat162float(dy[v * C + c]);
    red[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < C) {
        float t = 0.f;
        for (int k = 0; k < LANES; k++) t += red[k * C + threadIdx.x];
        part[(long long)blockIdx.x * C + threadIdx.x] = t;
    }
}

// --------------------------------------------------------------------------------------------------------
// elementwise / resampling kernels (channels-last)
// --------------------------------------------------------------------------------------------------------
// The grid operators below take one thread per (voxel, group of channels): 8 BF16 channels (16 bytes) or 4 FP32
// channels (16 bytes), on a launch grid of (ceil(nz x groups / 256), ny, nx) so that no 64-bit division is needed,
// consecutive threads touch consecutive 16-byte groups, and every sum keeps the order of a per-channel loop.
__device__ __forceinline__ void bf16x8_to_f32(const uint4 &u, float (&f)[8]) {
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int q = 0; q < 4; q++) {
        f[2 * q] = __uint_as_float(w[q] << 16);
        f[2 * q + 1] = __uint_as_float(w[q] & 0xffff0000u);
    }
}
__device__ __forceinline__ uint4 f32_to_bf16x8(const float (&f)[8]) {
    return make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]), pack_bf16(f[6], f[7]));
}

// 2x2x2 average pooling (children outside the grid count as absent, the sum is still divided by 8), BF16
template <int C>
__global__ void __launch_bounds__(256) k_pool(Dims d, Dims dc, const bf16 *__restrict__ x, bf16 *__restrict__ y) {
    constexpr int G = C / 8;
    const int t = blockIdx.x * 256 + threadIdx.x, K = t / G, g = t % G, J = blockIdx.y, I = blockIdx.z;
    if (K >= dc.nz) return;
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int i = 2 * I + (q & 1), j = 2 * J + ((q >> 1) & 1), k = 2 * K + (q >> 2);
        if (i < d.nx && j < d.ny && k < d.nz) {
            float f[8];
            bf16x8_to_f32(*reinterpret_cast<const uint4 *>(x + cid(d, i, j, k) * C + 8 * g), f);
#pragma unroll
            for (int e = 0; e < 8; e++) s[e] += f[e];
        }
    }
#pragma unroll
    for (int e = 0; e < 8; e++) s[e] *= 0.125f;
    *reinterpret_cast<uint4 *>(y + cid(dc, I, J, K) * C + 8 * g) = f32_to_bf16x8(s);
}

// y = up(xc) + s  (nearest parent), BF16
template <int C>
__global__ void __launch_bounds__(256) k_up_add(Dims d, Dims dc, const bf16 *__restrict__ xc,
                                                const bf16 *__restrict__ s, bf16 *__restrict__ y) {
    constexpr int G = C / 8;
    const int t = blockIdx.x * 256 + threadIdx.x, k = t / G, g = t % G, j = blockIdx.y, i = blockIdx.z;
    if (k >= d.nz) return;
    const long long v = cid(d, i, j, k);
    float a[8], b[8];
    bf16x8_to_f32(*reinterpret_cast<const uint4 *>(xc + cid(dc, i >> 1, j >> 1, k >> 1) * C + 8 * g), a);
    bf16x8_to_f32(*reinterpret_cast<const uint4 *>(s + v * C + 8 * g), b);
#pragma unroll
    for (int e = 0; e < 8; e++) a[e] += b[e];
    *reinterpret_cast<uint4 *>(y + v * C + 8 * g) = f32_to_bf16x8(a);
}

// dfine = dcoarse[parent] / 8 (+ dadd), FP32
template <int C>
__global__ void __launch_bounds__(256) k_pool_back(Dims d, Dims dc, const float *__restrict__ dcoarse,
                                                   const float *__restrict__ dadd, float *__restrict__ dfine) {
    constexpr int G = C / 4;
    const int t = blockIdx.x * 256 + threadIdx.x, k = t / G, g = t % G, j = blockIdx.y, i = blockIdx.z;
    if (k >= d.nz) return;
    const long long e = cid(d, i, j, k) * C + 4 * g;
    float4 r = *reinterpret_cast<const float4 *>(dcoarse + cid(dc, i >> 1, j >> 1, k >> 1) * C + 4 * g);
    r.x *= 0.125f;
    r.y *= 0.125f;
    r.z *= 0.125f;
    r.w *= 0.125f;
    if (dadd) {
        const float4 q = *reinterpret_cast<const float4 *>(dadd + e);
        r.x += q.x;
        r.y += q.y;
        r.z += q.z;
        r.w += q.w;
    }
    *reinterpret_cast<float4 *>(dfine + e) = r;
}

// dcoarse[V] = sum over the (in-grid) children of dfine, FP32
template <int C>
__global__ void __launch_bounds__(256) k_up_back(Dims d, Dims dc, const float *__restrict__ dfine,
                                                 float *__restrict__ dcoarse) {
    constexpr int G = C / 4;
    const int t = blockIdx.x * 256 + threadIdx.x, K = t / G, g = t % G, J = blockIdx.y, I = blockIdx.z;
    if (K >= dc.nz) return;
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int i = 2 * I + (q & 1), j = 2 * J + ((q >> 1) & 1), k = 2 * K + (q >> 2);
        if (i < d.nx && j < d.ny && k < d.nz) {
            const float4 f = *reinterpret_cast<const float4 *>(dfine + cid(d, i, j, k) * C + 4 * g);
            s.x += f.x;
            s.y += f.y;
            s.z += f.z;
            s.w += f.w;
        }
    }
    *reinterpret_cast<float4 *>(dcoarse + cid(dc, I, J, K) * C + 4 * g) = s;
}

// dpre = dpost * (post > 0), BF16 out (input of the MMA gradient kernels)
__global__ void k_relu_back(long long m, const float *__restrict__ dpost, const bf16 *__restrict__ post,
                            bf16 *__restrict__ dpre) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m; e += (long long)gridDim.x * blockDim.x)
        dpre[e] = __float2bfloat16(__bfloat162float(post[e]) > 0.f ? dpost[e] : 0.f);
}

// 1x1 head: out[v] = b + sum_c w[c] a[v][c]  (FP32 out), 16 channels read as two 16-byte groups
__global__ void __launch_bounds__(256) k_head_fwd(long long n, const bf16 *__restrict__ a, const float *__restrict__ w,
                                                  const float *__restrict__ b, float *__restrict__ out) {
    float wr[16];
#pragma unroll
    for (int c = 0; c < 16; c++) wr[c] = w[c];
    const float b0 = b[0];
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        float f0[8], f1[8];
        bf16x8_to_f32(*reinterpret_cast<const uint4 *>(a + v * 16), f0);
        bf16x8_to_f32(*reinterpret_cast<const uint4 *>(a + v * 16 + 8), f1);
        float s = b0;
#pragma unroll
        for (int c = 0; c < 8; c++) s += wr[c] * f0[c];
#pragma unroll
        for (int c = 0; c < 8; c++) s += wr[8 + c] * f1[c];
        out[v] = s;
    }
}

// head backward: da[v][c] = dout[v] w[c] (FP32); weight/bias partials per block chunk
__global__ void k_head_back(long long n, int C, const bf16 *__restrict__ a, const float *__restrict__ w,
                            const float *__restrict__ dout, float *__restrict__ da, int vchunk,
                            float *__restrict__ part /*[chunks][C+1]*/) {
    const long long v0 = (long long)blockIdx.x * vchunk, v1 = min(v0 + vchunk, n);
    __shared__ float sh[64][17];
    float acc[17];
    for (int c = 0; c <= C; c++) acc[c] = 0.f;
    for (long long v = v0 + threadIdx.x; v < v1; v += blockDim.x) {
        const float g = dout[v];
        for (int c = 0; c < C; c++) {
            da[v * C + c] = g * w[c];
            acc[c] += g * __bfloat162float(a[v * C + c]);
        }
        acc[C] += g;
    }
    for (int c = 0; c <= C; c++) sh[threadIdx.x][c] = acc[c];
    __syncthreads();
    if (threadIdx.x <= C) {
        float s = 0.f;
        for (int t = 0; t < (int)blockDim.x; t++) s += sh[t][threadIdx.x];
        part[(long long)blockIdx.x * (C + 1) + threadIdx.x] = s;
    }
}

// Adam on FP32 master weights, BF16 copy for the kernels
__global__ void k_adam(long long m, float *__restrict__ p, const float *__restrict__ gr, float *__restrict__ m1,
                       float *__restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2,
                       bf16 *__restrict__ pb) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m; e += (long long)gridDim.x * blockDim.x) {
        const float g = gr[e];
        const float a = b1 * m1[e] + (1.f - b1) * g;
        const float b = b2 * m2[e] + (1.f - b2) * g * g;
        m1[e] = a;
        m2[e] = b;
        const float v = p[e] - lr * (a / c1) / (sqrtf(b / c2) + eps);
        p[e] = v;
        if (pb) pb[e] = __float2bfloat16(v);
    }
}

// weights for the input gradient: wt[t'][ci][co] = w[taps-1-t'][co][ci] (mirrored taps, transposed channels)
__global__ void k_flip_weights(int taps, int CO, int CI, const float *__restrict__ w, bf16 *__restrict__ wt) {
    const long long m = (long long)taps * CO * CI;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m; e += (long long)gridDim.x * blockDim.x) {
        const int ci = (int)(e % CI), co = (int)((e / CI) % CO), t = (int)(e / ((long long)CI * CO));
        wt[((long long)(taps - 1 - t) * CI + ci) * CO + co] = __float2bfloat16(w[e]);
    }
}

// wp[9 dz + pr][co][ci] = w[3 pr + dz][co][ci]: the 27 taps reordered so that those of one z shift are
// consecutive (pr = 3 (dx + 1) + (dy + 1), dz the z shift + 1)
__global__ void k_taps_dz_major(long long m, int coci, const bf16 *__restrict__ w, bf16 *__restrict__ wp) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m; e += (long long)gridDim.x * blockDim.x) {
        const int tp = (int)(e / coci), r = (int)(e % coci);
        wp[e] = w[(long long)(3 * (tp % 9) + tp / 9) * coci + r];
    }
}

__global__ void k_f32_to_bf16(long long m, const float *__restrict__ a, bf16 *__restrict__ b) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m; e += (long long)gridDim.x * blockDim.x)
        b[e] = __float2bfloat16(a[e]);
}

}  // namespace sf
