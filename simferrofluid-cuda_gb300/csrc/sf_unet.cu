// sf_unet.cu -- host side of the learned solver's U-Net: parameters, workspaces, forward, backward, Adam.
#include <cmath>
#include <cstring>

#include <cudaTypedefs.h>

#include "sf_conv_tc.cuh"
#include "sf_unet.h"
#include "sf_unet_kernels.cuh"

namespace sf {

namespace {
constexpr int kVchunkMin = 512;

// launch grid of the per-voxel grid operators: (ceil(nz x groups / 256), ny, nx)
dim3 line_grid(const Dims &d, int groups) { return dim3((unsigned)((d.nz * groups + 255) / 256), d.ny, d.nx); }

int flat_blocks(long long n) {
    long long g = (n + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    return (int)(g < 1 ? 1 : g);
}

// cosine-loss dot products (o.t, o.o, t.t) with the deterministic grid reduction
__global__ void __launch_bounds__(256) k_cos_dots(long long n, const float *__restrict__ o, const float *__restrict__ t,
                                                  double *out, double *part, unsigned *ticket) {
    float a0 = 0, a1 = 0, a2 = 0;
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    for (long long c = blockIdx.x * 256LL + tid; c < n; c += (long long)gridDim.x * 256) {
        const float oc = o[c], tc = t[c];
        a0 += oc * tc;
        a1 += oc * oc;
        a2 += tc * tc;
    }
    float v[3] = {a0, a1, a2};
    double tot[3];
    if (grid_reduce<3>(v, part, ticket, tot)) {
        out[0] = tot[0];
        out[1] = tot[1];
        out[2] = tot[2];
    }
}

// d/do of 1 - (o.t)^2 / (|o|^2 |t|^2)
__global__ void k_cos_grad(long long n, const float *__restrict__ o, const float *__restrict__ t, const double *dots,
                           float *__restrict__ g) {
    const double ot = dots[0], oo = dots[1], tt = dots[2];
    const float ct = (float)(-2.0 * ot / (oo * tt));
    const float co = (float)(2.0 * ot * ot / (oo * oo * tt));
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        g[c] = ct * t[c] + co * o[c];
}

template <int CI, int CO>
void launch_conv(cudaStream_t st, int epi, const Dims &d, const bf16 *x, const bf16 *w, const float *b, void *y,
                 int taps) {
    const int blocks = (int)((d.n + 127) / 128);
    if (epi == 0)
        k_conv_mma<CI, CO, 0><<<blocks, 128, 0, st>>>(d, x, w, b, y, taps);
    else
        k_conv_mma<CI, CO, 1><<<blocks, 128, 0, st>>>(d, x, w, b, y, taps);
}

void conv_dispatch(cudaStream_t st, int ci, int co, int epi, const Dims &d, const bf16 *x, const bf16 *w,
                   const float *b, void *y, int taps) {
#define CASE(A, B)                                                  \
    if (ci == A && co == B) {                                       \
        launch_conv<A, B>(st, epi, d, x, w, b, y, taps);            \
        return;                                                     \
    }
    CASE(16, 16) CASE(16, 32) CASE(32, 16) CASE(32, 32) CASE(32, 64) CASE(64, 32) CASE(64, 64)
#undef CASE
}

// ------------------------------------------------------------------------------------------------ tcgen05 path
bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// The tcgen05 kernel takes 32 (z) x 4 (y) bricks: grids smaller than one brick use the warp-MMA kernel.
bool tc_shape_ok(int ci, int co, const Dims &d) {
    const bool ch = (ci == 16 || ci == 32 || ci == 64) && (co == 16 || co == 32 || co == 64);
    return ch && d.nz >= tc::kTileZ && d.ny >= tc::kTileY;
}

// MT tiles of 128 voxels per CTA (a 32 x 4 MT brick): the wide brick where the grid holds one along y, else one
// tile per CTA (the TMA box never extends past the grid along y).
template <int CI, int CO, int EPI, int MT>
cudaError_t launch_tc_mt(cudaStream_t st, const Dims &d, const bf16 *x, const bf16 *w, const float *b, void *y,
                         int *err) {
    auto enc = tensor_map_encoder();
    if (!enc || !aligned16(x) || !aligned16(w) || !aligned16(y)) return cudaErrorInvalidValue;
    CUtensorMap mx, mw;
    const cuuint64_t xd[4] = {(cuuint64_t)CI, (cuuint64_t)d.nz, (cuuint64_t)d.ny, (cuuint64_t)d.nx};
    const cuuint64_t xs[3] = {(cuuint64_t)CI * 2, (cuuint64_t)d.nz * CI * 2, (cuuint64_t)d.ny * d.nz * CI * 2};
    const cuuint32_t xb[4] = {8, tc::kTileZ, (cuuint32_t)(tc::kTileY * MT), 1};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    if (enc(&mx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16 *>(x), xd, xs, xb, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    const cuuint64_t wd[3] = {(cuuint64_t)CI, (cuuint64_t)CO, 27};
    const cuuint64_t ws[2] = {(cuuint64_t)CI * 2, (cuuint64_t)CO * CI * 2};
    const cuuint32_t wb[3] = {8, (cuuint32_t)CO, 1};
    if (enc(&mw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<bf16 *>(w), wd, ws, wb, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    using L = tc::Layout<CI, CO, MT>;
    cudaError_t e = cudaFuncSetAttribute(tc::k_conv_tc<CI, CO, EPI, MT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)L::kSmemBytes);
    if (e != cudaSuccess) return e;
    const long long tiles = (long long)((d.nz + tc::kTileZ - 1) / tc::kTileZ) *
                            ((d.ny + tc::kTileY * MT - 1) / (tc::kTileY * MT)) * d.nx;
    if (tiles > 0x7fffffffLL) return cudaErrorInvalidValue;
    tc::k_conv_tc<CI, CO, EPI, MT><<<(unsigned)tiles, 128, L::kSmemBytes, st>>>(mx, mw, d, b, y, err);
    return cudaGetLastError();
}

// 16 or 32 input channels, at most 32 output channels, on grids holding a 128 x 6 x (LX + 2) box: the z-line
// kernel (one halo'd box per z shift and chunk for nine taps)
bool line_shape_ok(int ci, int co, const Dims &d) {
    const int lx = ci == 16 ? tc::line_x<16>() : tc::line_x<32>();
    return (ci == 16 || ci == 32) && (co == 16 || co == 32) && d.nz >= tc::kLineZ && d.ny >= tc::kLineY + 2 &&
           d.nx >= lx + 2;
}

template <int CI, int CO, int EPI>
cudaError_t launch_tc_line(cudaStream_t st, const Dims &d, const bf16 *x, const bf16 *w, const float *b, void *y,
                           int *err) {
    auto enc = tensor_map_encoder();
    if (!enc || !aligned16(x) || !aligned16(w) || !aligned16(y)) return cudaErrorInvalidValue;
    CUtensorMap mx, mw;
    using L = tc::LineLayout<CI, CO>;
    const cuuint64_t xd[4] = {(cuuint64_t)CI, (cuuint64_t)d.nz, (cuuint64_t)d.ny, (cuuint64_t)d.nx};
    const cuuint64_t xs[3] = {(cuuint64_t)CI * 2, (cuuint64_t)d.nz * CI * 2, (cuuint64_t)d.ny * d.nz * CI * 2};
    // 16 channels (32 bytes) per box row, written in the 32-byte swizzled layout the MMA descriptors read
    const cuuint32_t xb[4] = {16, tc::kLineZ, tc::kLineY + 2, (cuuint32_t)L::LX + 2};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    if (enc(&mx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16 *>(x), xd, xs, xb, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    const cuuint64_t wd[3] = {(cuuint64_t)CI, (cuuint64_t)CO, 27};
    const cuuint64_t ws[2] = {(cuuint64_t)CI * 2, (cuuint64_t)CO * CI * 2};
    const cuuint32_t wb[3] = {16, (cuuint32_t)CO, 27};
    if (enc(&mw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<bf16 *>(w), wd, ws, wb, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(tc::k_conv_tc_line<CI, CO, EPI>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::kSmemBytes);
    if (e != cudaSuccess) return e;
    const long long nbricks = (long long)((d.nz + tc::kLineZ - 1) / tc::kLineZ) *
                              ((d.ny + tc::kLineY - 1) / tc::kLineY) * ((d.nx + L::LX - 1) / L::LX);
    const int grid = (int)(nbricks < 152 ? nbricks : 152);
    tc::k_conv_tc_line<CI, CO, EPI><<<grid, 192, L::kSmemBytes, st>>>(mx, mw, d, b, y, err);
    return cudaGetLastError();
}

// grids holding a 64 x 6 x 4 box: the 64-long z-line kernel (weights streamed per stage, taps ordered by z shift)
bool line64_shape_ok(int ci, int co, const Dims &d) {
    const bool ch = (ci == 16 || ci == 32 || ci == 64) && (co == 16 || co == 32 || co == 64);
    return ch && d.nz >= tc::kL64Z && d.ny >= tc::kL64Y + 2 && d.nx >= tc::kL64X + 2;
}

template <int CI, int CO, int EPI>
cudaError_t launch_tc_line64(cudaStream_t st, const Dims &d, const bf16 *x, const bf16 *wp, const float *b, void *y,
                             int *err) {
    auto enc = tensor_map_encoder();
    if (!enc || !aligned16(x) || !aligned16(wp) || !aligned16(y)) return cudaErrorInvalidValue;
    using L = tc::Line64Layout<CI, CO>;
    CUtensorMap mx, mw;
    const cuuint64_t xd[4] = {(cuuint64_t)CI, (cuuint64_t)d.nz, (cuuint64_t)d.ny, (cuuint64_t)d.nx};
    const cuuint64_t xs[3] = {(cuuint64_t)CI * 2, (cuuint64_t)d.nz * CI * 2, (cuuint64_t)d.ny * d.nz * CI * 2};
    const cuuint32_t xb[4] = {16, tc::kL64Z, tc::kL64Y + 2, tc::kL64X + 2};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    if (enc(&mx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16 *>(x), xd, xs, xb, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    const cuuint64_t wd[3] = {(cuuint64_t)CI, (cuuint64_t)CO, 27};
    const cuuint64_t ws[2] = {(cuuint64_t)CI * 2, (cuuint64_t)CO * CI * 2};
    const cuuint32_t wb[3] = {16, (cuuint32_t)CO, 9};
    if (enc(&mw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<bf16 *>(wp), wd, ws, wb, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(tc::k_conv_tc_line64<CI, CO, EPI>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::kSmemBytes);
    if (e != cudaSuccess) return e;
    const long long nbricks = (long long)((d.nz + tc::kL64Z - 1) / tc::kL64Z) *
                              ((d.ny + tc::kL64Y - 1) / tc::kL64Y) * ((d.nx + tc::kL64X - 1) / tc::kL64X);
    const int grid = (int)(nbricks < 152 ? nbricks : 152);
    tc::k_conv_tc_line64<CI, CO, EPI><<<grid, 192, L::kSmemBytes, st>>>(mx, mw, d, b, y, err);
    return cudaGetLastError();
}

template <int CI, int CO, int EPI>
cudaError_t launch_tc(cudaStream_t st, const Dims &d, const bf16 *x, const bf16 *w, const bf16 *wp, const float *b,
                      void *y, int *err) {
    if constexpr ((CI == 16 || CI == 32) && (CO == 16 || CO == 32))
        if (line_shape_ok(CI, CO, d)) return launch_tc_line<CI, CO, EPI>(st, d, x, w, b, y, err);
    if (wp && line64_shape_ok(CI, CO, d)) return launch_tc_line64<CI, CO, EPI>(st, d, x, wp, b, y, err);
    constexpr int MT = tc::tiles_per_cta<CI, CO>();
    if (d.ny >= tc::kTileY * MT) return launch_tc_mt<CI, CO, EPI, MT>(st, d, x, w, b, y, err);
    return launch_tc_mt<CI, CO, EPI, 1>(st, d, x, w, b, y, err);
}

// epi 0: forward (bias, ReLU, BF16 y); epi 1: input gradient (FP32 y, no bias).  wp: the weights with taps
// ordered by z shift (the 64-long z-line kernel), or nullptr
cudaError_t tc_dispatch(cudaStream_t st, int ci, int co, int epi, const Dims &d, const bf16 *x, const bf16 *w,
                        const bf16 *wp, const float *b, void *y, int *err) {
#define CASE(A, B)                                                                              \
    if (ci == A && co == B)                                                                     \
        return epi == 0 ? launch_tc<A, B, 0>(st, d, x, w, wp, b, y, err)                        \
                        : launch_tc<A, B, 1>(st, d, x, w, wp, b, y, err);
    CASE(16, 16) CASE(16, 32) CASE(32, 16) CASE(32, 32) CASE(32, 64) CASE(64, 32) CASE(64, 64)
#undef CASE
    return cudaErrorInvalidValue;
}

// The tcgen05 weight gradient takes 32 (z) x 4 (y) x 1 or 2 (x) bricks: every TMA box dimension within the grid's.
bool wgrad_tc_ok(int ci, int co, const Dims &d) {
    const bool ch = (ci == 16 || ci == 32 || ci == 64) && (co == 16 || co == 32 || co == 64);
    return ch && (d.nz + 7) / 8 >= 4 && d.ny >= 4 && d.nx >= 2;
}

// channel-major z-row copies of dY and of X with its three z shifts (k_to_chmajor), then k_wgrad_tc over all
// bricks; chunks receives the number of partial sums written to part
template <int CI, int CO>
cudaError_t launch_wgrad_tc(cudaStream_t st, const Dims &d, const bf16 *dy, const bf16 *x, bf16 *dyT, bf16 *xT,
                            float *part, long long part_cap, int &chunks, int *err) {
    auto enc = tensor_map_encoder();
    if (!enc || !aligned16(dyT) || !aligned16(xT) || !aligned16(part)) return cudaErrorInvalidValue;
    using L = tc::WgLayout<CI, CO>;
    const long long nzh = (d.nz + 7) / 8;
    const long long rows = nzh * d.nx * d.ny;  // 8-voxel z rows of one channel
    auto map5 = [&](CUtensorMap *m, const bf16 *base, int C) {
        const cuuint64_t dims[5] = {8, (cuuint64_t)C, (cuuint64_t)d.ny, (cuuint64_t)d.nx, (cuuint64_t)nzh};
        const cuuint64_t str[4] = {16, (cuuint64_t)C * 16, (cuuint64_t)d.ny * C * 16,
                                   (cuuint64_t)d.nx * d.ny * C * 16};
        const cuuint32_t box[5] = {8, (cuuint32_t)C, 4, (cuuint32_t)L::BX, 4};
        const cuuint32_t es[5] = {1, 1, 1, 1, 1};
        return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(base), dims, str, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    };
    CUtensorMap mdy, mx;
    if (!map5(&mdy, dyT, CO) || !map5(&mx, xT, 3 * CI)) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(tc::k_wgrad_tc<CI, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)L::kSmemBytes);
    if (e != cudaSuccess) return e;
    constexpr int NP = tc::wg_pairs_per_cta<CI>();
    constexpr int groups = (9 + NP - 1) / NP;
    const long long nbricks = (long long)((d.nz + 31) / 32) * ((d.ny + 3) / 4) * ((d.nx + L::BX - 1) / L::BX);
    long long G = 152 / groups;
    if (G > nbricks) G = nbricks;
    if (G * 27 * CO * CI > part_cap) G = part_cap / (27LL * CO * CI);
    if (G < 1) return cudaErrorInvalidValue;
    tc::k_to_chmajor<CO><<<flat_blocks(rows * CO), 256, 0, st>>>(d, 1, 0, dy, dyT);
    tc::k_to_chmajor<CI><<<flat_blocks(rows * CI), 256, 0, st>>>(d, 3, -1, x, xT);
    tc::k_wgrad_tc<CI, CO><<<dim3((unsigned)G, groups), 128, L::kSmemBytes, st>>>(mdy, mx, d, part, err);
    chunks = (int)G;
    return cudaGetLastError();
}

cudaError_t wgrad_tc_dispatch(cudaStream_t st, int ci, int co, const Dims &d, const bf16 *dy, const bf16 *x,
                              bf16 *dyT, bf16 *xT, float *part, long long part_cap, int &chunks, int *err) {
#define CASE(A, B)                                                                             \
    if (ci == A && co == B) return launch_wgrad_tc<A, B>(st, d, dy, x, dyT, xT, part, part_cap, chunks, err);
    CASE(16, 16) CASE(16, 32) CASE(32, 16) CASE(32, 32) CASE(32, 64) CASE(64, 32) CASE(64, 64)
#undef CASE
    return cudaErrorInvalidValue;
}

template <int CI, int CO>
void launch_wgrad(cudaStream_t st, const Dims &d, const bf16 *dy, const bf16 *x, float *part, int taps, int vchunk,
                  int chunks) {
    k_wgrad_mma<CI, CO><<<dim3(chunks, taps), 128, 0, st>>>(d, dy, x, part, taps, vchunk);
}

void wgrad_dispatch(cudaStream_t st, int ci, int co, const Dims &d, const bf16 *dy, const bf16 *x, float *part,
                    int taps, int vchunk, int chunks) {
#define CASE(A, B)                                                          \
    if (ci == A && co == B) {                                               \
        launch_wgrad<A, B>(st, d, dy, x, part, taps, vchunk, chunks);       \
        return;                                                             \
    }
    CASE(16, 16) CASE(16, 32) CASE(32, 16) CASE(32, 32) CASE(32, 64) CASE(64, 32) CASE(64, 64)
#undef CASE
}
}  // namespace

UNet::UNet(cudaStream_t st) : st_(st) {
    struct S {
        int ci, co, lv, taps;
    };
    const S spec[] = {{16, 16, 0, 27}, {16, 16, 0, 27}, {16, 32, 1, 27}, {32, 32, 1, 27}, {32, 64, 2, 27},
                      {64, 64, 2, 27}, {64, 64, 3, 27}, {64, 64, 3, 27}, {64, 64, 2, 27}, {64, 32, 2, 27},
                      {32, 32, 1, 27}, {32, 16, 1, 27}, {16, 16, 0, 27}, {16, 16, 0, 27}, {16, 1, 0, 1}};
    long long off = 0, boff = 0;
    for (const S &s : spec) {
        ConvLayer L{s.ci, s.co, s.lv, s.taps, off, off + (long long)s.taps * s.co * s.ci, boff};
        off = L.boff + s.co;
        boff += (long long)s.taps * s.co * s.ci;
        layers_.push_back(L);
    }
    nparams_ = off;
    nbf_ = boff;
    p_ = (float *)alloc(4 * nparams_);
    g_ = (float *)alloc(4 * nparams_);
    m1_ = (float *)alloc(4 * nparams_);
    m2_ = (float *)alloc(4 * nparams_);
    wb_ = (bf16 *)alloc(2 * nbf_);
    wt_ = (bf16 *)alloc(2 * nbf_);
    wbp_ = (bf16 *)alloc(2 * nbf_);
    wtp_ = (bf16 *)alloc(2 * nbf_);
    dots_ = (double *)alloc(8 * 8);
    redpart_ = (double *)alloc(8 * 4 * 1216);
    wpart_elems_ = 64LL * 27 * 64 * 64;
    wpart_ = (float *)alloc(4 * wpart_elems_);
    hpart_ = (float *)alloc(4 * 4096 * 17);
    err_ = (int *)alloc(256);
    cudaMallocHost(&dots_host_, 8 * 8);
    if (p_) {
        cudaMemsetAsync(p_, 0, 4 * nparams_, st_);
        cudaMemsetAsync(m1_, 0, 4 * nparams_, st_);
        cudaMemsetAsync(m2_, 0, 4 * nparams_, st_);
        cudaMemsetAsync(dots_, 0, 64, st_);
        cudaMemsetAsync(err_, 0, 256, st_);
    }
}

UNet::~UNet() {
    for (void *p : ws_) cudaFree(p);
    for (void *p : persist_) cudaFree(p);
    if (dots_host_) cudaFreeHost(dots_host_);
}

void *UNet::alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaMalloc(&p, bytes ? bytes : 256) != cudaSuccess) {
        last_error = "device allocation failed";
        return nullptr;
    }
    persist_.push_back(p);
    return p;
}

void UNet::refresh_bf16() {
    for (const ConvLayer &L : layers_) {
        if (L.taps != 27) continue;
        const long long m = (long long)L.taps * L.cout * L.cin;
        k_f32_to_bf16<<<flat_blocks(m), 256, 0, st_>>>(m, p_ + L.woff, wb_ + L.wbf);
        k_flip_weights<<<flat_blocks(m), 256, 0, st_>>>(L.taps, L.cout, L.cin, p_ + L.woff, wt_ + L.wbf);
        k_taps_dz_major<<<flat_blocks(m), 256, 0, st_>>>(m, L.cout * L.cin, wb_ + L.wbf, wbp_ + L.wbf);
        k_taps_dz_major<<<flat_blocks(m), 256, 0, st_>>>(m, L.cout * L.cin, wt_ + L.wbf, wtp_ + L.wbf);
    }
}

cudaError_t UNet::set_params(const float *host) {
    cudaError_t e = cudaMemcpyAsync(p_, host, 4 * nparams_, cudaMemcpyHostToDevice, st_);
    if (e != cudaSuccess) return e;
    refresh_bf16();
    cudaMemsetAsync(m1_, 0, 4 * nparams_, st_);
    cudaMemsetAsync(m2_, 0, 4 * nparams_, st_);
    step_ = 0;
    return cudaStreamSynchronize(st_);
}

cudaError_t UNet::get_params(float *host) {
    cudaError_t e = cudaMemcpyAsync(host, p_, 4 * nparams_, cudaMemcpyDeviceToHost, st_);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st_);
}

cudaError_t UNet::get_grads(float *host) {
    cudaError_t e = cudaMemcpyAsync(host, g_, 4 * nparams_, cudaMemcpyDeviceToHost, st_);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st_);
}

cudaError_t UNet::ensure(const Dims &d, bool training) {
    if (have_ws_ && dims_[0].nx == d.nx && dims_[0].ny == d.ny && dims_[0].nz == d.nz && (ws_training_ || !training))
        return cudaSuccess;
    for (void *p : ws_) cudaFree(p);
    ws_.clear();
    have_ws_ = false;
    wg_dy_ = wg_x_ = nullptr;
    dims_[0] = d;
    for (int l = 1; l < 4; l++)
        dims_[l] = make_dims((dims_[l - 1].nx + 1) / 2, (dims_[l - 1].ny + 1) / 2, (dims_[l - 1].nz + 1) / 2);
    bool ok = true;
    auto A = [&](size_t bytes) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 256) != cudaSuccess) {
            ok = false;
            return nullptr;
        }
        ws_.push_back(p);
        return p;
    };
    const long long n0 = dims_[0].n, n1 = dims_[1].n, n2 = dims_[2].n, n3 = dims_[3].n;
    auto B = [&](long long n, int c) { return (bf16 *)A(2 * (size_t)n * c); };
    if (!training) {
        // each decoder tensor takes a buffer of its level that is dead by then: U = up(..) + S goes where the
        // first encoder conv's output was, the first decoder conv's output where the skip S was, the second's
        // where the level's pooled input was (level 0: the first encoder buffer again)
        A0a = B(n0, 16); S0 = B(n0, 16); U0 = A0a; D0a = S0; D0b = A0a;
        P1 = B(n1, 16); A1a = B(n1, 32); S1 = B(n1, 32); U1 = A1a; D1a = S1; D1b = P1;
        P2 = B(n2, 32); A2a = B(n2, 64); S2 = B(n2, 64); U2 = A2a; D2a = S2; D2b = P2;
        P3 = B(n3, 64); A3a = B(n3, 64); A3b = B(n3, 64);
        out_ = dout_ = nullptr;
        if (!ok) {
            last_error = "U-Net workspace allocation failed";
            return cudaErrorMemoryAllocation;
        }
        have_ws_ = true;
        ws_training_ = false;
        return cudaSuccess;
    }
    A0a = B(n0, 16); S0 = B(n0, 16); U0 = B(n0, 16); D0a = B(n0, 16); D0b = B(n0, 16);
    P1 = B(n1, 16); A1a = B(n1, 32); S1 = B(n1, 32); U1 = B(n1, 32); D1a = B(n1, 32); D1b = B(n1, 16);
    P2 = B(n2, 32); A2a = B(n2, 64); S2 = B(n2, 64); U2 = B(n2, 64); D2a = B(n2, 64); D2b = B(n2, 32);
    P3 = B(n3, 64); A3a = B(n3, 64); A3b = B(n3, 64);
    const int cmax[4] = {16, 32, 64, 64};
    const long long nl[4] = {n0, n1, n2, n3};
    for (int l = 0; l < 4; l++) {
        gA[l] = (float *)A(4 * (size_t)nl[l] * cmax[l]);
        gB[l] = (float *)A(4 * (size_t)nl[l] * cmax[l]);
        gbf[l] = B(nl[l], cmax[l]);
        if (l < 3) gU[l] = (float *)A(4 * (size_t)nl[l] * cmax[l]);
    }
    out_ = (float *)A(4 * (size_t)n0);
    dout_ = (float *)A(4 * (size_t)n0);
    if (!ok) {
        last_error = "U-Net workspace allocation failed";
        return cudaErrorMemoryAllocation;
    }
    have_ws_ = true;
    ws_training_ = true;
    return cudaSuccess;
}

// channel-major copies for the tcgen05 weight gradient, sized for the largest level (allocated on first use)
cudaError_t UNet::ensure_wgrad_ws() {
    if (wg_dy_) return cudaSuccess;
    const int cmax[4] = {16, 32, 64, 64};
    long long el = 0;
    for (int l = 0; l < 4; l++) {
        const long long e = (long long)cmax[l] * dims_[l].nx * dims_[l].ny * 8 * ((dims_[l].nz + 7) / 8);
        if (e > el) el = e;
    }
    void *a = nullptr, *b = nullptr;
    // on failure the caller falls back to the warp-MMA kernel: clear the error so that it is not reported later
    if (cudaMalloc(&a, 2 * (size_t)el) != cudaSuccess) {
        cudaGetLastError();
        return cudaErrorMemoryAllocation;
    }
    ws_.push_back(a);
    if (cudaMalloc(&b, 6 * (size_t)el) != cudaSuccess) {
        cudaGetLastError();
        return cudaErrorMemoryAllocation;
    }
    ws_.push_back(b);
    wg_dy_ = (bf16 *)a;
    wg_x_ = (bf16 *)b;
    return cudaSuccess;
}

void UNet::conv_fwd(const ConvLayer &L, const Dims &d, const bf16 *x, bf16 *y) {
    if (mode_ == 1 && L.taps == 27 && tc_shape_ok(L.cin, L.cout, d)) {
        cudaError_t e = tc_dispatch(st_, L.cin, L.cout, 0, d, x, wb_ + L.wbf, wbp_ + L.wbf, p_ + L.boff, y, err_);
        if (e == cudaSuccess) {
            tc_launches_++;
            return;
        }
        last_error = std::string("tcgen05 convolution not launched: ") + cudaGetErrorString(e);
        cudaGetLastError();  // the warp-MMA kernel below runs instead: the refused launch is not an error
    }
    conv_dispatch(st_, L.cin, L.cout, 0, d, x, wb_ + L.wbf, p_ + L.boff, y, L.taps);
}

cudaError_t UNet::check_device_errors() {
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, err_, sizeof(int), cudaMemcpyDeviceToHost, st_);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return e;
    if (h != 0) {
        last_error = "tcgen05 convolution: a bounded wait timed out";
        cudaMemsetAsync(err_, 0, sizeof(int), st_);
        return cudaErrorLaunchFailure;
    }
    return cudaSuccess;
}

cudaError_t UNet::forward(const Dims &d, const bf16 *feat, float *out, bool training) {
    if (!training && !out) return cudaErrorInvalidValue;
    cudaError_t e = ensure(d, training);
    if (e != cudaSuccess) return e;
    feat_ = feat;
    const ConvLayer *Ls = layers_.data();
    const Dims &d0 = dims_[0], &d1 = dims_[1], &d2 = dims_[2], &d3 = dims_[3];
    conv_fwd(Ls[0], d0, feat, A0a);
    conv_fwd(Ls[1], d0, A0a, S0);
    k_pool<16><<<line_grid(d1, 2), 256, 0, st_>>>(d0, d1, S0, P1);
    conv_fwd(Ls[2], d1, P1, A1a);
    conv_fwd(Ls[3], d1, A1a, S1);
    k_pool<32><<<line_grid(d2, 4), 256, 0, st_>>>(d1, d2, S1, P2);
    conv_fwd(Ls[4], d2, P2, A2a);
    conv_fwd(Ls[5], d2, A2a, S2);
    k_pool<64><<<line_grid(d3, 8), 256, 0, st_>>>(d2, d3, S2, P3);
    conv_fwd(Ls[6], d3, P3, A3a);
    conv_fwd(Ls[7], d3, A3a, A3b);
    k_up_add<64><<<line_grid(d2, 8), 256, 0, st_>>>(d2, d3, A3b, S2, U2);
    conv_fwd(Ls[8], d2, U2, D2a);
    conv_fwd(Ls[9], d2, D2a, D2b);
    k_up_add<32><<<line_grid(d1, 4), 256, 0, st_>>>(d1, d2, D2b, S1, U1);
    conv_fwd(Ls[10], d1, U1, D1a);
    conv_fwd(Ls[11], d1, D1a, D1b);
    k_up_add<16><<<line_grid(d0, 2), 256, 0, st_>>>(d0, d1, D1b, S0, U0);
    conv_fwd(Ls[12], d0, U0, D0a);
    conv_fwd(Ls[13], d0, D0a, D0b);
    const ConvLayer &H = Ls[14];
    k_head_fwd<<<flat_blocks(d0.n), 256, 0, st_>>>(d0.n, D0b, p_ + H.woff, p_ + H.boff, out ? out : out_);
    return cudaGetLastError();
}

// relu backward, weight/bias gradients and (optionally) the input gradient of one conv layer
void UNet::conv_bwd(const ConvLayer &L, const Dims &d, const bf16 *x, const bf16 *post, const float *dpost,
                    float *dx) {
    const long long m = d.n * L.cout;
    bf16 *dy = gbf[L.level];
    k_relu_back<<<flat_blocks(m), 256, 0, st_>>>(m, dpost, post, dy);
    long long vchunk = (d.n + 63) / 64;
    if (vchunk < kVchunkMin) vchunk = kVchunkMin;
    const int chunks = (int)((d.n + vchunk - 1) / vchunk);
    int wchunks = 0;
    if (mode_ >= 1 && L.taps == 27 && wgrad_tc_ok(L.cin, L.cout, d)) {
        cudaError_t e = ensure_wgrad_ws();
        if (e == cudaSuccess)
            e = wgrad_tc_dispatch(st_, L.cin, L.cout, d, dy, x, wg_dy_, wg_x_, wpart_, wpart_elems_, wchunks, err_);
        if (e == cudaSuccess)
            tc_launches_++;
        else {
            wchunks = 0;
            last_error = std::string("tcgen05 weight gradient not launched: ") + cudaGetErrorString(e);
            cudaGetLastError();  // the warp-MMA kernel runs instead
        }
    }
    if (wchunks == 0) {
        wgrad_dispatch(st_, L.cin, L.cout, d, dy, x, wpart_, L.taps, (int)vchunk, chunks);
        wchunks = chunks;
    }
    const long long mw = (long long)L.taps * L.cout * L.cin;
    k_reduce_chunks<<<flat_blocks(mw), 256, 0, st_>>>(wpart_, wchunks, mw, g_ + L.woff);
    // bias gradient: up to 1024 chunks of at least 256 voxels (partials fit the 4096 x 17 scratch for 64 channels)
    long long bvchunk = (d.n + 1023) / 1024;
    if (bvchunk < 256) bvchunk = 256;
    const int bchunks = (int)((d.n + bvchunk - 1) / bvchunk);
    if (L.cout == 16)
        k_bias_grad<16><<<bchunks, 256, 0, st_>>>(d.n, dy, (int)bvchunk, hpart_);
    else if (L.cout == 32)
        k_bias_grad<32><<<bchunks, 256, 0, st_>>>(d.n, dy, (int)bvchunk, hpart_);
    else
        k_bias_grad<64><<<bchunks, 256, 0, st_>>>(d.n, dy, (int)bvchunk, hpart_);
    k_reduce_chunks<<<1, 64, 0, st_>>>(hpart_, bchunks, L.cout, g_ + L.boff);
    if (!dx) return;
    // input gradient: the forward convolution with the mirrored, transposed weights (FP32 out, no bias)
    if (mode_ == 1 && L.taps == 27 && tc_shape_ok(L.cout, L.cin, d)) {
        const cudaError_t e = tc_dispatch(st_, L.cout, L.cin, 1, d, dy, wt_ + L.wbf, wtp_ + L.wbf, nullptr, dx, err_);
        if (e == cudaSuccess) {
            tc_launches_++;
            return;
        }
        last_error = std::string("tcgen05 convolution not launched: ") + cudaGetErrorString(e);
        cudaGetLastError();  // the warp-MMA kernel below runs instead: the refused launch is not an error
    }
    conv_dispatch(st_, L.cout, L.cin, 1, d, dy, wt_ + L.wbf, nullptr, dx, L.taps);
}

cudaError_t UNet::backward(const Dims &d, const float *dout) {
    if (!have_ws_ || !ws_training_ || dims_[0].nx != d.nx || dims_[0].ny != d.ny || dims_[0].nz != d.nz)
        return cudaErrorInvalidValue;
    const ConvLayer *Ls = layers_.data();
    const Dims &d0 = dims_[0], &d1 = dims_[1], &d2 = dims_[2], &d3 = dims_[3];
    // head (1x1): da = dout w, dw = sum dout a, db = sum dout
    {
        const ConvLayer &H = Ls[14];
        long long vchunk = (d0.n + 4095) / 4096;
        if (vchunk < 256) vchunk = 256;
        const int chunks = (int)((d0.n + vchunk - 1) / vchunk);
        k_head_back<<<chunks, 64, 0, st_>>>(d0.n, 16, D0b, p_ + H.woff, dout, gA[0], (int)vchunk, hpart_);
        k_reduce_chunks<<<1, 64, 0, st_>>>(hpart_, chunks, 17, g_ + H.woff);  // 16 weights then the bias
    }
    conv_bwd(Ls[13], d0, D0a, D0b, gA[0], gB[0]);
    conv_bwd(Ls[12], d0, U0, D0a, gB[0], gU[0]);
    k_up_back<16><<<line_grid(d1, 4), 256, 0, st_>>>(d0, d1, gU[0], gA[1]);
    conv_bwd(Ls[11], d1, D1a, D1b, gA[1], gB[1]);
    conv_bwd(Ls[10], d1, U1, D1a, gB[1], gU[1]);
    k_up_back<32><<<line_grid(d2, 8), 256, 0, st_>>>(d1, d2, gU[1], gA[2]);
    conv_bwd(Ls[9], d2, D2a, D2b, gA[2], gB[2]);
    conv_bwd(Ls[8], d2, U2, D2a, gB[2], gU[2]);
    k_up_back<64><<<line_grid(d3, 16), 256, 0, st_>>>(d2, d3, gU[2], gA[3]);
    conv_bwd(Ls[7], d3, A3a, A3b, gA[3], gB[3]);
    conv_bwd(Ls[6], d3, P3, A3a, gB[3], gA[3]);
    k_pool_back<64><<<line_grid(d2, 16), 256, 0, st_>>>(d2, d3, gA[3], gU[2], gA[2]);
    conv_bwd(Ls[5], d2, A2a, S2, gA[2], gB[2]);
    conv_bwd(Ls[4], d2, P2, A2a, gB[2], gA[2]);
    k_pool_back<32><<<line_grid(d1, 8), 256, 0, st_>>>(d1, d2, gA[2], gU[1], gA[1]);
    conv_bwd(Ls[3], d1, A1a, S1, gA[1], gB[1]);
    conv_bwd(Ls[2], d1, P1, A1a, gB[1], gA[1]);
    k_pool_back<16><<<line_grid(d0, 4), 256, 0, st_>>>(d0, d1, gA[1], gU[0], gA[0]);
    conv_bwd(Ls[1], d0, A0a, S0, gA[0], gB[0]);
    conv_bwd(Ls[0], d0, feat_, A0a, gB[0], nullptr);
    return cudaGetLastError();
}

cudaError_t UNet::train_step(const Dims &d, const bf16 *feat, const float *target, float lr, double &loss) {
    cudaError_t e = forward(d, feat, nullptr);
    if (e != cudaSuccess) return e;
    unsigned *ticket = reinterpret_cast<unsigned *>(dots_ + 4);
    k_cos_dots<<<1216, dim3(32, 8), 0, st_>>>(d.n, out_, target, dots_, redpart_, ticket);
    k_cos_grad<<<flat_blocks(d.n), 256, 0, st_>>>(d.n, out_, target, dots_, dout_);
    e = backward(d, dout_);
    if (e != cudaSuccess) return e;
    if (mode_ >= 1 && (e = check_device_errors()) != cudaSuccess) return e;
    step_++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)step_), c2 = 1.f - powf(b2, (float)step_);
    k_adam<<<flat_blocks(nparams_), 256, 0, st_>>>(nparams_, p_, g_, m1_, m2_, lr, b1, b2, 1e-8f, c1, c2, nullptr);
    refresh_bf16();
    cudaMemcpyAsync(dots_host_, dots_, 24, cudaMemcpyDeviceToHost, st_);
    e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return e;
    const double ot = dots_host_[0], oo = dots_host_[1], tt = dots_host_[2];
    loss = (oo > 0 && tt > 0) ? 1.0 - ot * ot / (oo * tt) : 1.0;
    return cudaSuccess;
}

// ------------------------------------------------------------------------------------------------ features
// Input channels of the network for a system A x = b in face-coefficient form (FP64 fine level):
//   0: b / rms(b)  1: active (D > 0)  2-4: lower-face couplings ax, ay, az divided by D  5: dex / D
//   6-15: zero.  Everything is dimensionless, so one network serves the pressure and the potential systems.
__global__ void k_features(Dims d, Coef<double> cf, const double *__restrict__ b, double inv_rms, bf16 *__restrict__ f) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < d.n; c += (long long)gridDim.x * blockDim.x) {
        const double D = cf.D[c];
        const float inv = D > 0 ? (float)(1.0 / D) : 0.f;
        float v[16] = {0};
        v[0] = (float)(b[c] * inv_rms);
        v[1] = D > 0 ? 1.f : 0.f;
        v[2] = (float)cf.ax[c] * inv;
        v[3] = (float)cf.ay[c] * inv;
        v[4] = (float)cf.az[c] * inv;
        v[5] = (float)cf.dex[c] * inv;
        uint32_t w[8];
#pragma unroll
        for (int q = 0; q < 8; q++) w[q] = pack_bf16(v[2 * q], v[2 * q + 1]);
        uint4 *dst = reinterpret_cast<uint4 *>(f + c * 16);
        dst[0] = make_uint4(w[0], w[1], w[2], w[3]);
        dst[1] = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

__global__ void __launch_bounds__(256) k_sumsq_active(long long n, const double *__restrict__ b,
                                                      const double *__restrict__ D, double *out, double *part,
                                                      unsigned *ticket) {
    double v[2] = {0, 0};
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    for (long long c = blockIdx.x * 256LL + tid; c < n; c += (long long)gridDim.x * 256) {
        if (D[c] > 0) {
            v[0] += b[c] * b[c];
            v[1] += 1.0;
        }
    }
    double tot[2];
    if (grid_reduce<2>(v, part, ticket, tot)) {
        out[0] = tot[0];
        out[1] = tot[1];
    }
}

cudaError_t UNet::features(const Dims &d, const Coef<double> &cf, const double *b, bf16 *feat) {
    unsigned *ticket = reinterpret_cast<unsigned *>(dots_ + 4);
    k_sumsq_active<<<1216, dim3(32, 8), 0, st_>>>(d.n, b, cf.D, dots_, redpart_, ticket);
    cudaMemcpyAsync(dots_host_, dots_, 16, cudaMemcpyDeviceToHost, st_);
    cudaError_t e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return e;
    const double cnt = dots_host_[1] > 0 ? dots_host_[1] : 1.0;
    active_ = dots_host_[1];
    const double rms = std::sqrt(dots_host_[0] / cnt);
    const double inv = rms > 0 ? 1.0 / rms : 0.0;
    k_features<<<flat_blocks(d.n), 256, 0, st_>>>(d, cf, b, inv, feat);
    return cudaGetLastError();
}

__global__ void k_feat_rhs(long long n, const float *__restrict__ r, float inv_rms, bf16 *__restrict__ f) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        f[c * 16] = __float2bfloat16_rn(r[c] * inv_rms);
}

cudaError_t UNet::set_rhs_channel(const Dims &d, const float *r, double inv_rms, bf16 *feat) {
    k_feat_rhs<<<flat_blocks(d.n), 256, 0, st_>>>(d.n, r, (float)inv_rms, feat);
    return cudaGetLastError();
}

}  // namespace sf
