// sf_conv_tc.cuh -- 3x3x3 convolution forward on the 5th-generation tensor cores (tcgen05 + TMA, sm_103a).
//
// Implicit GEMM per CTA: MT tiles of M = 128 output voxels (a 32 (z) x 4 MT (y) x 1 (x) brick), N = Cout,
// K = 27 taps x Cin.  Operands are staged by TMA in the no-swizzle K-major "core matrix" layout: one 4-D box of
// 8 channels x (32 x 4 MT x 1) voxels per 8-channel chunk and tap lands as 128 MT rows x 16 B, i.e. 8-row x 16-B
// core matrices with a 128-B stride along M, one tile per 2 KB and one (2 MT)-KB chunk per 8 channels along K;
// taps outside the grid are filled with zeros by the TMA unit (the convolution's zero padding).  Weights
// [tap][Cout][Cin] are staged the same way, once per tap for all MT tiles.  Lane 0 of warp 1 issues the TMA loads
// and lane 0 of warp 0 the tcgen05.mma (M=128, N=Cout, K=16, BF16 in, FP32 accumulate in TMEM, one accumulator of
// Cout columns per tile) through a ring of stages guarded by mbarriers; all four warps read the accumulators back
// with tcgen05.ld and apply bias + ReLU + BF16 conversion.  Every wait is bounded: on timeout the CTA records an error code and
// returns after releasing its tensor memory.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "sf_internal.cuh"
#include "sf_tma.cuh"

namespace sf {
namespace tc {

constexpr int kMaxStages = 4;
// Shared-memory matrix descriptor, no swizzle, K-major: start, leading (K) and stride (M/N) byte offsets in
// 16-byte units, descriptor version 1 (bits 46..48 = 0b001), swizzle mode 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo_bytes, uint32_t sbo_bytes) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo_bytes >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo_bytes >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// The same descriptor for the 32-byte swizzled K-major layout (layout type 6): rows of 32 bytes (16 BF16 along K)
// whose two 16-byte halves swap in rows 4-7 of every 8-row, 256-byte atom, as TMA writes them with
// CU_TENSOR_MAP_SWIZZLE_32B; the stride (M/N) byte offset is the 256-byte atom, the leading offset is unused.
__device__ __forceinline__ uint64_t smem_desc_sw32(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(256u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)6 << 61;
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t instr_desc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

template <int N>
__device__ __forceinline__ void tmem_ld_x16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 16; q++) v[q] = __uint_as_float(r[q]);
}

constexpr int kTileZ = 32, kTileY = 4;

// M tiles per CTA: four (the weights of a tap staged once for 512 voxels), two for 64 input channels, whose
// stages are twice as large
template <int CI, int CO>
constexpr int tiles_per_cta() {
    return CI == 64 ? 2 : 4;
}

template <int CI, int CO, int MT>
struct Layout {
    static constexpr int kChunks = CI / 8;
    static constexpr uint32_t kChunkBytes = 128u * 16u * MT;  // 128 MT rows x 16 B per 8-channel chunk
    static constexpr uint32_t kABytes = kChunkBytes * kChunks;
    static constexpr uint32_t kBBytes = (uint32_t)CO * 16u * kChunks;
    static constexpr uint32_t kStageBytes = kABytes + kBBytes;
    // stages within about 100 KB, so that two or more CTAs share an SM where the stages are small
    static constexpr int kStages = (int)(100u * 1024u / kStageBytes) > kMaxStages ? kMaxStages
                                   : (int)(100u * 1024u / kStageBytes) < 2    ? 2
                                                                              : (int)(100u * 1024u / kStageBytes);
    // accumulator columns: one Cout-wide block per tile, allocated as a power of two >= 32
    static constexpr uint32_t kCols = (uint32_t)(MT * CO) <= 32u    ? 32u
                                      : (uint32_t)(MT * CO) <= 64u  ? 64u
                                      : (uint32_t)(MT * CO) <= 128u ? 128u
                                      : (uint32_t)(MT * CO) <= 256u ? 256u
                                                                    : 512u;
    static constexpr uint32_t kNeed = kStages * kStageBytes + 1024 /* alignment */ + 256 /* barriers */;
    // enough shared memory that at most 512 / kCols CTAs share an SM, so every CTA's TMEM allocation fits
    static constexpr uint32_t kMinSmem = 233472u / (512u / kCols + 1u) + 1024u;
    static constexpr uint32_t kSmemBytes = kNeed > kMinSmem ? kNeed : kMinSmem;
    static_assert(kSmemBytes <= 227u * 1024u, "shared memory");
    static_assert(MT * CO <= 512, "TMEM columns");
};

// err: first error code of any CTA (1 = TMA/MMA wait timed out).
// EPI 0: + bias, ReLU, BF16 out (forward).  EPI 1: FP32 out, no bias (input gradient, with the mirrored and
// transposed weights).
template <int CI, int CO, int EPI = 0, int MT = tiles_per_cta<CI, CO>()>
__global__ void __launch_bounds__(128, 1) k_conv_tc(const __grid_constant__ CUtensorMap tmap_x,
                                                    const __grid_constant__ CUtensorMap tmap_w, Dims d,
                                                    const float *__restrict__ bias, void *__restrict__ yout,
                                                    int *err) {
    static_assert(CI % 16 == 0 && CO % 16 == 0 && CO <= 256, "shape");
    using L = Layout<CI, CO, MT>;
    constexpr int kStages = L::kStages;
    extern __shared__ uint8_t smem_raw[];
    // 1024-byte aligned stage buffers, barriers after them
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kStages * L::kStageBytes);
    // sh: [0] TMEM base, [1] status, [2] MMA side ok, [3] stages waited, [4] TMA side ok, [5] stages issued
    volatile uint32_t *sh = reinterpret_cast<volatile uint32_t *>(bars + 2 * kStages + 1);
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + kStages), done = smem_u32(bars + 2 * kStages);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    const int tiles_z = (d.nz + kTileZ - 1) / kTileZ, tiles_y = (d.ny + kTileY * MT - 1) / (kTileY * MT);
    const int bz = blockIdx.x % tiles_z, by = (blockIdx.x / tiles_z) % tiles_y, bx = blockIdx.x / (tiles_z * tiles_y);
    const int z0 = bz * kTileZ, y0 = by * kTileY * MT, x0 = bx;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; s++) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        mbar_init(done, 1);
        for (int k = 1; k < 6; k++) sh[k] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(const_cast<uint32_t *>(sh))),
                     "r"(L::kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = sh[0];

    // warp specialised: lane 0 of warp 1 issues the TMA loads of the 27 taps through the ring of stages, lane 0 of
    // warp 0 the MMAs, so a stage is refilled as soon as its MMAs complete without holding up the next MMAs
    constexpr int T = 27;
    if (warp == 1 && lane == 0) {
        bool ok = true;
        int issued = 0;
        for (int t = 0; t < T; t++) {
            const int s = t % kStages;
            if (t >= kStages && !mbar_wait(empty0 + 8 * s, (uint32_t)(t / kStages - 1) & 1u)) {
                ok = false;
                break;
            }
            const uint32_t a = smem_u32(smem + s * L::kStageBytes), b = a + L::kABytes;
            const uint32_t bar = full0 + 8 * s;
            mbar_expect_tx(bar, L::kStageBytes);
            const int dx = t / 9 - 1, dy = (t / 3) % 3 - 1, dz = t % 3 - 1;
#pragma unroll
            for (int c = 0; c < L::kChunks; c++) {
                tma_load_4d(a + c * L::kChunkBytes, &tmap_x, bar, 8 * c, z0 + dz, y0 + dy, x0 + dx);
                tma_load_3d(b + c * (uint32_t)CO * 16u, &tmap_w, bar, 8 * c, 0, t);
            }
            issued = t + 1;
        }
        sh[4] = ok ? 1u : 0u;
        sh[5] = (uint32_t)issued;
    } else if (warp == 0 && lane == 0) {
        constexpr uint32_t idesc = instr_desc_bf16(CO);
        bool ok = true;
        int waited = 0;
        for (int t = 0; t < T; t++) {
            const int s = t % kStages;
            if (!mbar_wait(full0 + 8 * s, (uint32_t)(t / kStages) & 1u)) {
                ok = false;
                break;
            }
            waited = t + 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a = smem_u32(smem + s * L::kStageBytes), b = a + L::kABytes;
            // K = 16 spans two 8-channel chunks: leading (K) offset = one chunk, stride (M/N) = 8 rows; tile m's rows
            // start 2 KB further into each chunk, its accumulator CO columns further.  The descriptors are bases plus
            // compile-time offsets in 16-byte units (no carry: shared addresses stay below 256 KB).
            const uint64_t ad0 = smem_desc(a, L::kChunkBytes, 128u), bd0 = smem_desc(b, (uint32_t)CO * 16u, 128u);
            const uint32_t acc0 = t > 0 ? 1u : 0u;
#pragma unroll
            for (int j = 0; j < CI / 16; j++) {
                const uint64_t bd = bd0 + (uint64_t)(j * 2 * CO);
#pragma unroll
                for (int m = 0; m < MT; m++) {
                    const uint64_t ad = ad0 + (uint64_t)((j * 2 * L::kChunkBytes + m * 2048u) >> 4);
                    mma_bf16(tmem + (uint32_t)(m * CO), ad, bd, idesc, j > 0 ? 1u : acc0);
                }
            }
            mma_commit(empty0 + 8 * s);
        }
        if (waited > 0) {  // completion of every MMA issued (also on the error path, before TMEM is released)
            mma_commit(done);
            if (!mbar_wait(done, 0)) ok = false;
        }
        sh[2] = ok ? 1u : 0u;
        sh[3] = (uint32_t)waited;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const bool ok = sh[2] && sh[4];
        if (!ok) {  // drain loads still in flight into this CTA's shared memory (bounded)
            for (uint32_t t = sh[3]; t < sh[5]; t++) mbar_wait(full0 + 8 * (t % kStages), (t / kStages) & 1u);
            atomicCAS(err, 0, 1);
        }
        sh[1] = ok ? 1u : 0u;
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (sh[1]) {  // uniform across the CTA
#pragma unroll 1
        for (int m = 0; m < MT; m++) {
        const int r = 32 * warp + lane;  // TMEM lane = tile row
        const int z = z0 + (r % kTileZ), yy = y0 + kTileY * m + r / kTileZ;
        const bool inb = z < d.nz && yy < d.ny && x0 < d.nx;
        const long long v = inb ? cid(d, x0, yy, z) : 0;
#pragma unroll
        for (int c0 = 0; c0 < CO; c0 += 16) {
            float acc[16];
            tmem_ld_x16<16>(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(m * CO + c0), acc);
            if (inb && EPI == 0) {
                uint32_t pk[8];
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    const float a0 = fmaxf(acc[2 * q] + bias[c0 + 2 * q], 0.f);
                    const float a1 = fmaxf(acc[2 * q + 1] + bias[c0 + 2 * q + 1], 0.f);
                    __nv_bfloat162 h2 = __floats2bfloat162_rn(a0, a1);
                    pk[q] = *reinterpret_cast<uint32_t *>(&h2);
                }
                uint4 *dst = reinterpret_cast<uint4 *>(reinterpret_cast<__nv_bfloat16 *>(yout) + v * CO + c0);
                dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
            } else if (inb) {
                float4 *dst = reinterpret_cast<float4 *>(reinterpret_cast<float *>(yout) + v * CO + c0);
#pragma unroll
                for (int q = 0; q < 4; q++) dst[q] = make_float4(acc[4 * q], acc[4 * q + 1], acc[4 * q + 2], acc[4 * q + 3]);
            }
        }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(L::kCols) : "memory");
    }
}

// ------------------------------------------------------------------------------------------------ z lines
// Forward (and input gradient) for Cin = 16 or 32, Cout <= 32, on grids with nz >= 128: a persistent CTA per SM
// takes bricks of 128 (z) x 4 (y) x LX (x) voxels (LX = 2 for 16 input channels, 1 for 32), 4 LX M tiles of one
// z line of 128 voxels each.  A pipeline stage is one z shift dz and one group of 16 channels (K = 16): one TMA box,
// (16 channels, 128 z, 6 y, LX + 2 x) from (z0 + dz, y0 - 1, x0 - 1), lands as 32-byte rows in the 32-byte swizzled
// K-major layout and carries the tile rows of all nine (dx, dy) taps: tile (yy, xx) of tap (dx, dy) starts
// 4 KB x ((yy + 1 + dy) + 6 (xx + 1 + dx)) into the box, so each box is read once for nine taps (the 27-box kernel
// above reads nine times as many rows, of 16 bytes, each half of a 32-byte sector).  The 27 taps' weights stay in
// shared memory, swizzled the same way, for the CTA's whole run.  Warp 1 lane 0 issues the TMA loads through two stages, warp 0 lane 0
// the MMAs (M = 128, N = Cout, K = 16) into one of two TMEM accumulator sets, and warps 2-5 read the other set back
// (bias + ReLU + BF16, or FP32), so the epilogue of a brick overlaps the MMAs of the next.  Every wait is bounded; a
// timeout stops all roles, drains the copies in flight and sets the error flag.
constexpr int kLineZ = 128, kLineY = 4;

template <int CI>
__host__ __device__ constexpr int line_x() {
    return CI == 16 ? 2 : 1;
}

template <int CI, int CO>
struct LineLayout {
    static constexpr int LX = line_x<CI>(), kTiles = kLineY * LX, KP = CI / 16;  // 16-channel groups
    static constexpr uint32_t kBoxRows = kLineZ * (kLineY + 2) * (LX + 2);
    static constexpr uint32_t kStageBytes = kBoxRows * 32u;  // 96 KB (LX 2) or 72 KB (LX 1)
    static constexpr uint32_t kWChunkRaw = 27u * CO * 32u;  // [tap][co] rows of 16 channels
    static constexpr uint32_t kWChunk = (kWChunkRaw + 1023u) & ~1023u;
    static constexpr uint32_t kCols = kTiles * CO;  // one accumulator set
    static constexpr uint32_t kAlloc = 2u * kCols <= 256u ? 256u : 512u;
    static constexpr uint32_t kSmemBytes = 1024u + 2u * kStageBytes + KP * kWChunk + 256u;
    static_assert(CI % 16 == 0 && 2u * kCols <= 512u && kSmemBytes <= 227u * 1024u, "line layout");
};

template <int CI, int CO, int EPI>
__global__ void __launch_bounds__(192, 1) k_conv_tc_line(const __grid_constant__ CUtensorMap tmap_x,
                                                         const __grid_constant__ CUtensorMap tmap_w, Dims d,
                                                         const float *__restrict__ bias, void *__restrict__ yout,
                                                         int *err) {
    using L = LineLayout<CI, CO>;
    constexpr int LX = L::LX, kTiles = L::kTiles, KP = L::KP;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *wbuf = smem + 2 * L::kStageBytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(wbuf + KP * L::kWChunk);
    // barriers: [0,2) stage full, [2,4) stage empty, 4 weights, [5,7) accumulators full, [7,9) accumulators
    // empty (four epilogue warps), 9 done
    volatile uint32_t *sh = reinterpret_cast<volatile uint32_t *>(bars + 10);
    // sh: [0] TMEM base, [1] abort, [2] stage jobs issued, [3] stage jobs waited, [4] weights waited
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + 2), wfull = smem_u32(bars + 4),
                   tfull0 = smem_u32(bars + 5), tempty0 = smem_u32(bars + 7), done = smem_u32(bars + 9);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int bz_n = (d.nz + kLineZ - 1) / kLineZ, by_n = (d.ny + kLineY - 1) / kLineY;
    const long long nbricks = (long long)bz_n * by_n * ((d.nx + LX - 1) / LX);
    const int nb = nbricks > blockIdx.x ? (int)((nbricks - 1 - blockIdx.x) / gridDim.x + 1) : 0;
    auto brick = [&](int bi, int &z0, int &y0, int &x0) {
        const long long br = blockIdx.x + (long long)bi * gridDim.x;
        z0 = kLineZ * (int)(br % bz_n);
        y0 = kLineY * (int)((br / bz_n) % by_n);
        x0 = LX * (int)(br / ((long long)bz_n * by_n));
    };

    if (threadIdx.x == 0) {
        for (int s = 0; s < 2; s++) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
            mbar_init(tfull0 + 8 * s, 1);
            mbar_init(tempty0 + 8 * s, 4);
        }
        mbar_init(wfull, 1);
        mbar_init(done, 1);
        for (int k = 1; k < 5; k++) sh[k] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(const_cast<uint32_t *>(sh))),
                     "r"(L::kAlloc)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = sh[0];

    if (warp == 1 && lane == 0 && nb > 0) {  // TMA producer
        mbar_expect_tx(wfull, KP * L::kWChunkRaw);
        for (int c = 0; c < KP; c++) tma_load_3d(smem_u32(wbuf + c * L::kWChunk), &tmap_w, wfull, 16 * c, 0, 0);
        int q = 0;
        for (int bi = 0; bi < nb && !sh[1]; bi++) {
            int z0, y0, x0;
            brick(bi, z0, y0, x0);
            for (int st = 0; st < 3 * KP && !sh[1]; st++, q++) {  // stage = (dz, 16-channel group)
                const int dz = st / KP, jp = st % KP, s = q & 1;
                if (q >= 2 && !mbar_wait(empty0 + 8 * s, (uint32_t)((q >> 1) - 1) & 1u)) {
                    sh[1] = 1;
                    break;
                }
                mbar_expect_tx(full0 + 8 * s, L::kStageBytes);
                tma_load_4d(smem_u32(smem + s * L::kStageBytes), &tmap_x, full0 + 8 * s, 16 * jp, z0 + dz - 1, y0 - 1,
                            x0 - 1);
                sh[2] = (uint32_t)(q + 1);
            }
        }
    } else if (warp == 0 && lane == 0 && nb > 0) {  // MMA issuer
        constexpr uint32_t idesc = instr_desc_bf16(CO);
        bool any = false;
        if (!mbar_wait(wfull, 0)) sh[1] = 1;
        else sh[4] = 1;
        int q = 0;
        for (int bi = 0; bi < nb && !sh[1]; bi++) {
            const int tb = bi & 1;
            if (bi >= 2 && !mbar_wait(tempty0 + 8 * tb, (uint32_t)((bi - 2) >> 1) & 1u)) {
                sh[1] = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int st = 0; st < 3 * KP; st++, q++) {
                const int dz = st / KP, jp = st % KP, s = q & 1;
                if (!mbar_wait(full0 + 8 * s, (uint32_t)(q >> 1) & 1u)) {
                    sh[1] = 1;
                    break;
                }
                sh[3] = (uint32_t)(q + 1);
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                // descriptor bases of this stage; every MMA below adds a compile-time offset in 16-byte units (the
                // start field cannot carry: shared addresses stay below 256 KB)
                const uint64_t ad0 = smem_desc_sw32(smem_u32(smem + s * L::kStageBytes));
                const uint64_t bd0 = smem_desc_sw32(smem_u32(wbuf) + jp * L::kWChunk + (uint32_t)dz * CO * 32u);
                const uint32_t tacc = tmem + (uint32_t)(tb * L::kCols);
                const uint32_t acc0 = st > 0 ? 1u : 0u;
#pragma unroll
                for (int pr = 0; pr < 9; pr++) {
                    const int dx = pr / 3 - 1, dy = pr % 3 - 1;
                    const uint64_t bd = bd0 + (uint64_t)((9 * (dx + 1) + 3 * (dy + 1)) * CO * 2);
#pragma unroll
                    for (int tile = 0; tile < kTiles; tile++) {
                        const int yy = tile % kLineY, xx = tile / kLineY;
                        const uint64_t ad = ad0 + (uint64_t)(256 * ((yy + 1 + dy) + (kLineY + 2) * (xx + 1 + dx)));
                        mma_bf16(tacc + (uint32_t)(tile * CO), ad, bd, idesc, pr > 0 ? 1u : acc0);
                    }
                }
                any = true;
                mma_commit(empty0 + 8 * s);
            }
            if (sh[1]) break;
            mma_commit(tfull0 + 8 * tb);
        }
        if (any) {  // completion of every MMA issued (also on the error path, before TMEM is released)
            mma_commit(done);
            if (!mbar_wait(done, 0)) sh[1] = 1;
        }
    } else if (warp >= 2 && nb > 0) {  // epilogue
        const int q4 = warp & 3;  // TMEM lane quarter of this warp
        for (int bi = 0; bi < nb; bi++) {
            const int tb = bi & 1;
            const uint32_t par = (uint32_t)(bi >> 1) & 1u;
            // lane 0 decides for the warp, so that the warp-collective TMEM loads below are never divergent
            int go = 0;
            if (lane == 0) go = (!sh[1] && mbar_wait(tfull0 + 8 * tb, par)) ? 1 : 0;
            go = __shfl_sync(0xffffffffu, go, 0);
            if (!go) {
                if (lane == 0) sh[1] = 1;
                break;
            }
            mbar_wait(tfull0 + 8 * tb, par);  // completed: returns at once, with this thread's acquire
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            int z0, y0, x0;
            brick(bi, z0, y0, x0);
            const int z = z0 + 32 * q4 + lane;
#pragma unroll 1
            for (int tile = 0; tile < kTiles; tile++) {
                const int yy = y0 + tile % kLineY, xx = x0 + tile / kLineY;
                const bool inb = z < d.nz && yy < d.ny && xx < d.nx;
                const long long v = inb ? cid(d, xx, yy, z) : 0;
#pragma unroll
                for (int c0 = 0; c0 < CO; c0 += 16) {
                    float acc[16];
                    tmem_ld_x16<16>(tmem + ((uint32_t)(32 * q4) << 16) + (uint32_t)(tb * L::kCols + tile * CO + c0),
                                    acc);
                    if (inb && EPI == 0) {
                        uint32_t pk[8];
#pragma unroll
                        for (int k = 0; k < 8; k++) {
                            const float a0 = fmaxf(acc[2 * k] + bias[c0 + 2 * k], 0.f);
                            const float a1 = fmaxf(acc[2 * k + 1] + bias[c0 + 2 * k + 1], 0.f);
                            __nv_bfloat162 h2 = __floats2bfloat162_rn(a0, a1);
                            pk[k] = *reinterpret_cast<uint32_t *>(&h2);
                        }
                        uint4 *dst = reinterpret_cast<uint4 *>(reinterpret_cast<__nv_bfloat16 *>(yout) + v * CO + c0);
                        dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                        dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
                    } else if (inb) {
                        float4 *dst = reinterpret_cast<float4 *>(reinterpret_cast<float *>(yout) + v * CO + c0);
#pragma unroll
                        for (int k = 0; k < 4; k++)
                            dst[k] = make_float4(acc[4 * k], acc[4 * k + 1], acc[4 * k + 2], acc[4 * k + 3]);
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tempty0 + 8 * tb) : "memory");
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && sh[1]) {  // drain copies still in flight into this CTA's shared memory (bounded)
        for (uint32_t q = sh[3]; q < sh[2]; q++) mbar_wait(full0 + 8 * (q & 1), (q >> 1) & 1u);
        if (!sh[4] && nb > 0) mbar_wait(wfull, 0);
        atomicCAS(err, 0, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(L::kAlloc) : "memory");
    }
}

// ------------------------------------------------------------------------------------------------ 64-long z lines
// The z-line kernel for grids with 64 <= nz (the 64^3 level of a 256^3 network), any of 16, 32, 64 channels in and
// out: bricks of 64 (z) x 4 (y) x 2 (x) voxels, four M tiles of 64 z x 2 y (128 rows: two z lines).  A stage is one z
// shift dz and one group of 16 input channels: the halo'd box (16 channels, 64 z, 6 y, 4 x) from
// (z0 + dz - 1, y0 - 1, x0 - 1), 32-byte swizzled, whose tile (ty, xx) of tap (dx, dy) starts 2 KB x
// ((2 ty + 1 + dy) + 6 (xx + 1 + dx)) into it, and the weights of the nine taps (dx, dy, dz) for those 16 channels,
// one box (16 channels, Cout, 9) of a copy of the weights whose taps are ordered (dz, dx, dy) (the weights of a
// 64-channel layer do not fit in shared memory whole).  Three stages; otherwise as k_conv_tc_line.
constexpr int kL64Z = 64, kL64Y = 4, kL64X = 2, kL64Stages = 3;

template <int CI, int CO>
struct Line64Layout {
    static constexpr int KP = CI / 16, kTiles = (kL64Y / 2) * kL64X;
    static constexpr uint32_t kABytes = kL64Z * (kL64Y + 2) * (kL64X + 2) * 32u;  // 48 KB
    static constexpr uint32_t kWRaw = 9u * CO * 32u;
    static constexpr uint32_t kWBytes = (kWRaw + 1023u) & ~1023u;
    static constexpr uint32_t kStageBytes = kABytes + kWBytes;
    static constexpr uint32_t kCols = kTiles * CO;
    static constexpr uint32_t kAlloc = 2u * kCols <= 32u ? 32u : 2u * kCols <= 64u ? 64u : 2u * kCols <= 128u ? 128u
                                                                                    : 2u * kCols <= 256u ? 256u
                                                                                                         : 512u;
    static constexpr uint32_t kSmemBytes = 1024u + kL64Stages * kStageBytes + 256u;
    static_assert(CI % 16 == 0 && CO % 16 == 0 && 2u * kCols <= 512u && kSmemBytes <= 227u * 1024u, "layout");
};

template <int CI, int CO, int EPI>
__global__ void __launch_bounds__(192, 1) k_conv_tc_line64(const __grid_constant__ CUtensorMap tmap_x,
                                                           const __grid_constant__ CUtensorMap tmap_wp, Dims d,
                                                           const float *__restrict__ bias, void *__restrict__ yout,
                                                           int *err) {
    using L = Line64Layout<CI, CO>;
    constexpr int KP = L::KP, S = kL64Stages, kTiles = L::kTiles;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + S * L::kStageBytes);
    // barriers: [0,S) stage full, [S,2S) stage empty, [2S,2S+2) accumulators full, [2S+2,2S+4) accumulators empty
    // (four epilogue warps), 2S+4 done
    volatile uint32_t *sh = reinterpret_cast<volatile uint32_t *>(bars + 2 * S + 5);
    // sh: [0] TMEM base, [1] abort, [2] stage jobs issued, [3] stage jobs waited
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + S), tfull0 = smem_u32(bars + 2 * S),
                   tempty0 = smem_u32(bars + 2 * S + 2), done = smem_u32(bars + 2 * S + 4);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int bz_n = (d.nz + kL64Z - 1) / kL64Z, by_n = (d.ny + kL64Y - 1) / kL64Y;
    const long long nbricks = (long long)bz_n * by_n * ((d.nx + kL64X - 1) / kL64X);
    const int nb = nbricks > blockIdx.x ? (int)((nbricks - 1 - blockIdx.x) / gridDim.x + 1) : 0;
    auto brick = [&](int bi, int &z0, int &y0, int &x0) {
        const long long br = blockIdx.x + (long long)bi * gridDim.x;
        z0 = kL64Z * (int)(br % bz_n);
        y0 = kL64Y * (int)((br / bz_n) % by_n);
        x0 = kL64X * (int)(br / ((long long)bz_n * by_n));
    };

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        for (int s = 0; s < 2; s++) {
            mbar_init(tfull0 + 8 * s, 1);
            mbar_init(tempty0 + 8 * s, 4);
        }
        mbar_init(done, 1);
        for (int k = 1; k < 4; k++) sh[k] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(const_cast<uint32_t *>(sh))),
                     "r"(L::kAlloc)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = sh[0];

    if (warp == 1 && lane == 0 && nb > 0) {  // TMA producer
        int q = 0;
        for (int bi = 0; bi < nb && !sh[1]; bi++) {
            int z0, y0, x0;
            brick(bi, z0, y0, x0);
            for (int st = 0; st < 3 * KP && !sh[1]; st++, q++) {  // stage = (dz, 16-channel group)
                const int dz = st / KP, jp = st % KP, s = q % S;
                if (q >= S && !mbar_wait(empty0 + 8 * s, (uint32_t)(q / S - 1) & 1u)) {
                    sh[1] = 1;
                    break;
                }
                const uint32_t a = smem_u32(smem + s * L::kStageBytes);
                mbar_expect_tx(full0 + 8 * s, L::kABytes + L::kWRaw);
                tma_load_4d(a, &tmap_x, full0 + 8 * s, 16 * jp, z0 + dz - 1, y0 - 1, x0 - 1);
                tma_load_3d(a + L::kABytes, &tmap_wp, full0 + 8 * s, 16 * jp, 0, 9 * dz);
                sh[2] = (uint32_t)(q + 1);
            }
        }
    } else if (warp == 0 && lane == 0 && nb > 0) {  // MMA issuer
        constexpr uint32_t idesc = instr_desc_bf16(CO);
        bool any = false;
        int q = 0;
        for (int bi = 0; bi < nb && !sh[1]; bi++) {
            const int tb = bi & 1;
            if (bi >= 2 && !mbar_wait(tempty0 + 8 * tb, (uint32_t)((bi - 2) >> 1) & 1u)) {
                sh[1] = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int st = 0; st < 3 * KP; st++, q++) {
                const int s = q % S;
                if (!mbar_wait(full0 + 8 * s, (uint32_t)(q / S) & 1u)) {
                    sh[1] = 1;
                    break;
                }
                sh[3] = (uint32_t)(q + 1);
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                // descriptor bases of this stage plus compile-time offsets in 16-byte units (no carry: shared
                // addresses stay below 256 KB)
                const uint32_t a = smem_u32(smem + s * L::kStageBytes);
                const uint64_t ad0 = smem_desc_sw32(a), bd0 = smem_desc_sw32(a + L::kABytes);
                const uint32_t tacc = tmem + (uint32_t)(tb * L::kCols);
                const uint32_t acc0 = st > 0 ? 1u : 0u;
#pragma unroll
                for (int pr = 0; pr < 9; pr++) {
                    const int dx = pr / 3 - 1, dy = pr % 3 - 1;
                    const uint64_t bd = bd0 + (uint64_t)(pr * CO * 2);
#pragma unroll
                    for (int tile = 0; tile < kTiles; tile++) {
                        const int ty = tile % (kL64Y / 2), xx = tile / (kL64Y / 2);
                        const uint64_t ad = ad0 + (uint64_t)(128 * ((2 * ty + 1 + dy) + (kL64Y + 2) * (xx + 1 + dx)));
                        mma_bf16(tacc + (uint32_t)(tile * CO), ad, bd, idesc, pr > 0 ? 1u : acc0);
                    }
                }
                any = true;
                mma_commit(empty0 + 8 * s);
            }
            if (sh[1]) break;
            mma_commit(tfull0 + 8 * tb);
        }
        if (any) {  // completion of every MMA issued (also on the error path, before TMEM is released)
            mma_commit(done);
            if (!mbar_wait(done, 0)) sh[1] = 1;
        }
    } else if (warp >= 2 && nb > 0) {  // epilogue
        const int q4 = warp & 3;  // TMEM lane quarter of this warp
        for (int bi = 0; bi < nb; bi++) {
            const int tb = bi & 1;
            const uint32_t par = (uint32_t)(bi >> 1) & 1u;
            // lane 0 decides for the warp, so that the warp-collective TMEM loads below are never divergent
            int go = 0;
            if (lane == 0) go = (!sh[1] && mbar_wait(tfull0 + 8 * tb, par)) ? 1 : 0;
            go = __shfl_sync(0xffffffffu, go, 0);
            if (!go) {
                if (lane == 0) sh[1] = 1;
                break;
            }
            mbar_wait(tfull0 + 8 * tb, par);  // completed: returns at once, with this thread's acquire
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            int z0, y0, x0;
            brick(bi, z0, y0, x0);
            const int m = 32 * q4 + lane;  // TMEM lane = tile row: z = m % 64, y = m / 64
            const int z = z0 + (m & (kL64Z - 1));
#pragma unroll 1
            for (int tile = 0; tile < kTiles; tile++) {
                const int yy = y0 + 2 * (tile % (kL64Y / 2)) + (m >> 6), xx = x0 + tile / (kL64Y / 2);
                const bool inb = z < d.nz && yy < d.ny && xx < d.nx;
                const long long v = inb ? cid(d, xx, yy, z) : 0;
#pragma unroll
                for (int c0 = 0; c0 < CO; c0 += 16) {
                    float acc[16];
                    tmem_ld_x16<16>(tmem + ((uint32_t)(32 * q4) << 16) + (uint32_t)(tb * L::kCols + tile * CO + c0),
                                    acc);
                    if (inb && EPI == 0) {
                        uint32_t pk[8];
#pragma unroll
                        for (int k = 0; k < 8; k++) {
                            const float a0 = fmaxf(acc[2 * k] + bias[c0 + 2 * k], 0.f);
                            const float a1 = fmaxf(acc[2 * k + 1] + bias[c0 + 2 * k + 1], 0.f);
                            __nv_bfloat162 h2 = __floats2bfloat162_rn(a0, a1);
                            pk[k] = *reinterpret_cast<uint32_t *>(&h2);
                        }
                        uint4 *dst = reinterpret_cast<uint4 *>(reinterpret_cast<__nv_bfloat16 *>(yout) + v * CO + c0);
                        dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                        dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
                    } else if (inb) {
                        float4 *dst = reinterpret_cast<float4 *>(reinterpret_cast<float *>(yout) + v * CO + c0);
#pragma unroll
                        for (int k = 0; k < 4; k++)
                            dst[k] = make_float4(acc[4 * k], acc[4 * k + 1], acc[4 * k + 2], acc[4 * k + 3]);
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tempty0 + 8 * tb) : "memory");
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && sh[1]) {  // drain copies still in flight into this CTA's shared memory (bounded)
        for (uint32_t q = sh[3]; q < sh[2]; q++) mbar_wait(full0 + 8 * (q % S), (q / S) & 1u);
        atomicCAS(err, 0, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(L::kAlloc) : "memory");
    }
}

// ------------------------------------------------------------------------------------------------ weight gradient
// dW[tap][co][ci] = sum over voxels v of dY[v][co] X[v + off(tap)][ci]: GEMMs with M = Cout, K = voxels and
// N = (dz, Cin), both operands K-major with 8 consecutive z per 16-byte row.  k_to_chmajor makes channel-major copies
// with z split into 8-voxel rows: dYT[zh][x][y][co][zl] and XT[zh][x][y][s][ci][zl] = X[x][y][8 zh + zl + s - 1][ci]
// (zero outside), the three z shifts s = dz + 1 interleaved per row so that one TMA box starting on a row boundary
// carries all three.  A job is one (dx, dy) pair over one brick of 32 (z) x 4 (y) x BX (x) voxels: one 5-D TMA box
// (8, C, 4, BX, 4) lands as rows c + C k of 16 B, k = y + 4 (x + BX zh) the K index of the 8-voxel core matrices,
// so consecutive K steps are C x 16 B apart (LBO) and 8-row groups 128 B (SBO); the y and x shifts are box
// coordinates (outside the grid: zero fill).  One MMA (K = 16) then accumulates the three taps (dx, dy, -1..1) into
// 3 Cin TMEM columns.  M = 128 rows of which the first Cout are dY channels; the rows past them read the next K
// steps' rows (or a zeroed slack after the buffer) and land in accumulator lanes that are never read.
// One CTA (one per SM, 512 TMEM columns) runs a group of (dx, dy) pairs over a strided set of bricks, warp
// specialised: lane 0 of warp 1 issues the TMA loads (dY of a brick once, into one of two buffers; X per pair through
// a ring of stages), lane 0 of warp 0 the MMAs, so neither waits on the other's latency.  The CTA writes its partial
// sums part[chunk][tap][co][ci] (FP32), reduced over chunks in fixed order afterwards.  Every wait is bounded as in
// k_conv_tc.
constexpr uint32_t kWgSlack = 2048;

template <int CI>
__host__ __device__ constexpr int wg_bx() {  // x extent of a brick
    return CI == 16 ? 2 : 1;
}
// (dx, dy) pairs per CTA: 3 CI columns each, at most 512
template <int CI>
__host__ __device__ constexpr int wg_pairs_per_cta() {
    return CI == 16 ? 9 : CI == 32 ? 5 : 2;
}

template <int CI, int CO>
struct WgLayout {
    static constexpr int BX = wg_bx<CI>();
    static constexpr uint32_t kABytes = 256u * CO * BX;  // 8 z x CO x 4 y x BX x x 4 zh, BF16
    static constexpr uint32_t kBBytes = 768u * CI * BX;  // 8 z x 3 CI x 4 y x BX x x 4 zh
    static constexpr uint32_t kAStride = kABytes + kWgSlack;
    static constexpr int kStagesRaw = (int)((216u * 1024u - 2u * kAStride) / kBBytes);
    static constexpr int kStages = kStagesRaw > 8 ? 8 : kStagesRaw;
    static constexpr uint32_t kNeed = 2u * kAStride + kStages * kBBytes + 1024u + 512u;
    // at least 116 KB: one CTA per SM, whose 512 TMEM columns are then always free
    static constexpr uint32_t kSmemBytes = kNeed > 116u * 1024u ? kNeed : 116u * 1024u;
    static_assert(kStages >= 2 && kSmemBytes <= 227u * 1024u, "shared memory");
};

// dst[zh][x][y][s][c][zl] = src[x][y][8 zh + zl + s + shift0][c] where 8 zh + zl < nz and the shifted z lies in the
// grid, else 0; s < ns, zh < nzh = ceil(nz / 8).  One thread per (zh, x, y, c): 16-byte stores.
template <int C>
__global__ void __launch_bounds__(256) k_to_chmajor(Dims d, int ns, int shift0, const __nv_bfloat16 *__restrict__ src,
                                                    __nv_bfloat16 *__restrict__ dst) {
    const int nzh = (d.nz + 7) / 8;
    const long long m = (long long)nzh * d.nx * d.ny * C;
    const unsigned short *s16 = reinterpret_cast<const unsigned short *>(src);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % C);
        const long long r = e / C;  // ((zh nx + x) ny + y)
        const int y = (int)(r % d.ny);
        const long long t = r / d.ny;
        const int x = (int)(t % d.nx), zh = (int)(t / d.nx);
        const long long row = (((long long)x * d.ny + y) * d.nz) * C + c;  // src index of (x, y, 0, c)
        for (int s = 0; s < ns; s++) {
            uint32_t w[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                uint32_t h[2];
#pragma unroll
                for (int u = 0; u < 2; u++) {
                    const int z = 8 * zh + 2 * q + u, zs = z + s + shift0;
                    h[u] = (z < d.nz && zs >= 0 && zs < d.nz) ? (uint32_t)s16[row + (long long)zs * C] : 0u;
                }
                w[q] = h[0] | (h[1] << 16);
            }
            *reinterpret_cast<uint4 *>(dst + ((r * ns + s) * C + c) * 8) = make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
}

template <int CI, int CO>
__global__ void __launch_bounds__(128, 1) k_wgrad_tc(const __grid_constant__ CUtensorMap tmap_dy,
                                                     const __grid_constant__ CUtensorMap tmap_x, Dims d,
                                                     float *__restrict__ part, int *err) {
    constexpr int NP = wg_pairs_per_cta<CI>();
    constexpr int N = 3 * CI;
    static_assert(NP * N <= 512 && CO <= 128 && CI % 16 == 0 && CO % 16 == 0 && N <= 256, "shape");
    using L = WgLayout<CI, CO>;
    constexpr int S = L::kStages, BX = L::BX;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *abuf = smem, *bbuf = smem + 2 * L::kAStride;
    uint64_t *bars = reinterpret_cast<uint64_t *>(bbuf + S * L::kBBytes);
    // [0, 2) dY full, [2, 4) dY empty, [4, 4 + S) X full, [4 + S, 4 + 2S) X empty, then done
    // sh: [0] TMEM base, [1] status, [2] MMA side ok, [3] X jobs waited, [4] bricks waited, [5] TMA side ok,
    //     [6] X jobs issued, [7] bricks issued
    volatile uint32_t *sh = reinterpret_cast<volatile uint32_t *>(bars + 4 + 2 * S + 1);
    const uint32_t afull0 = smem_u32(bars), aempty0 = smem_u32(bars + 2), bfull0 = smem_u32(bars + 4),
                   bempty0 = smem_u32(bars + 4 + S), done = smem_u32(bars + 4 + 2 * S);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int pair0 = blockIdx.y * NP, npair = min(NP, 9 - pair0);
    const int bz_n = (d.nz + 31) / 32, by_n = (d.ny + 3) / 4, bx_n = (d.nx + BX - 1) / BX;
    const long long nbricks = (long long)bz_n * by_n * bx_n;
    const int nb = nbricks > blockIdx.x ? (int)((nbricks - 1 - blockIdx.x) / gridDim.x + 1) : 0;
    const int J = nb * npair;

    // zero the slack after each dY buffer (read by the MMA rows past Cout)
    for (uint32_t i = threadIdx.x; i < kWgSlack / 16; i += blockDim.x) {
        reinterpret_cast<uint4 *>(abuf + L::kABytes)[i] = make_uint4(0, 0, 0, 0);
        reinterpret_cast<uint4 *>(abuf + L::kAStride + L::kABytes)[i] = make_uint4(0, 0, 0, 0);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (threadIdx.x == 0) {
        for (int s = 0; s < 2; s++) {
            mbar_init(afull0 + 8 * s, 1);
            mbar_init(aempty0 + 8 * s, 1);
        }
        for (int s = 0; s < S; s++) {
            mbar_init(bfull0 + 8 * s, 1);
            mbar_init(bempty0 + 8 * s, 1);
        }
        mbar_init(done, 1);
        for (int k = 1; k < 8; k++) sh[k] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(const_cast<uint32_t *>(sh))),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = sh[0];

    auto brick = [&](int bi, int &z0, int &y0, int &x0) {
        const long long br = blockIdx.x + (long long)bi * gridDim.x;
        z0 = 32 * (int)(br % bz_n);
        y0 = 4 * (int)((br / bz_n) % by_n);
        x0 = BX * (int)(br / ((long long)bz_n * by_n));
    };
    if (warp == 1 && lane == 0) {  // TMA producer
        bool ok = true;
        int a_issued = 0, b_issued = 0;
        for (int q = 0; q < J && ok; q++) {
            const int bi = q / npair, jj = q % npair;
            int z0, y0, x0;
            brick(bi, z0, y0, x0);
            if (jj == 0) {
                const int ab = bi & 1;
                if (bi >= 2 && !mbar_wait(aempty0 + 8 * ab, (uint32_t)((bi - 2) >> 1) & 1u)) {
                    ok = false;
                    break;
                }
                mbar_expect_tx(afull0 + 8 * ab, L::kABytes);
                tma_load_5d(smem_u32(abuf + ab * L::kAStride), &tmap_dy, afull0 + 8 * ab, 0, 0, y0, x0, z0 / 8);
                a_issued = bi + 1;
            }
            const int pr = pair0 + jj, dx = pr / 3 - 1, dy = pr % 3 - 1;
            const int s = q % S;
            if (q >= S && !mbar_wait(bempty0 + 8 * s, (uint32_t)(q / S - 1) & 1u)) {
                ok = false;
                break;
            }
            mbar_expect_tx(bfull0 + 8 * s, L::kBBytes);
            tma_load_5d(smem_u32(bbuf + s * L::kBBytes), &tmap_x, bfull0 + 8 * s, 0, 0, y0 + dy, x0 + dx, z0 / 8);
            b_issued = q + 1;
        }
        sh[5] = ok ? 1u : 0u;
        sh[6] = (uint32_t)b_issued;
        sh[7] = (uint32_t)a_issued;
    } else if (warp == 0 && lane == 0) {  // MMA issuer
        constexpr uint32_t idesc = instr_desc_bf16(N);
        bool ok = true;
        int a_waited = 0, b_waited = 0;
        for (int q = 0; q < J; q++) {
            const int bi = q / npair, jj = q % npair, ab = bi & 1, s = q % S;
            if (jj == 0) {
                if (!mbar_wait(afull0 + 8 * ab, (uint32_t)(bi >> 1) & 1u)) {
                    ok = false;
                    break;
                }
                a_waited = bi + 1;
            }
            if (!mbar_wait(bfull0 + 8 * s, (uint32_t)(q / S) & 1u)) {
                ok = false;
                break;
            }
            b_waited = q + 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint64_t ad0 = smem_desc(smem_u32(abuf + ab * L::kAStride), (uint32_t)CO * 16u, 128u);
            const uint64_t bd0 = smem_desc(smem_u32(bbuf + s * L::kBBytes), (uint32_t)N * 16u, 128u);
#pragma unroll
            for (int p = 0; p < 8 * BX; p++)  // start addresses advance in 16-byte units (no carry: < 256 KB)
                mma_bf16(tmem + (uint32_t)(jj * N), ad0 + (uint64_t)(2 * p * CO), bd0 + (uint64_t)(2 * p * N), idesc,
                         (bi > 0 || p > 0) ? 1u : 0u);
            mma_commit(bempty0 + 8 * s);
            if (jj == npair - 1) mma_commit(aempty0 + 8 * ab);
        }
        if (b_waited > 0) {  // completion of every MMA issued (also on the error path, before TMEM is released)
            mma_commit(done);
            if (!mbar_wait(done, 0)) ok = false;
        }
        sh[2] = ok ? 1u : 0u;
        sh[3] = (uint32_t)b_waited;
        sh[4] = (uint32_t)a_waited;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const bool ok = sh[2] && sh[5];
        if (!ok) {  // drain copies still in flight into this CTA's shared memory (bounded)
            for (uint32_t q = sh[3]; q < sh[6]; q++) mbar_wait(bfull0 + 8 * (q % S), (q / S) & 1u);
            for (uint32_t q = sh[4]; q < sh[7]; q++) mbar_wait(afull0 + 8 * (q & 1), (q >> 1) & 1u);
            atomicCAS(err, 0, 1);
        }
        sh[1] = ok ? (J > 0 ? 1u : 2u) : 0u;
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t st = sh[1];
    if (st != 0 && 32 * warp < CO) {  // 1: the accumulators hold this CTA's sums; 2: no brick, the sums are zero
        const int co = 32 * warp + lane;  // TMEM lane = dY channel
        for (int jj = 0; jj < npair; jj++) {
#pragma unroll
            for (int sz = 0; sz < 3; sz++) {
                float *out = part + (((long long)blockIdx.x * 27 + 3 * (pair0 + jj) + sz) * CO) * CI;
#pragma unroll
                for (int c0 = 0; c0 < CI; c0 += 16) {
                    float acc[16];
                    if (st == 1) {
                        tmem_ld_x16<16>(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(jj * N + sz * CI + c0), acc);
                    } else {
#pragma unroll
                        for (int q = 0; q < 16; q++) acc[q] = 0.f;
                    }
                    if (co < CO) {
                        float4 *dst = reinterpret_cast<float4 *>(out + (long long)co * CI + c0);
#pragma unroll
                        for (int q = 0; q < 4; q++)
                            dst[q] = make_float4(acc[4 * q], acc[4 * q + 1], acc[4 * q + 2], acc[4 * q + 3]);
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
    }
}

}  // namespace tc
}  // namespace sf
