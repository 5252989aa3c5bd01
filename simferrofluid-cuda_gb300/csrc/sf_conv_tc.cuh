// sf_conv_tc.cuh -- 3x3x3 convolution forward on the 5th-generation tensor cores (tcgen05 + TMA, sm_103a).
//
// Implicit GEMM per CTA: MT tiles of M = 128 output voxels (a 32 (z) x 4 MT (y) x 1 (x) brick), N = Cout,
// K = 27 taps x Cin.  Operands are staged by TMA in the no-swizzle K-major "core matrix" layout: one 4-D box of
// 8 channels x (32 x 4 MT x 1) voxels per 8-channel chunk and tap lands as 128 MT rows x 16 B, i.e. 8-row x 16-B
// core matrices with a 128-B stride along M, one tile per 2 KB and one (2 MT)-KB chunk per 8 channels along K;
// taps outside the grid are filled with zeros by the TMA unit (the convolution's zero padding).  Weights
// [tap][Cout][Cin] are staged the same way, once per tap for all MT tiles.  One thread issues TMA loads and
// tcgen05.mma (M=128, N=Cout, K=16, BF16 in, FP32 accumulate in TMEM, one accumulator of Cout columns per tile)
// through a ring of stages guarded by mbarriers; all four warps read the accumulators back with tcgen05.ld and
// apply bias + ReLU + BF16 conversion.  Every wait is bounded: on timeout the CTA records an error code and
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
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * kStages + 1);  // [0] TMEM base, [1] status
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
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(L::kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    volatile int *flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    if (threadIdx.x == 0) {
        constexpr uint32_t idesc = instr_desc_bf16(CO);
        constexpr int T = 27;
        int issued = 0, waited = 0;
        bool ok = true;
        auto load = [&](int t, int s) {
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
        };
        for (int t = 0; t < kStages && t < T; t++) load(t, t);
        for (int t = 0; t < T; t++) {
            const int s = t % kStages;
            const uint32_t ph = (uint32_t)(t / kStages) & 1u;
            if (!mbar_wait(full0 + 8 * s, ph)) {
                ok = false;
                break;
            }
            waited = t + 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a = smem_u32(smem + s * L::kStageBytes), b = a + L::kABytes;
#pragma unroll
            for (int j = 0; j < CI / 16; j++) {
                // K = 16 spans two 8-channel chunks: leading (K) offset = one chunk, stride (M/N) = 8 rows;
                // tile m's rows start 2 KB further into each chunk, its accumulator CO columns further
                const uint64_t bd = smem_desc(b + j * 2u * (uint32_t)CO * 16u, (uint32_t)CO * 16u, 128u);
#pragma unroll
                for (int m = 0; m < MT; m++) {
                    const uint64_t ad = smem_desc(a + j * 2u * L::kChunkBytes + (uint32_t)m * 2048u, L::kChunkBytes,
                                                  128u);
                    mma_bf16(tmem + (uint32_t)(m * CO), ad, bd, idesc, (t > 0 || j > 0) ? 1u : 0u);
                }
            }
            mma_commit(empty0 + 8 * s);
            if (t + kStages < T) {
                if (!mbar_wait(empty0 + 8 * s, ph)) {
                    ok = false;
                    break;
                }
                load(t + kStages, s);
            }
        }
        // completion of every MMA issued so far (also on the error path, before TMEM is released)
        mma_commit(done);
        if (!mbar_wait(done, 0)) ok = false;
        if (!ok) {
            // drain loads still in flight into this CTA's shared memory (bounded)
            for (int t = waited; t < issued; t++) mbar_wait(full0 + 8 * (t % kStages), (uint32_t)(t / kStages) & 1u);
            atomicCAS(err, 0, 1);
        }
        *flag = ok ? 1 : 0;
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (*flag) {  // uniform across the CTA
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

}  // namespace tc
}  // namespace sf
