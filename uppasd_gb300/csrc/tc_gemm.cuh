// tc_gemm.cuh -- BF16 tensor-core GEMM for sm_103a: C = A * B^T with FP32
// accumulation in tensor memory, operands staged by TMA.
//
//   A : M x K, K contiguous (row-major), bf16        M % 128 == 0
//   B : N x K, K contiguous (row-major), bf16        N % BN == 0
//   K % 64 == 0; every pointer 16-byte aligned.
//
// One CTA computes a 128 x BN tile.  Four warps: warp 0 lane 0 issues the TMA
// loads (64-wide K slices, 128-byte swizzle, a ring of kStages stages guarded
// by full/empty mbarriers), warp 1 lane 0 issues tcgen05.mma (M = 128, N = BN,
// K = 16 per instruction, accumulator in TMEM columns [0, BN)), and after the
// last MMA commits, all four warps read the accumulator back with tcgen05.ld
// (warp w owns TMEM lanes 32w..32w+31 = tile rows) and apply the fused epilogue.
//
// Every mbarrier wait is bounded; a wait that runs out records an error code in
// *err and the kernel still walks the rest of its protocol (each remaining wait
// bounded too), frees its TMEM and returns.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace uppasd {
namespace tc {

constexpr int kBM = 128;
constexpr int kBK = 64;       // bf16 elements per K slice = one 128-byte swizzle row
constexpr int kMaxStages = 4;
constexpr int kThreads = 128;
// a pipeline wait gives up after about a second of %globaltimer time
constexpr long long kWaitLimitNs = 1000000000LL;

enum Epilogue : int {
    kEpiStoreF32 = 0,     // C_f32 = acc
    kEpiBiasF32 = 1,      // C_f32 = acc + bias[n]
    kEpiBiasTanhBF16 = 2, // C_bf16 = tanh(acc + bias[n])
    kEpiDTanhBF16 = 3,    // C_bf16 = acc * (1 - Y[m,n]^2), Y bf16 (M x N)
};

struct GemmArgs {
    int M, N, K;
    const float *bias;          // kEpiBias*
    const __nv_bfloat16 *Y;     // kEpiDTanhBF16
    float *Cf;                  // f32 outputs, M x N row-major
    __nv_bfloat16 *Cb;          // bf16 outputs, M x N row-major
    int *err;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ long long tc_globaltimer() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait for the phase with parity `parity` to complete; false once about
// kWaitLimitNs have passed.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    long long t0 = 0;
    for (long long it = 0;; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (it == 64) t0 = tc_globaltimer();
        if (it > 64) {
            if ((it & 63) == 0 && tc_globaltimer() - t0 > kWaitLimitNs) return false;
            __nanosleep(64);
        }
    }
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, rows of
// 128 bytes, 8-row groups 1024 bytes apart (stride byte offset), version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);        // start address
    d |= (uint64_t)1 << 16;                        // leading byte offset (unused with this swizzle)
    d |= (uint64_t)(1024 >> 4) << 32;              // stride byte offset
    d |= (uint64_t)1 << 46;                        // descriptor version
    d |= (uint64_t)2 << 61;                        // 128-byte swizzle
    return d;
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4)                       // D format F32
           | (1u << 7)                     // A format BF16
           | (1u << 10)                    // B format BF16
           | ((uint32_t)(N >> 3) << 17)    // N / 8
           | ((uint32_t)(M >> 4) << 24);   // M / 16
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float tanh_fast(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

template <int BN, int EPI, int kStages>
__global__ void __launch_bounds__(kThreads, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, GemmArgs g) {
    static_assert(kStages >= 1 && kStages <= kMaxStages, "stages");
    static_assert(BN == 64 || BN == 128 || BN == 256, "BN");
    constexpr uint32_t kABytes = kBM * kBK * 2, kBBytes = BN * kBK * 2;
    constexpr uint32_t kStageBytes = kABytes + kBBytes;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // 1024-byte alignment of every tile (the swizzle atom)
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t full[kStages], empty[kStages], done;
    __shared__ uint32_t tmem_base_s;
    __shared__ int failed;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
    const int nk = g.K / kBK;

    if (threadIdx.x == 0) {
        failed = 0;
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                     "r"((uint32_t)BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_s;

    if (warp == 0 && lane == 0) {
        // producer: fill the ring; a stage is refilled once the MMAs reading it have committed
        for (int kb = 0; kb < nk; ++kb) {
            const int s = kb % kStages;
            if (kb >= kStages && !mbar_wait(&empty[s], ((kb / kStages) - 1) & 1)) {
                failed = 1;
                atomicExch(g.err, 1);
            }
            uint8_t *sa = smem + s * kStageBytes;
            mbar_expect_tx(&full[s], kStageBytes);
            tma_load_2d(sa, &mapA, &full[s], kb * kBK, m0);
            tma_load_2d(sa + kABytes, &mapB, &full[s], kb * kBK, n0);
        }
    } else if (warp == 1 && lane == 0) {
        constexpr uint32_t idesc = idesc_bf16(kBM, BN);
        for (int kb = 0; kb < nk; ++kb) {
            const int s = kb % kStages;
            if (!mbar_wait(&full[s], (kb / kStages) & 1)) {
                failed = 1;
                atomicExch(g.err, 2);
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = smem_u32(smem + s * kStageBytes);
            const uint32_t sb = sa + kABytes;
#pragma unroll
            for (int k = 0; k < kBK / 16; ++k) {
                // advancing K by 16 elements = 32 bytes inside the 128-byte swizzled row
                mma_bf16(tmem, sw128_desc(sa + k * 32), sw128_desc(sb + k * 32), idesc, (kb | k) ? 1u : 0u);
            }
            mma_commit(&empty[s]);
        }
        mma_commit(&done);
    }
    __syncwarp();
    // epilogue: one lane per warp waits for the accumulator, then the warp reconverges
    // (tcgen05.ld is warp-collective)
    if (lane == 0 && !mbar_wait(&done, 0)) {
        failed = 1;
        atomicExch(g.err, 3);
    }
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int row = m0 + warp * 32 + lane;
    const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
    for (int c = 0; c < BN; c += 16) {
        float v[16];
        tmem_ld16(tl + c, v);
        const int col = n0 + c;
        if (EPI == kEpiStoreF32 || EPI == kEpiBiasF32) {
            float4 *o = reinterpret_cast<float4 *>(g.Cf + (size_t)row * g.N + col);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float4 w = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                if (EPI == kEpiBiasF32) {
                    w.x += g.bias[col + 4 * q];
                    w.y += g.bias[col + 4 * q + 1];
                    w.z += g.bias[col + 4 * q + 2];
                    w.w += g.bias[col + 4 * q + 3];
                }
                o[q] = w;
            }
        } else {
            __align__(16) __nv_bfloat16 h[16];
            if (EPI == kEpiBiasTanhBF16) {
#pragma unroll
                for (int i = 0; i < 16; ++i) h[i] = __float2bfloat16_rn(tanh_fast(v[i] + g.bias[col + i]));
            } else {
                __align__(16) __nv_bfloat16 y[16];
                const uint4 *ys = reinterpret_cast<const uint4 *>(g.Y + (size_t)row * g.N + col);
                *reinterpret_cast<uint4 *>(&y[0]) = ys[0];
                *reinterpret_cast<uint4 *>(&y[8]) = ys[1];
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const float t = __bfloat162float(y[i]);
                    h[i] = __float2bfloat16_rn(v[i] * (1.0f - t * t));
                }
            }
            uint4 *o = reinterpret_cast<uint4 *>(g.Cb + (size_t)row * g.N + col);
            o[0] = *reinterpret_cast<const uint4 *>(&h[0]);
            o[1] = *reinterpret_cast<const uint4 *>(&h[8]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)BN)
                     : "memory");
    }
}

template <int BN, int STAGES>
constexpr size_t gemm_smem_bytes() {
    return (size_t)STAGES * (kBM * kBK * 2 + BN * kBK * 2) + 1024;
}

}  // namespace tc
}  // namespace uppasd
