// tc_mlp.cuh -- the learned proposal's whole forward pass (192 -> 256 -> 256 -> 256 -> 64,
// tanh hidden layers) in one kernel per 128-row tile, activations kept on chip.
//
// Per CTA: the 128 x 192 input tile arrives by TMA (128-byte swizzle) in the
// activation buffer A; for each layer the weight matrix streams through a
// 4-stage TMA ring in 64-column K slices, one thread issues tcgen05.mma
// (M = 128, N = 256 or 64, K = 16) into TMEM columns [0, N), and the four compute
// warps read the accumulator back (tcgen05.ld, warp w = rows 32w..32w+31), apply
// bias + tanh, round to bf16 and write the result into A in the same swizzled
// K-major layout the next layer's MMAs read.  Eight compute warps share the
// epilogue: warps w and w + 4 read the same TMEM lane quadrant (w % 4, the rows
// 32 (w % 4) .. + 31) and take one half of the columns each.  The last layer writes
// fp32 outputs (bias, no activation) to global memory.  A ninth warp is the TMA
// producer, so the compute warps' named barrier never waits on it.
//
// Shared memory: A 64 KB (the input tile uses 48 KB of it, then each hidden
// layer's activations) + ring 4 x 32 KB.  TMEM: 256 columns.  Every wait is
// bounded; a wait that runs out records an error code and the kernel finishes
// its protocol and frees TMEM.
#pragma once
#include "tc_gemm.cuh"

namespace uppasd {
namespace tc {

constexpr int kMlpIn = 192, kMlpHid = 256, kMlpOut = 64;
constexpr int kMlpCompute = 8;                    // compute warps (two per TMEM lane quadrant)
constexpr int kMlpThreads = 32 * (kMlpCompute + 1); // + 1 producer warp
constexpr uint32_t kMlpABytes = 128 * 256 * 2;    // activation tile: 4 K-slices of 16 KB
constexpr uint32_t kMlpStageBytes = 256 * 64 * 2; // one weight K-slice (N <= 256)
constexpr int kMlpStages = 4;
constexpr int kMlpChunks = 3 + 4 + 4 + 4;         // weight K-slices over the four layers

struct MlpArgs {
    const float *bias[4];
    float *out;  // rows x 64 fp32
    int rows;
    int *err;
};

__host__ __device__ constexpr int mlp_layer_of_chunk(int g) { return g < 3 ? 0 : (g - 3) / 4 + 1; }
__host__ __device__ constexpr int mlp_k_of_chunk(int g) { return g < 3 ? g : (g - 3) % 4; }
__host__ __device__ constexpr int mlp_n(int l) { return l == 3 ? kMlpOut : kMlpHid; }
__host__ __device__ constexpr int mlp_kslices(int l) { return l == 0 ? 3 : 4; }

__device__ __forceinline__ void named_bar_compute() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

__global__ void __launch_bounds__(kMlpThreads, 1)
    tc_mlp_kernel(const __grid_constant__ CUtensorMap mapX, const __grid_constant__ CUtensorMap mapW0,
                  const __grid_constant__ CUtensorMap mapW1, const __grid_constant__ CUtensorMap mapW2,
                  const __grid_constant__ CUtensorMap mapW3, MlpArgs a) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint8_t *abuf = smem;                    // activations (K-major, swizzled, 4 slices of 128 x 64)
    uint8_t *ring = smem + kMlpABytes;       // weight slices
    __shared__ __align__(8) uint64_t full[kMlpStages], empty[kMlpStages], xfull, done;
    __shared__ uint32_t tmem_base_s;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * 128;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kMlpStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&xfull, 1);
        mbar_init(&done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                     "r"(256u)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_s;

    if (warp == kMlpCompute) {
        // producer: the input tile, then every weight K-slice of every layer through the ring
        if (lane == 0) {
            mbar_expect_tx(&xfull, 128 * kMlpIn * 2);
            for (int k = 0; k < 3; ++k) tma_load_2d(abuf + k * 16384, &mapX, &xfull, k * 64, m0);
            const CUtensorMap *maps[4] = {&mapW0, &mapW1, &mapW2, &mapW3};
            for (int g = 0; g < kMlpChunks; ++g) {
                const int s = g % kMlpStages, l = mlp_layer_of_chunk(g), k = mlp_k_of_chunk(g);
                if (g >= kMlpStages && !mbar_wait(&empty[s], ((g / kMlpStages) - 1) & 1)) atomicExch(a.err, 11);
                mbar_expect_tx(&full[s], (uint32_t)mlp_n(l) * 64 * 2);
                tma_load_2d(ring + s * kMlpStageBytes, maps[l], &full[s], k * 64, 0);
            }
        }
    } else {
        int g = 0;
        for (int l = 0; l < 4; ++l) {
            const int N = mlp_n(l);
            // MMAs of layer l (one thread); the activations in abuf are complete
            if (warp == 1 && lane == 0) {
                if (l == 0 && !mbar_wait(&xfull, 0)) atomicExch(a.err, 12);
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t idesc = idesc_bf16(128, N);
                for (int k = 0; k < mlp_kslices(l); ++k, ++g) {
                    const int s = g % kMlpStages;
                    if (!mbar_wait(&full[s], (g / kMlpStages) & 1)) atomicExch(a.err, 13);
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t sa = smem_u32(abuf + k * 16384), sb = smem_u32(ring + s * kMlpStageBytes);
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        mma_bf16(tmem, sw128_desc(sa + q * 32), sw128_desc(sb + q * 32), idesc, (k | q) ? 1u : 0u);
                    mma_commit(&empty[s]);
                }
                mma_commit(&done);
            }
            __syncwarp();
            if (lane == 0 && !mbar_wait(&done, l & 1)) atomicExch(a.err, 14);
            __syncwarp();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // epilogue: row r = 32 (warp % 4) + lane, column half warp / 4, slices of 16
            const int quad = warp & 3, half = warp >> 2;
            const int r = quad * 32 + lane;
            const uint32_t tl = tmem + ((uint32_t)(quad * 32) << 16);
            const float *bias = a.bias[l];
            for (int c = half * (N / 2); c < (half + 1) * (N / 2); c += 16) {
                float v[16];
                tmem_ld16(tl + c, v);
                if (l < 3) {
                    __align__(16) __nv_bfloat16 h[16];
#pragma unroll
                    for (int i = 0; i < 16; ++i) h[i] = __float2bfloat16_rn(tanh_fast(v[i] + bias[c + i]));
                    // K-major 128-byte swizzle: slice c/64, 16-byte chunk ((c%64)/8 + j) ^ (r%8)
                    uint8_t *rowp = abuf + (c >> 6) * 16384 + r * 128;
                    const int ch = (c & 63) >> 3;
#pragma unroll
                    for (int j = 0; j < 2; ++j)
                        *reinterpret_cast<uint4 *>(rowp + (((ch + j) ^ (r & 7)) << 4)) =
                            *reinterpret_cast<const uint4 *>(&h[8 * j]);
                } else if (m0 + r < a.rows) {
                    float4 *o = reinterpret_cast<float4 *>(a.out + (size_t)(m0 + r) * kMlpOut + c);
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        o[q] = make_float4(v[4 * q] + bias[c + 4 * q], v[4 * q + 1] + bias[c + 4 * q + 1],
                                           v[4 * q + 2] + bias[c + 4 * q + 2], v[4 * q + 3] + bias[c + 4 * q + 3]);
                }
            }
            // the next layer's MMAs read abuf (async proxy) and overwrite TMEM
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            named_bar_compute();
        }
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256u) : "memory");
    }
}

constexpr size_t mlp_smem_bytes() { return (size_t)kMlpABytes + kMlpStages * kMlpStageBytes + 1024; }

}  // namespace tc
}  // namespace uppasd
