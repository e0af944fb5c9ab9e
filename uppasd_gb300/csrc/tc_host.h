// tc_host.h -- host interface of the tcgen05 GEMM (tc_gemm.cuh).
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace uppasd {
namespace tc {

// A prepared GEMM: shapes, epilogue, tile width and the two TMA tensor maps.
struct Gemm {
    CUtensorMap ma, mb;
    int M = 0, N = 0, K = 0, epi = 0, bn = 0, stages = 4;
};

// C(M x N) = A(M x K) B(N x K)^T; A, B device bf16 row-major.  Checks shapes and alignment.
// stages: depth of the TMA ring (2 or 4; 2 lets more CTAs share an SM when K is short).
int gemm_prepare(Gemm &op, const __nv_bfloat16 *A, const __nv_bfloat16 *B, int M, int N, int K, int epi, int bn,
                 int stages = 4);
// 2-D bf16 TMA map over a rows x cols row-major matrix (box 64 columns x box_rows,
// 128-byte swizzle); checks base alignment and row pitch.
int make_map(CUtensorMap *m, const void *ptr, int rows, int cols, int box_rows);
// Any tiled TMA map (no interleave, no swizzle, L2 promotion 128 B, out-of-range
// elements filled with zeros): rank <= 5, dims / box innermost first, strides in bytes
// of dims 1 .. rank-1.  Checks the 16-byte rules on the base, strides and inner box.
int encode_tiled(CUtensorMap *m, CUtensorMapDataType dt, int elem_bytes, int rank, const void *ptr,
                 const uint64_t *dims, const uint64_t *strides, const uint32_t *box);
// Launch on `st` (capturable).  Outputs/extra operands by epilogue (see tc_gemm.cuh).
int gemm_run(const Gemm &op, const float *bias, const __nv_bfloat16 *Y, float *Cf, __nv_bfloat16 *Cb, int *err,
             cudaStream_t st);

}  // namespace tc
}  // namespace uppasd
