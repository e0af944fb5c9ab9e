// tc_host.cu -- host side of the tcgen05 GEMM: TMA tensor maps (cuTensorMapEncodeTiled,
// reached through the runtime's driver entry point so nothing links libcuda), the
// launcher that checks every shape and alignment rule before a launch, and a
// host-buffer entry point used to validate the kernel against a CPU product.
#include <mutex>
#include <string>

#include "sim.h"
#include "tc_gemm.cuh"
#include "tc_host.h"

namespace uppasd {
namespace tc {

namespace {
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn g_encode = nullptr;
std::mutex g_encode_mu;

int encode_fn() {
    std::lock_guard<std::mutex> lk(g_encode_mu);
    if (g_encode) return UPPASD_GPU_OK;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
        set_error("tensor-map encoder unavailable from the driver");
        return UPPASD_GPU_ECUDA;
    }
    g_encode = reinterpret_cast<EncodeTiledFn>(fn);
    return UPPASD_GPU_OK;
}

}  // namespace

// 2-D bf16 map over a rows x cols row-major matrix, box = 64 columns x box_rows, 128-byte swizzle
int make_map(CUtensorMap *m, const void *ptr, int rows, int cols, int box_rows) {
    int rc = encode_fn();
    if (rc) return rc;
    if ((reinterpret_cast<uintptr_t>(ptr) & 15) || (cols * 2) % 16) {
        set_error("tensor map: base must be 16-byte aligned and rows a multiple of 16 bytes");
        return UPPASD_GPU_EINVAL;
    }
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
    cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed with " + std::to_string((int)r));
        return UPPASD_GPU_ECUDA;
    }
    return UPPASD_GPU_OK;
}

int encode_tiled(CUtensorMap *m, CUtensorMapDataType dt, int elem_bytes, int rank, const void *ptr,
                 const uint64_t *dims, const uint64_t *strides, const uint32_t *box) {
    int rc = encode_fn();
    if (rc) return rc;
    if (rank < 1 || rank > 5 || (reinterpret_cast<uintptr_t>(ptr) & 15) || ((uint64_t)box[0] * elem_bytes) % 16) {
        set_error("tensor map: rank 1..5, 16-byte aligned base and inner box a multiple of 16 bytes");
        return UPPASD_GPU_EINVAL;
    }
    cuuint64_t d[5], st[4];
    cuuint32_t b[5], es[5];
    for (int i = 0; i < rank; ++i) {
        d[i] = dims[i];
        b[i] = box[i];
        es[i] = 1;
        if (box[i] < 1 || box[i] > 256) {
            set_error("tensor map: box extents must be 1..256");
            return UPPASD_GPU_EINVAL;
        }
    }
    for (int i = 0; i + 1 < rank; ++i) {
        st[i] = strides[i];
        if (strides[i] % 16) {
            set_error("tensor map: strides must be multiples of 16 bytes");
            return UPPASD_GPU_EINVAL;
        }
    }
    CUresult r = g_encode(m, dt, (cuuint32_t)rank, const_cast<void *>(ptr), d, st, b, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed with " + std::to_string((int)r));
        return UPPASD_GPU_ECUDA;
    }
    return UPPASD_GPU_OK;
}

namespace {

template <int BN, int EPI, int ST>
int launch_bn(const CUtensorMap &ma, const CUtensorMap &mb, const GemmArgs &g, cudaStream_t st) {
    auto kern = tc_gemm_kernel<BN, EPI, ST>;
    const size_t smem = gemm_smem_bytes<BN, ST>();
    static bool attr_set = false;  // per instantiation
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) {
            set_error(std::string("tc_gemm smem attribute: ") + cudaGetErrorString(e));
            return UPPASD_GPU_ECUDA;
        }
        attr_set = true;
    }
    kern<<<dim3(g.M / kBM, g.N / BN), kThreads, smem, st>>>(ma, mb, g);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("tc_gemm launch: ") + cudaGetErrorString(e));
        return UPPASD_GPU_ECUDA;
    }
    return UPPASD_GPU_OK;
}

template <int BN, int ST>
int launch_epi(int epi, const CUtensorMap &ma, const CUtensorMap &mb, const GemmArgs &g, cudaStream_t st) {
    switch (epi) {
    case kEpiStoreF32: return launch_bn<BN, kEpiStoreF32, ST>(ma, mb, g, st);
    case kEpiBiasF32: return launch_bn<BN, kEpiBiasF32, ST>(ma, mb, g, st);
    case kEpiBiasTanhBF16: return launch_bn<BN, kEpiBiasTanhBF16, ST>(ma, mb, g, st);
    case kEpiDTanhBF16: return launch_bn<BN, kEpiDTanhBF16, ST>(ma, mb, g, st);
    }
    set_error("tc_gemm: unknown epilogue");
    return UPPASD_GPU_EINVAL;
}
}  // namespace

int gemm_prepare(Gemm &op, const __nv_bfloat16 *A, const __nv_bfloat16 *B, int M, int N, int K, int epi, int bn,
                 int stages) {
    if (stages != 2 && stages != 4) {
        set_error("tc_gemm: stages must be 2 or 4");
        return UPPASD_GPU_EINVAL;
    }
    if (M <= 0 || N <= 0 || K <= 0 || M % kBM || K % kBK || !(bn == 64 || bn == 128 || bn == 256) || N % bn) {
        set_error("tc_gemm: need M % 128 == 0, K % 64 == 0, N % BN == 0 with BN in {64, 128, 256}");
        return UPPASD_GPU_EINVAL;
    }
    if (epi < 0 || epi > kEpiDTanhBF16) {
        set_error("tc_gemm: unknown epilogue");
        return UPPASD_GPU_EINVAL;
    }
    int rc = make_map(&op.ma, A, M, K, kBM);
    if (!rc) rc = make_map(&op.mb, B, N, K, bn);
    if (rc) return rc;
    op.M = M;
    op.N = N;
    op.K = K;
    op.epi = epi;
    op.bn = bn;
    op.stages = stages;
    return UPPASD_GPU_OK;
}

int gemm_run(const Gemm &op, const float *bias, const __nv_bfloat16 *Y, float *Cf, __nv_bfloat16 *Cb, int *err,
             cudaStream_t st) {
    const bool f32 = op.epi == kEpiStoreF32 || op.epi == kEpiBiasF32;
    if ((f32 && !Cf) || (!f32 && !Cb) || ((op.epi == kEpiBiasF32 || op.epi == kEpiBiasTanhBF16) && !bias) ||
        (op.epi == kEpiDTanhBF16 && !Y) || !err) {
        set_error("tc_gemm: missing operand for the epilogue");
        return UPPASD_GPU_EINVAL;
    }
    if ((Cf && (reinterpret_cast<uintptr_t>(Cf) & 15)) || (Cb && (reinterpret_cast<uintptr_t>(Cb) & 15)) ||
        (Y && (reinterpret_cast<uintptr_t>(Y) & 15))) {
        set_error("tc_gemm: outputs must be 16-byte aligned");
        return UPPASD_GPU_EINVAL;
    }
    GemmArgs g{op.M, op.N, op.K, bias, Y, Cf, Cb, err};
    // a short K loop (<= 2 slices per stage ring) fits 2 stages and more resident CTAs
    if (op.stages == 2) {
        switch (op.bn) {
        case 64: return launch_epi<64, 2>(op.epi, op.ma, op.mb, g, st);
        case 128: return launch_epi<128, 2>(op.epi, op.ma, op.mb, g, st);
        default: return launch_epi<256, 2>(op.epi, op.ma, op.mb, g, st);
        }
    }
    switch (op.bn) {
    case 64: return launch_epi<64, 4>(op.epi, op.ma, op.mb, g, st);
    case 128: return launch_epi<128, 4>(op.epi, op.ma, op.mb, g, st);
    default: return launch_epi<256, 4>(op.epi, op.ma, op.mb, g, st);
    }
}

}  // namespace tc
}  // namespace uppasd

extern "C" int uppasd_gpu_tc_gemm(int32_t M, int32_t N, int32_t K, const uint16_t *A, const uint16_t *B,
                                  const float *bias, const uint16_t *Y, int32_t epilogue, int32_t bn, float *Cf,
                                  uint16_t *Cb) {
    using namespace uppasd;
    if (!A || !B || M <= 0 || N <= 0 || K <= 0) {
        set_error("tc_gemm: bad arguments");
        return UPPASD_GPU_EINVAL;
    }
    if (M % tc::kBM || K % tc::kBK || !(bn == 64 || bn == 128 || bn == 256) || N % bn) {
        set_error("tc_gemm: need M % 128 == 0, K % 64 == 0, N % BN == 0 with BN in {64, 128, 256}");
        return UPPASD_GPU_EINVAL;
    }
    const bool f32 = epilogue == tc::kEpiStoreF32 || epilogue == tc::kEpiBiasF32;
    if (epilogue < 0 || epilogue > tc::kEpiDTanhBF16 || (f32 && !Cf) || (!f32 && !Cb) ||
        ((epilogue == tc::kEpiBiasF32 || epilogue == tc::kEpiBiasTanhBF16) && !bias) ||
        (epilogue == tc::kEpiDTanhBF16 && !Y)) {
        set_error("tc_gemm: epilogue operands missing");
        return UPPASD_GPU_EINVAL;
    }
    int dev = 0, major = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess || major < 10) {
        set_error("tc_gemm: needs an sm_10x device");
        return UPPASD_GPU_ENODEV;
    }
    __nv_bfloat16 *dA = nullptr, *dB = nullptr, *dY = nullptr, *dCb = nullptr;
    float *dbias = nullptr, *dCf = nullptr;
    int *derr = nullptr;
    const size_t nA = (size_t)M * K, nB = (size_t)N * K, nC = (size_t)M * N;
    cudaError_t e = cudaMalloc(&dA, nA * 2);
    if (e == cudaSuccess) e = cudaMalloc(&dB, nB * 2);
    if (e == cudaSuccess) e = cudaMalloc(&derr, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(derr, 0, sizeof(int));
    if (e == cudaSuccess && bias) e = cudaMalloc(&dbias, (size_t)N * 4);
    if (e == cudaSuccess && Y) e = cudaMalloc(&dY, nC * 2);
    if (e == cudaSuccess && f32) e = cudaMalloc(&dCf, nC * 4);
    if (e == cudaSuccess && !f32) e = cudaMalloc(&dCb, nC * 2);
    if (e == cudaSuccess) e = cudaMemcpy(dA, A, nA * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dB, B, nB * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && bias) e = cudaMemcpy(dbias, bias, (size_t)N * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && Y) e = cudaMemcpy(dY, Y, nC * 2, cudaMemcpyHostToDevice);
    int rc = UPPASD_GPU_OK;
    if (e != cudaSuccess) {
        set_error(std::string("tc_gemm: ") + cudaGetErrorString(e));
        rc = UPPASD_GPU_ECUDA;
    }
    tc::Gemm op;
    if (!rc) rc = tc::gemm_prepare(op, dA, dB, M, N, K, epilogue, bn, K > 128 ? 4 : 2);
    if (!rc) rc = tc::gemm_run(op, dbias, dY, dCf, dCb, derr, 0);
    int herr = 0;
    if (!rc) {
        e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && f32) e = cudaMemcpy(Cf, dCf, nC * 4, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && !f32) e = cudaMemcpy(Cb, dCb, nC * 2, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            set_error(std::string("tc_gemm: ") + cudaGetErrorString(e));
            rc = UPPASD_GPU_ECUDA;
        } else if (herr) {
            set_error("tc_gemm: a pipeline wait ran past its limit (code " + std::to_string(herr) + ")");
            rc = UPPASD_GPU_ESTATE;
        }
    }
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dY);
    cudaFree(dCb);
    cudaFree(dbias);
    cudaFree(dCf);
    cudaFree(derr);
    return rc;
}

namespace uppasd {
namespace tc {
namespace {

// One CTA waits on an mbarrier that nothing arrives at, through the GEMM pipeline's own
// bounded wait: it gives up after about kWaitLimitNs and records code 4.  No copy or MMA
// is issued, so nothing is left in flight when the CTA returns.
__global__ void wait_selftest_kernel(int *err) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (!mbar_wait(&bar, 0)) atomicExch(err, 4);
    }
}

}  // namespace
}  // namespace tc
}  // namespace uppasd

extern "C" int uppasd_gpu_tc_wait_selftest(void) {
    using namespace uppasd;
    int *derr = nullptr, herr = 0;
    cudaError_t e = cudaMalloc(&derr, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(derr, 0, sizeof(int));
    if (e == cudaSuccess) {
        tc::wait_selftest_kernel<<<1, 32>>>(derr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(derr);
    if (e != cudaSuccess) {
        set_error(std::string("tc_wait_selftest: ") + cudaGetErrorString(e));
        return UPPASD_GPU_ECUDA;
    }
    if (herr) {
        set_error("tc_wait_selftest: a pipeline wait ran past its limit (code " + std::to_string(herr) + ")");
        return UPPASD_GPU_ESTATE;
    }
    set_error("tc_wait_selftest: the wait completed although nothing arrived");
    return UPPASD_GPU_ECUDA;
}
