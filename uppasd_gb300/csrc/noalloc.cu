// noalloc.cu -- magnetisation sums without any device allocation.
//
// uppasd_gpu_moment_sums_noalloc() reduces a caller-owned device array of
// moments to per-ensemble sums and |M|/natom, writing a caller-owned device
// output.  Its only scratch is the file-scope array below, which every GPU that
// loads this library holds until the process exits.  It exists for callers that
// must not allocate device memory at all: a host code that keeps its own pool
// or arena (and forbids allocations behind it), code running while a CUDA graph
// is being captured on its stream elsewhere, or an embedding runtime that
// pre-reserves the device at start-up.  See the declaration in
// include/uppasd_gpu.h for the exact contract.
#include <cuda.h>

#include <cstdio>
#include <mutex>
#include <string>

#include "sim.h"

namespace uppasd {

namespace {

// Limits of the allocation-free reduction.
constexpr int kNaMaxEnsembles = 64;   // mensemble <= 64
constexpr int kNaBlocks = 128;        // partial-sum blocks per ensemble
constexpr int kNaThreads = 256;
constexpr int kNaMaxDevices = 64;

// Block partials: [ensemble][block][x, y, z].  64 * 128 * 3 doubles = 192 KiB.
// Every call overwrites the entries it reads back, so nothing needs clearing;
// two calls that overlap on the GPU (different streams) race on this array.
__device__ __align__(256) double g_partials[kNaMaxEnsembles * kNaBlocks * 3];

// The looked-up address per device, with the unique id of the context it belongs to:
// a device reset makes a new primary context (with a new id), and the address is then
// looked up again.
double *g_partials_addr[kNaMaxDevices] = {};
unsigned long long g_partials_ctx[kNaMaxDevices] = {};
std::mutex g_partials_mutex;

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry point (nothing links
// libcuda); both only read the calling thread's state.
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;

// Id of the current context; 0 when no context is current yet.
int current_context_id(unsigned long long *id) {
    *id = 0;
    if (!g_ctx_current || !g_ctx_id) {
        void *f1 = nullptr, *f2 = nullptr;
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
        cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
            q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return UPPASD_GPU_ECUDA;
        g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        g_ctx_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    CUcontext ctx = nullptr;
    if (g_ctx_current(&ctx) != CUDA_SUCCESS) return UPPASD_GPU_ECUDA;
    if (ctx && g_ctx_id(ctx, id) != CUDA_SUCCESS) return UPPASD_GPU_ECUDA;
    return UPPASD_GPU_OK;
}

__device__ __forceinline__ double warp_sum_na(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Pass 1: block b of ensemble k sums sites b, b + kNaBlocks*256, ... of the
// reference-layout array emomM(3, natom, mensemble).
__global__ void __launch_bounds__(kNaThreads) na_partials(const double *__restrict__ emomM, int natom,
                                                          double *__restrict__ partials) {
    const int k = blockIdx.y;
    const double *m = emomM + (size_t)3 * natom * k;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    // 64-bit site index: natom close to INT32_MAX must not overflow the stride
    for (int64_t i = (int64_t)blockIdx.x * kNaThreads + threadIdx.x; i < natom; i += (int64_t)kNaBlocks * kNaThreads) {
        s0 += m[3 * i];
        s1 += m[3 * i + 1];
        s2 += m[3 * i + 2];
    }
    __shared__ double part[kNaThreads / 32][3];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    s0 = warp_sum_na(s0);
    s1 = warp_sum_na(s1);
    s2 = warp_sum_na(s2);
    if (lane == 0) {
        part[wid][0] = s0;
        part[wid][1] = s1;
        part[wid][2] = s2;
    }
    __syncthreads();
    if (wid == 0) {
        double a0 = lane < kNaThreads / 32 ? part[lane][0] : 0.0;
        double a1 = lane < kNaThreads / 32 ? part[lane][1] : 0.0;
        double a2 = lane < kNaThreads / 32 ? part[lane][2] : 0.0;
        a0 = warp_sum_na(a0);
        a1 = warp_sum_na(a1);
        a2 = warp_sum_na(a2);
        if (lane == 0) {
            double *o = partials + 3 * ((size_t)k * kNaBlocks + blockIdx.x);
            o[0] = a0;
            o[1] = a1;
            o[2] = a2;
        }
    }
}

// Pass 2: one warp per ensemble folds the kNaBlocks partials in a fixed order.
__global__ void na_finish(const double *__restrict__ partials, int natom, int mensemble, double *__restrict__ out) {
    const int k = blockIdx.x;
    const int lane = threadIdx.x;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int b = lane; b < kNaBlocks; b += 32) {
        const double *p = partials + 3 * ((size_t)k * kNaBlocks + b);
        a0 += p[0];
        a1 += p[1];
        a2 += p[2];
    }
    a0 = warp_sum_na(a0);
    a1 = warp_sum_na(a1);
    a2 = warp_sum_na(a2);
    if (lane == 0) {
        out[4 * k] = a0;
        out[4 * k + 1] = a1;
        out[4 * k + 2] = a2;
        out[4 * k + 3] = sqrt(a0 * a0 + a1 * a1 + a2 * a2) / natom;
    }
    (void)mensemble;
}

// Device address of g_partials for the current device, resolved once per device
// context.
int partials_address(double **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_error(std::string("moment_sums_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return UPPASD_GPU_ENODEV;
    }
    if (dev < 0 || dev >= kNaMaxDevices) {
        set_error("moment_sums_noalloc: device index beyond the supported 64");
        return UPPASD_GPU_ENODEV;
    }
    std::lock_guard<std::mutex> lock(g_partials_mutex);
    unsigned long long ctx = 0;
    if (current_context_id(&ctx)) {
        set_error("moment_sums_noalloc: the driver's context query failed");
        return UPPASD_GPU_ECUDA;
    }
    // ctx == 0: no context is current yet, so nothing can have been looked up in it
    if (!g_partials_addr[dev] || ctx == 0 || g_partials_ctx[dev] != ctx) {
        double *ptr = nullptr;
        e = cudaGetSymbolAddress((void **)&ptr, g_partials);  // makes the primary context current
        if (e != cudaSuccess || !ptr) {
            set_error(std::string("moment_sums_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            return UPPASD_GPU_ECUDA;
        }
        if (current_context_id(&ctx) || ctx == 0) {
            set_error("moment_sums_noalloc: no current CUDA context after the address lookup");
            return UPPASD_GPU_ECUDA;
        }
        g_partials_addr[dev] = ptr;
        g_partials_ctx[dev] = ctx;
    }
    *out = g_partials_addr[dev];
    return UPPASD_GPU_OK;
}

}  // namespace
}  // namespace uppasd

extern "C" int uppasd_gpu_moment_sums_noalloc(const double *d_emomM, int32_t natom, int32_t mensemble, double *d_out,
                                              void *cuda_stream) {
    using namespace uppasd;
    if (!d_emomM || !d_out) {
        set_error("moment_sums_noalloc: null device pointer");
        return UPPASD_GPU_EINVAL;
    }
    if (natom <= 0 || mensemble <= 0) {
        set_error("moment_sums_noalloc: natom and mensemble must be positive");
        return UPPASD_GPU_EINVAL;
    }
    if (mensemble > kNaMaxEnsembles) {
        char buf[128];
        snprintf(buf, sizeof(buf), "moment_sums_noalloc: mensemble = %d exceeds the fixed maximum of %d", mensemble,
                 kNaMaxEnsembles);
        set_error(buf);
        return UPPASD_GPU_EINVAL;
    }
    double *partials = nullptr;
    int rc = partials_address(&partials);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    na_partials<<<dim3(kNaBlocks, mensemble), kNaThreads, 0, st>>>(d_emomM, natom, partials);
    na_finish<<<mensemble, 32, 0, st>>>(partials, natom, mensemble, d_out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("moment_sums_noalloc: launch: ") + cudaGetErrorString(e));
        return UPPASD_GPU_ECUDA;
    }
    return UPPASD_GPU_OK;
}
