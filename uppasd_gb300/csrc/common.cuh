// common.cuh -- device helpers shared by the sm_103a kernels.
//
// Physical constants follow Parameters/constants.f90:14-19 of the reference.
// The counter-based RNG is Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11),
// written here from the published round function and constants.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace uppasd {

constexpr double kGama = 1.760859644e11;   // s^-1 T^-1
constexpr double kKbolt = 1.38064852e-23;  // J/K
constexpr double kMub = 9.274009994e-24;   // J/T
constexpr double kMry = 2.179872325e-21;   // J
constexpr double kPi = 3.141592653589793238462643383279502884197;

// Philox streams: one per consumer so draws never collide.
enum : uint32_t { kStreamLLG = 0u, kStreamMC = 1u, kStreamMCGauss = 2u, kStreamLearned = 3u, kStreamPT = 8u };

struct Philox4 {
    uint32_t x, y, z, w;
};

__host__ __device__ inline Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                 uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return Philox4{c0, c1, c2, c3};
}

// Counter layout: (site, ensemble, step low word, step high 16 bits | stream << 16).
__host__ __device__ inline Philox4 philox_draw(uint64_t seed, int64_t site, int32_t ens, int64_t step,
                                               uint32_t stream) {
    return philox4x32_10((uint32_t)site, (uint32_t)ens, (uint32_t)step,
                         ((uint32_t)((uint64_t)step >> 32) & 0xFFFFu) | (stream << 16), (uint32_t)seed,
                         (uint32_t)(seed >> 32));
}

__host__ __device__ inline double u01_open(uint32_t x) { return ((double)x + 0.5) * 2.3283064365386963e-10; }
__host__ __device__ inline float u01_openf(uint32_t x) {
    return ((float)(x >> 8) + 0.5f) * 5.9604644775390625e-08f;  // 24-bit grid in (0,1)
}

// Three N(0,1) draws in FP64 (Box-Muller on the four Philox words).
__device__ inline void normal3_f64(uint64_t seed, int64_t site, int32_t ens, int64_t step, uint32_t stream,
                                   double z[3]) {
    Philox4 w = philox_draw(seed, site, ens, step, stream);
    const double twopi = 2.0 * kPi;
    double r0 = sqrt(-2.0 * log(u01_open(w.x)));
    double t0 = twopi * u01_open(w.y);
    double r1 = sqrt(-2.0 * log(u01_open(w.z)));
    double t1 = twopi * u01_open(w.w);
    z[0] = r0 * cos(t0);
    z[1] = r0 * sin(t0);
    z[2] = r1 * cos(t1);
}

// Three N(0,1) draws in FP32.
__device__ inline void normal3_f32(uint64_t seed, int64_t site, int32_t ens, int64_t step, uint32_t stream,
                                   float z[3]) {
    Philox4 w = philox_draw(seed, site, ens, step, stream);
    // radii from the full 32-bit words (relative precision of u, not absolute,
    // is what the tail of -2 ln u needs), angles from the 24-bit grid
    const float k32 = 2.3283064365386963e-10f;
    float r0 = sqrtf(-2.0f * logf(fmaf((float)w.x, k32, 0.5f * k32)));
    float r1 = sqrtf(-2.0f * logf(fmaf((float)w.z, k32, 0.5f * k32)));
    float s0, c0, s1, c1;
    sincospif(2.0f * u01_openf(w.y), &s0, &c0);
    sincospif(2.0f * u01_openf(w.w), &s1, &c1);
    z[0] = r0 * c0;
    z[1] = r0 * s0;
    z[2] = r1 * c1;
}

// Three N(0,1) draws in FP32 with the MUFU approximations of log, sin and cos
// (absolute error ~4e-7 per draw): the thermal field of the mixed-precision path.
__device__ inline void normal3_f32_fast(uint64_t seed, int64_t site, int32_t ens, int64_t step, uint32_t stream,
                                        float z[3]) {
    Philox4 w = philox_draw(seed, site, ens, step, stream);
    const float k32 = 2.3283064365386963e-10f;
    const float twopi = 6.283185307179586f;
    // radii as x rsqrt(x) (the approximate reciprocal square root, two instructions);
    // x is 0 when u rounds to 1, hence the floor inside the rsqrt
    const float x0 = -2.0f * __logf(fmaf((float)w.x, k32, 0.5f * k32));
    const float x1 = -2.0f * __logf(fmaf((float)w.z, k32, 0.5f * k32));
    const float r0 = x0 * rsqrtf(fmaxf(x0, 1e-30f));
    const float r1 = x1 * rsqrtf(fmaxf(x1, 1e-30f));
    // angles shifted into [-pi, pi] (the approximations' accurate range):
    // cos(2 pi u) = -cos(2 pi (u - 1/2)), sin(2 pi u) = -sin(2 pi (u - 1/2))
    float s0, c0;
    __sincosf(twopi * (fmaf((float)w.y, k32, 0.5f * k32) - 0.5f), &s0, &c0);
    float c1 = __cosf(twopi * (fmaf((float)w.w, k32, 0.5f * k32) - 0.5f));
    z[0] = -r0 * c0;
    z[1] = -r0 * s0;
    z[2] = -r1 * c1;
}

// Double-single helpers (Dekker / Knuth error-free transformations), host-callable so
// that their error bounds are checked on the CPU too.
__host__ __device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
__host__ __device__ __forceinline__ void quick_two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    e = b - (s - a);
}
__host__ __device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
    p = a * b;
    e = fmaf(a, b, -p);
}
// FP32 estimate of 1/sqrt(x) for the Newton step below (the device's rsqrtf; on the host
// the correctly rounded quotient, which the step refines the same way)
__host__ __device__ __forceinline__ float rsqrt_estimate(float x) {
#ifdef __CUDA_ARCH__
    return rsqrtf(x);
#else
    return 1.0f / sqrtf(x);
#endif
}

// A unit vector held as double-single pairs (hi + lo per component, ~48 bits) plus a
// change d: the sum, then |e|^2 - 1 from exact products, and the renormalisation by
// 1/sqrt(1 + x) to second order (|x| below ~1e-7 for the norm-preserving updates, so the
// truncation is below 1e-21), the correction added back with error-free sums.
__host__ __device__ __forceinline__ void ds_add_renorm(float hi[3], float lo[3], const float d[3]) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float sm, er;
        two_sum(hi[c], d[c], sm, er);
        quick_two_sum(sm, er + lo[c], hi[c], lo[c]);
    }
    float n2h = 0.f, n2l = 0.f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float pp, pe, sm, er;
        two_prod(hi[c], hi[c], pp, pe);
        two_sum(n2h, pp, sm, er);
        n2h = sm;
        n2l += er + pe + 2.0f * hi[c] * lo[c];
    }
    float xs, xe;
    two_sum(n2h, -1.0f, xs, xe);
    const float xx = xs + (xe + n2l);
    const float sm1 = xx * fmaf(0.375f, xx, -0.5f);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float corr = hi[c] * sm1 + lo[c] * sm1;
        float sm, er;
        two_sum(hi[c], corr, sm, er);
        quick_two_sum(sm, er + lo[c], hi[c], lo[c]);
    }
}

// The same for updates that leave the sphere at first order (Heun, LLGI: |x| reaches a
// few 1e-2 at finite temperature): 1/sqrt(1 + x) - 1 as a double-single pair from one
// Newton step on the FP32 estimate y0, y = y0 + y0 r / 2 with r = 1 - (1 + x) y0^2 formed
// from exact products (1 - p and the difference of the two near-equal O(x) terms are exact
// by Sterbenz's lemma for |x| < 1/2), so s_hi = y0 - 1 (exact) and s_lo = y0 r / 2; the
// correction e (s_hi + s_lo) is added with an exact product for its leading term.
__host__ __device__ __forceinline__ void ds_add_renorm_wide(float hi[3], float lo[3], const float d[3]) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float sm, er;
        two_sum(hi[c], d[c], sm, er);
        quick_two_sum(sm, er + lo[c], hi[c], lo[c]);
    }
    float n2h = 0.f, n2l = 0.f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float pp, pe, sm, er;
        two_prod(hi[c], hi[c], pp, pe);
        two_sum(n2h, pp, sm, er);
        n2h = sm;
        n2l += er + pe + 2.0f * hi[c] * lo[c];
    }
    float xs, xe;
    two_sum(n2h, -1.0f, xs, xe);
    const float xl = xe + n2l;  // x = xs + xl
    const float y0 = rsqrt_estimate(1.0f + xs);
    float p, pe, q, qe;
    two_prod(y0, y0, p, pe);  // y0^2 = p + pe
    two_prod(xs, p, q, qe);   // xs p = q + qe
    const float r = ((1.0f - p) - q) - (pe + qe + xs * pe + xl * p);
    const float s_hi = y0 - 1.0f;
    const float s_lo = 0.5f * y0 * r;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float p, pe, sm, er;
        two_prod(hi[c], s_hi, p, pe);
        const float rest = pe + hi[c] * s_lo + lo[c] * (s_hi + s_lo);
        two_sum(hi[c], p, sm, er);
        quick_two_sum(sm, er + (lo[c] + rest), hi[c], lo[c]);
    }
}

}  // namespace uppasd
