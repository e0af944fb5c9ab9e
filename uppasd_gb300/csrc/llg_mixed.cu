// llg_mixed.cu -- precision 3: LLG on any Hamiltonian the FP64 path takes (scalar or
// tensor exchange, DMI, uniaxial/cubic anisotropy, Zeeman; full or reduced), with the
// field gathered in FP32 and the FP64 state e / eM kept as the master.
//
// The FP64 path spends its time in FP64 arithmetic, which GB300 runs at about 1/70
// of the FP32 rate.  Here each step reads an FP32 mirror of the spins (float4: unit
// vector, moment in w), computes the field, the thermal field and the solver's
// rotation in FP32, and adds the resulting change to the FP64 master, which is
// renormalised in FP64 every step; the mirror is refreshed from the master.  The
// couplings are read from the same FP64 arrays as the FP64 path (rounded on use), so
// set_jtensor and reduced Hamiltonians need nothing extra.
//   Depondt   Evolution/depondt.f90:50-333 (thermal field drawn once per step)
//   midpoint  Evolution/midpoint.f90:34-323, noise rannum (RNG/randomnumbers.f90:625-771)
// The noise is the FP64 path's Philox stream (site, ensemble, step), drawn with the
// FP32 Box-Muller of the structured path.
#include <algorithm>
#include <cstdlib>
#include <string>
#include <type_traits>
#include <cstring>
#include <map>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "field_f32.cuh"
#include "field_fp64.cuh"
#include "sim.h"

namespace uppasd {

namespace {

struct MixArgs {
    HamDev h;
    const double *lambda, *temp, *landeg, *mmom;
    // per-step constants, computed once on the host (per-site FP64 divisions and square
    // roots would cost more than the whole FP32 step on GB300's FP64 pipe)
    float dt_dep;   // delta_t gama: Depondt rotation angle per |B| is dt_dep / (1 + lambda^2)
    float dt_mid;   // delta_t bn gama: midpoint dt = dt_mid / (1 + lambda^2)
    float c_dp;     // 2 kB / (delta_t gama muB): Depondt D = c_dp lambda
    float c_dk;     // kB / (muB bn): midpoint D = c_dk lambda / (1 + lambda^2)
    float c_heun;   // delta_t gama kB / muB: Heun sigma^2 / 2 = c_heun lambda / (1 + lambda^2) T / m
    float tau_dt;   // LLGI relaxtime / delta_t
    float dtg_llgi; // LLGI -delta_t gama
    float temprescale;
    int noise_on;
    int perp;       // field projected perpendicular to emom before each half-step
    NoiseArgs nz;          // Philox (FP32 Box-Muller here), injected normals, or none
    const int64_t *d_step;
    int64_t step_off;
    Vec3D e, eM;           // FP64 master
    Vec3D mpast;           // LLGI m(t - dt), FP64
    MixedDev c;            // mirrors, predictor, b2, FP32 couplings
};

// Rodrigues rotation increment R e - e about h = bd/|bd| by v = |bd| dtg.
__device__ __forceinline__ void rotation_delta_f32(const float bd[3], const float e[3], float dtg, float d[3]) {
    const float bn = sqrtf(bd[0] * bd[0] + bd[1] * bd[1] + bd[2] * bd[2]) + 1e-15f;
    const float inv = 1.0f / bn;
    const float hx = bd[0] * inv, hy = bd[1] * inv, hz = bd[2] * inv;
    const float v = bn * dtg;
    float sv, cv;
    sincosf(v, &sv, &cv);
    const float sh = sinf(0.5f * v);
    const float u = 2.0f * sh * sh;  // 1 - cos v without cancellation
    const float he = hx * e[0] + hy * e[1] + hz * e[2];
    d[0] = u * (he * hx - e[0]) + sv * (hy * e[2] - hz * e[1]);
    d[1] = u * (he * hy - e[1]) + sv * (hz * e[0] - hx * e[2]);
    d[2] = u * (he * hz - e[2]) + sv * (hx * e[1] - hy * e[0]);
}

// midpoint: A = dtg/2 a1 + sqrt(dt) g/2 s1 and the Cayley transform of e by A
__device__ __forceinline__ void midpoint_A_f32(float lam, float dtg, float sqrtdtg, const float e[3], const float b[3],
                                               const float r[3], float A[3]) {
    const float a1[3] = {-b[0] - lam * (e[1] * b[2] - e[2] * b[1]), -b[1] - lam * (e[2] * b[0] - e[0] * b[2]),
                         -b[2] - lam * (e[0] * b[1] - e[1] * b[0])};
    const float s1[3] = {-r[0] - lam * (e[1] * r[2] - e[2] * r[1]), -r[1] - lam * (e[2] * r[0] - e[0] * r[2]),
                         -r[2] - lam * (e[0] * r[1] - e[1] * r[0])};
#pragma unroll
    for (int c = 0; c < 3; ++c) A[c] = 0.5f * dtg * a1[c] + 0.5f * sqrtdtg * s1[c];
}

__device__ __forceinline__ void cayley_f32(const float A[3], const float e[3], float out[3]) {
    const float detAi = 1.0f / (1.0f + (A[0] * A[0] + A[1] * A[1] + A[2] * A[2]));
    const float a0 = e[0] + e[1] * A[2] - e[2] * A[1];
    const float a1 = e[1] + e[2] * A[0] - e[0] * A[2];
    const float a2 = e[2] + e[0] * A[1] - e[1] * A[0];
    out[0] = (a0 * (1.0f + A[0] * A[0]) + a1 * (A[0] * A[1] + A[2]) + a2 * (A[0] * A[2] - A[1])) * detAi;
    out[1] = (a0 * (A[1] * A[0] - A[2]) + a1 * (1.0f + A[1] * A[1]) + a2 * (A[1] * A[2] + A[0])) * detAi;
    out[2] = (a0 * (A[2] * A[0] + A[1]) + a1 * (A[2] * A[1] - A[0]) + a2 * (1.0f + A[2] * A[2])) * detAi;
}

// SIB (sphmidpoint.f90:36-477) in FP32: a1 = -b - lam e x b, s1 likewise with the
// noise, then the fixed point of e' = e + dtg f x a1 + sqrt(dt) g f x s1 with
// f = (e + e')/2.  The FP64 path stops at 1e-12 per component; FP32 converges to
// its rounding, so the tolerance here is 2e-7.
__device__ __forceinline__ void sib_f32(float lam, const float e[3], const float b[3], const float r[3],
                                        const float e1[3], float dtg, float sqrtdtg, float out[3]) {
    const float a1[3] = {-b[0] - lam * (e[1] * b[2] - e[2] * b[1]), -b[1] - lam * (e[2] * b[0] - e[0] * b[2]),
                         -b[2] - lam * (e[0] * b[1] - e[1] * b[0])};
    const float s1[3] = {-r[0] - lam * (e[1] * r[2] - e[2] * r[1]), -r[1] - lam * (e[2] * r[0] - e[0] * r[2]),
                         -r[2] - lam * (e[0] * r[1] - e[1] * r[0])};
    float f0[3] = {e1[0], e1[1], e1[2]};
    for (int it = 0; it < 100; ++it) {
        float fd[3], fs[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float f1 = 0.5f * (e1[c] + f0[c]);
            fd[c] = dtg * f1;
            fs[c] = sqrtdtg * f1;
        }
        out[0] = e1[0] + fd[1] * a1[2] - fd[2] * a1[1] + fs[1] * s1[2] - fs[2] * s1[1];
        out[1] = e1[1] + fd[2] * a1[0] - fd[0] * a1[2] + fs[2] * s1[0] - fs[0] * s1[2];
        out[2] = e1[2] + fd[0] * a1[1] - fd[1] * a1[0] + fs[0] * s1[1] - fs[1] * s1[0];
        const bool done = fabsf(f0[0] - out[0]) < 2e-7f && fabsf(f0[1] - out[1]) < 2e-7f &&
                          fabsf(f0[2] - out[2]) < 2e-7f;
        f0[0] = out[0];
        f0[1] = out[1];
        f0[2] = out[2];
        if (done) break;
    }
}

// Spherical SIB (sispht / sisphf, sphmidpoint.f90:485-923) in FP32: the SIB iteration with
// the midpoint direction u = (e1 + f0) / |e1 + f0|.  out is the last iterate, f0 the one
// before it when the tolerance ended the loop (else the last one).
__device__ __forceinline__ void sisph_f32(float lam, const float e[3], const float b[3], const float r[3],
                                          const float e1[3], float dtg, float sqrtdtg, float out[3], float f0[3]) {
    const float a1[3] = {-b[0] - lam * (e[1] * b[2] - e[2] * b[1]), -b[1] - lam * (e[2] * b[0] - e[0] * b[2]),
                         -b[2] - lam * (e[0] * b[1] - e[1] * b[0])};
    const float s1[3] = {-r[0] - lam * (e[1] * r[2] - e[2] * r[1]), -r[1] - lam * (e[2] * r[0] - e[0] * r[2]),
                         -r[2] - lam * (e[0] * r[1] - e[1] * r[0])};
    f0[0] = e1[0];
    f0[1] = e1[1];
    f0[2] = e1[2];
    for (int it = 0; it < 100; ++it) {
        const float w[3] = {e1[0] + f0[0], e1[1] + f0[1], e1[2] + f0[2]};
        const float inv = 1.0f / sqrtf(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        float fd[3], fs[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            fd[c] = dtg * w[c] * inv;
            fs[c] = sqrtdtg * w[c] * inv;
        }
        out[0] = e1[0] + fd[1] * a1[2] - fd[2] * a1[1] + fs[1] * s1[2] - fs[2] * s1[1];
        out[1] = e1[1] + fd[2] * a1[0] - fd[0] * a1[2] + fs[2] * s1[0] - fs[0] * s1[2];
        out[2] = e1[2] + fd[0] * a1[1] - fd[1] * a1[0] + fs[0] * s1[1] - fs[1] * s1[0];
        if (fabsf(f0[0] - out[0]) < 2e-7f && fabsf(f0[1] - out[1]) < 2e-7f && fabsf(f0[2] - out[2]) < 2e-7f) break;
        f0[0] = out[0];
        f0[1] = out[1];
        f0[2] = out[2];
    }
}

// Heun drift a = lam h + e x h - e (e . lam h) and diffusion matrix b of one half
// (heun_proper.f90:28-161, 261-530); zzq reproduces the corrector's b1zz expression.
__device__ __forceinline__ void heun_ab(float lam, const float e[3], const float h[3], bool zzq, float a[3],
                                        float bm[9]) {
    const float hl[3] = {lam * h[0], lam * h[1], lam * h[2]};
    const float prot = e[0] * hl[0] + e[1] * hl[1] + e[2] * hl[2];
    a[0] = hl[0] + e[2] * h[1] - e[1] * h[2] - e[0] * prot;
    a[1] = hl[1] - e[2] * h[0] + e[0] * h[2] - e[1] * prot;
    a[2] = hl[2] + e[1] * h[0] - e[0] * h[1] - e[2] * prot;
    bm[0] = lam - e[0] * e[0] * lam;
    bm[1] = e[2] - e[0] * e[1] * lam;
    bm[2] = -e[1] - e[0] * e[2] * lam;
    bm[3] = -e[2] - e[1] * e[0] * lam;
    bm[4] = lam - e[1] * e[1] * lam;
    bm[5] = e[0] - e[1] * e[2] * lam;
    bm[6] = e[1] - e[2] * e[0] * lam;
    bm[7] = -e[0] - e[2] * e[1] * lam;
    bm[8] = zzq ? lam - e[2] * e[2] - lam : lam - e[2] * e[2] * lam;
}

// llgiheun (llgi.f90:178-278) in FP32: m = A^-1 B, A = I + beta [e1]x
__device__ __forceinline__ void llgi_f32(float lam, float tau_dt, float dtg, const float et[3], const float e1[3],
                                         const float h[3], float out[3]) {
    const float beta = -lam * (1.0f + tau_dt), zeta = -lam * tau_dt;
    const float A12 = -beta * e1[2], A13 = beta * e1[1], A21 = beta * e1[2], A23 = -beta * e1[0];
    const float A31 = -beta * e1[1], A32 = beta * e1[0];
    const float det = 1.0f / (1.0f - A23 * A32 - A12 * A21 - A13 * A31);
    const float B1 = e1[0] + dtg * (e1[1] * h[2] - e1[2] * h[1]) + zeta * (e1[2] * et[1] - e1[1] * et[2]);
    const float B2 = e1[1] + dtg * (e1[2] * h[0] - e1[0] * h[2]) + zeta * (e1[0] * et[2] - e1[2] * et[0]);
    const float B3 = e1[2] + dtg * (e1[0] * h[1] - e1[1] * h[0]) + zeta * (e1[1] * et[0] - e1[0] * et[1]);
    out[0] = ((1.0f - A32 * A23) * B1 + (A13 * A32 - A12) * B2 + (A12 * A23 - A13) * B3) * det;
    out[1] = ((A23 * A31 - A21) * B1 + (1.0f - A31 * A13) * B2 + (A13 * A21 - A23) * B3) * det;
    out[2] = ((A21 * A32 - A31) * B1 + (A12 * A31 - A32) * B2 + (1.0f - A21 * A12) * B3) * det;
}

// 1 / sqrt(1 + x) in FP64: the second-order series when |x| < 1e-7 (the rotating
// solvers; truncation below 1e-21), else two Newton steps from the FP32 estimate
// (Heun and LLGI leave the sphere at first order, |x| up to ~1e-4).
__device__ __forceinline__ double renorm_scale(double x) {
    if (fabs(x) < 1e-7) return fma(x, fma(0.375, x, -0.5), 1.0);
    const double n2 = 1.0 + x;
    double y = (double)rsqrtf((float)n2);
    y = y * fma(-0.5 * n2, y * y, 1.5);
    y = y * fma(-0.5 * n2, y * y, 1.5);
    return y;
}

__device__ __forceinline__ void perp_f32(float B[3], const float e[3]) {
    const float d = B[0] * e[0] + B[1] * e[1] + B[2] * e[2];
    B[0] -= e[0] * d;
    B[1] -= e[1] * d;
    B[2] -= e[2] * d;
}

// Noise of site i at `step` (the corrector draws the same numbers again), scaled as
// each solver scales it: Depondt / LLGI thermal field, rannum (midpoint, SIB; off
// when min(lambda) <= 1e-12), Heun's dW (with the Lande factor applied by the caller).
template <int ALG>
__device__ __forceinline__ void noise_f32(const MixArgs &a, int i, int k, int64_t step, float lam, float mm,
                                          float out[3]) {
    float z[3];
    if ((ALG == 1 || ALG == 6 || ALG == 7) && !a.noise_on) {
        out[0] = out[1] = out[2] = 0.f;
        return;
    }
    if (a.nz.mode == 0) {
        normal3_f32_fast(a.nz.seed, i, k, step, kStreamLLG, z);
    } else {
        double zd[3];
        noise3(a.nz, i, k, a.h.natom, a.h.mensemble, step, zd);
        z[0] = (float)zd[0];
        z[1] = (float)zd[1];
        z[2] = (float)zd[2];
    }
    const float T = (a.c.uni_T ? a.c.T_u : (float)a.temp[i]) * a.temprescale;
    float sigma;
    if (ALG == 5 || ALG == 11) sigma = sqrtf(a.c_dp * lam * T / mm);
    else if (ALG == 4) sigma = sqrtf(2.0f * (a.c_heun * lam / (1.0f + lam * lam)) * T / mm);
    else sigma = sqrtf(2.0f * (a.c_dk * lam / (1.0f + lam * lam)) * T / mm);
    out[0] = z[0] * sigma;
    out[1] = z[1] * sigma;
    out[2] = z[2] * sigma;
}

template <int ALG>
__global__ void __launch_bounds__(256) mixed_predict(MixArgs a) {
    const int N = a.h.natom, M = a.h.mensemble;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)N * M) return;
    const int k = (int)(t / N), i = (int)(t - (int64_t)k * N);
    const size_t o = (size_t)k * N + i;
    const int64_t step = *a.d_step + a.step_off;
    float B[3];
    field_f32(a.h, a.c, a.c.mt, i, k, B);
    const float4 me = a.c.mt[o];
    const float e[3] = {me.x, me.y, me.z};
    if (a.perp) perp_f32(B, e);
    const float lam = (a.c.uni_lam ? a.c.lam_u : (float)a.lambda[i]), mm = me.w;
    float r[3];
    noise_f32<ALG>(a, i, k, step, lam, mm, r);
    float p[3];
    if (ALG == 5) {
        const float bl[3] = {B[0] + r[0], B[1] + r[1], B[2] + r[2]};
        const float bd[3] = {bl[0] + lam * (e[1] * bl[2] - e[2] * bl[1]), bl[1] + lam * (e[2] * bl[0] - e[0] * bl[2]),
                             bl[2] + lam * (e[0] * bl[1] - e[1] * bl[0])};
        float d[3];
        rotation_delta_f32(bd, e, a.dt_dep / (1.0f + lam * lam), d);
        p[0] = e[0] + d[0];
        p[1] = e[1] + d[1];
        p[2] = e[2] + d[2];
        a.c.b2x[o] = bd[0];
        a.c.b2y[o] = bd[1];
        a.c.b2z[o] = bd[2];
    } else if (ALG == 11) {
        const float bd[3] = {B[0] + r[0], B[1] + r[1], B[2] + r[2]};
        const float et[3] = {(float)a.mpast.x[o], (float)a.mpast.y[o], (float)a.mpast.z[o]};
        llgi_f32(lam, a.tau_dt, a.dtg_llgi, et, e, bd, p);
        a.c.b2x[o] = bd[0];
        a.c.b2y[o] = bd[1];
        a.c.b2z[o] = bd[2];
    } else if (ALG == 4) {
        const float g = (a.c.uni_g ? a.c.g_u : (float)a.landeg[i]);
        const float dtg = a.dt_dep * g / (1.0f + lam * lam);
        const float dw[3] = {r[0] * g, r[1] * g, r[2] * g};
        float ah[3], bm[9];
        heun_ab(lam, e, B, false, ah, bm);
#pragma unroll
        for (int c = 0; c < 3; ++c)
            p[c] = e[c] + ah[c] * dtg + bm[3 * c] * dw[0] + bm[3 * c + 1] * dw[1] + bm[3 * c + 2] * dw[2];
        a.c.b2x[o] = B[0];
        a.c.b2y[o] = B[1];
        a.c.b2z[o] = B[2];
    } else {
        const float dt = a.dt_mid / (1.0f + lam * lam);
        const float g = (a.c.uni_g ? a.c.g_u : (float)a.landeg[i]);
        const float dtg = dt * g, sqrtdtg = sqrtf(dt) * g;
        float et[3];
        if (ALG == 7) {
            float f0[3];
            sisph_f32(lam, e, B, r, e, dtg, sqrtdtg, et, f0);
            const float w[3] = {e[0] + f0[0], e[1] + f0[1], e[2] + f0[2]};
            const float inv = 1.0f / sqrtf(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
            p[0] = w[0] * inv;
            p[1] = w[1] * inv;
            p[2] = w[2] * inv;
        } else {
            if (ALG == 1) {
                float A[3];
                midpoint_A_f32(lam, dtg, sqrtdtg, e, B, r, A);
                cayley_f32(A, e, et);
            } else {
                sib_f32(lam, e, B, r, e, dtg, sqrtdtg, et);
            }
            p[0] = 0.5f * (e[0] + et[0]);
            p[1] = 0.5f * (e[1] + et[1]);
            p[2] = 0.5f * (e[2] + et[2]);
        }
    }
    a.c.mp[o] = make_float4(p[0], p[1], p[2], mm);
}

template <int ALG, bool DS>
__global__ void __launch_bounds__(256) mixed_correct(MixArgs a) {
    const int N = a.h.natom, M = a.h.mensemble;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)N * M) return;
    const int k = (int)(t / N), i = (int)(t - (int64_t)k * N);
    const size_t o = (size_t)k * N + i;
    const int64_t step = *a.d_step + a.step_off;
    float B[3];
    field_f32(a.h, a.c, a.c.mp, i, k, B);
    const float4 me = a.c.mt[o], mpv = a.c.mp[o];
    const float e[3] = {me.x, me.y, me.z}, pr[3] = {mpv.x, mpv.y, mpv.z};
    // emom at the second half-step: m(t) for midpoint and SIB, the predictor otherwise
    if (a.perp) perp_f32(B, (ALG == 1 || ALG == 6 || ALG == 7) ? e : pr);
    const float lam = (a.c.uni_lam ? a.c.lam_u : (float)a.lambda[i]), mm = me.w;
    float r[3];
    noise_f32<ALG>(a, i, k, step, lam, mm, r);
    float out[3];
    bool unit = false;  // out is the new spin (else e + out)
    if (ALG == 5) {
        const float bl[3] = {B[0] + r[0], B[1] + r[1], B[2] + r[2]};
        float bd[3] = {bl[0] + lam * (pr[1] * bl[2] - pr[2] * bl[1]), bl[1] + lam * (pr[2] * bl[0] - pr[0] * bl[2]),
                       bl[2] + lam * (pr[0] * bl[1] - pr[1] * bl[0])};
        bd[0] = 0.5f * bd[0] + 0.5f * a.c.b2x[o];
        bd[1] = 0.5f * bd[1] + 0.5f * a.c.b2y[o];
        bd[2] = 0.5f * bd[2] + 0.5f * a.c.b2z[o];
        rotation_delta_f32(bd, e, a.dt_dep / (1.0f + lam * lam), out);
    } else if (ALG == 11) {
        const float bd[3] = {0.5f * (B[0] + r[0]) + 0.5f * a.c.b2x[o], 0.5f * (B[1] + r[1]) + 0.5f * a.c.b2y[o],
                             0.5f * (B[2] + r[2]) + 0.5f * a.c.b2z[o]};
        const float et[3] = {(float)a.mpast.x[o], (float)a.mpast.y[o], (float)a.mpast.z[o]};
        // m(t) becomes the previous step (FP64, from the master)
        if constexpr (DS) {
            a.mpast.x[o] = (double)e[0] + (double)a.c.lox[o];
            a.mpast.y[o] = (double)e[1] + (double)a.c.loy[o];
            a.mpast.z[o] = (double)e[2] + (double)a.c.loz[o];
        } else {
            a.mpast.x[o] = a.e.x[o];
            a.mpast.y[o] = a.e.y[o];
            a.mpast.z[o] = a.e.z[o];
        }
        llgi_f32(lam, a.tau_dt, a.dtg_llgi, et, e, bd, out);
        unit = true;
    } else if (ALG == 4) {
        const float g = (a.c.uni_g ? a.c.g_u : (float)a.landeg[i]);
        const float dtg = a.dt_dep * g / (1.0f + lam * lam);
        const float dw[3] = {r[0] * g, r[1] * g, r[2] * g};
        const float h2[3] = {a.c.b2x[o], a.c.b2y[o], a.c.b2z[o]};
        float a1[3], b1[9], a2[3], b2[9];
        heun_ab(lam, pr, B, true, a1, b1);
        heun_ab(lam, e, h2, false, a2, b2);
#pragma unroll
        for (int c = 0; c < 3; ++c)
            out[c] = e[c] + 0.5f * ((a1[c] + a2[c]) * dtg + (b1[3 * c] + b2[3 * c]) * dw[0] +
                                    (b1[3 * c + 1] + b2[3 * c + 1]) * dw[1] + (b1[3 * c + 2] + b2[3 * c + 2]) * dw[2]);
        unit = true;
    } else {
        const float dt = a.dt_mid / (1.0f + lam * lam);
        const float g = (a.c.uni_g ? a.c.g_u : (float)a.landeg[i]);
        const float dtg = dt * g, sqrtdtg = sqrtf(dt) * g;
        if (ALG == 1) {
            float A[3];
            midpoint_A_f32(lam, dtg, sqrtdtg, pr, B, r, A);
            cayley_f32(A, e, out);
        } else if (ALG == 6) {
            sib_f32(lam, pr, B, r, e, dtg, sqrtdtg, out);
        } else {
            float f0[3];
            sisph_f32(lam, pr, B, r, e, dtg, sqrtdtg, out, f0);
        }
        unit = true;
    }
    float d[3];
    if (unit) {
        d[0] = out[0] - e[0];
        d[1] = out[1] - e[1];
        d[2] = out[2] - e[2];
    } else {
        d[0] = out[0];
        d[1] = out[1];
        d[2] = out[2];
    }
    if constexpr (DS) {
        // double-single master (precision 4): hi is the mirror, the change and the
        // renormalisation in error-free FP32 arithmetic; e / eM are made on demand
        float hi[3] = {e[0], e[1], e[2]}, lo[3] = {a.c.lox[o], a.c.loy[o], a.c.loz[o]};
        if constexpr (ALG == 4 || ALG == 11) ds_add_renorm_wide(hi, lo, d);  // off the sphere at first order
        else ds_add_renorm(hi, lo, d);
        a.c.lox[o] = lo[0];
        a.c.loy[o] = lo[1];
        a.c.loz[o] = lo[2];
        a.c.mt[o] = make_float4(hi[0], hi[1], hi[2], mm);
        return;
    }
    // FP64 master: add the change, renormalise, refresh the mirror
    double e0 = a.e.x[o] + (double)d[0], e1 = a.e.y[o] + (double)d[1], e2 = a.e.z[o] + (double)d[2];
    const double sc = renorm_scale(fma(e2, e2, fma(e1, e1, e0 * e0)) - 1.0);
    e0 *= sc;
    e1 *= sc;
    e2 *= sc;
    const double mmd = a.c.uni_m ? a.c.mmom_u : a.mmom[o];
    a.e.x[o] = e0;
    a.e.y[o] = e1;
    a.e.z[o] = e2;
    a.eM.x[o] = mmd * e0;
    a.eM.y[o] = mmd * e1;
    a.eM.z[o] = mmd * e2;
    a.c.mt[o] = make_float4((float)e0, (float)e1, (float)e2, mm);
}

// Heat bath of one colour (flip_h, MonteCarlo/montecarlo_common.f90:371-422) on the
// FP32 mirror: the field over the caller's neighbour lists, the draw in FP32 with the
// FP64 path's Philox counters (site, ensemble, sweep), written to the mirror only.  Every
// site is drawn again each sweep and its FP64 value is the draw renormalised in FP64, so
// e / eM are made from the mirror once after the sweeps (mixed_master_from_mirror) rather
// than written on every update: each colour writes every other site, and the FP64 state's
// 48 bytes per site went to DRAM as read-modify-writes of half-written sectors.  Same
// checkerboard chain as mc_colour_kernel.
__global__ void __launch_bounds__(256) mixed_heat_bath(HamDev h, MixedDev c, const int32_t *sites, int nsites,
                                                       float beta_mub, const float *betak, uint64_t seed,
                                                       int64_t sweep) {
    const int N = h.natom;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nsites * h.mensemble) return;
    const int k = (int)(t / nsites);
    const int i = sites[t - (int64_t)k * nsites];
    const size_t o = (size_t)k * N + i;
    float4 *mt = c.mt;
    float B[3];
    field_f32(h, c, mt, i, k, B);
    const float mm = mt[o].w;
    const Philox4 w = philox_draw(seed, i, k, sweep, kStreamMC);
    const float k32 = 2.3283064365386963e-10f;
    const float q = fmaf((float)w.x, k32, 0.5f * k32), fp = fmaf((float)w.y, k32, 0.5f * k32);
    const float3 n = heat_bath_f32(make_float3(B[0], B[1], B[2]), (betak ? betak[k] : beta_mub) * mm, q, fp);
    mt[o] = make_float4(n.x, n.y, n.z, mm);
}

// The FP64 state from the mirror after Monte Carlo sweeps: the draw renormalised in FP64,
// as the LLG steps leave a spin, and the full moment; with `moved` (Metropolis) only at
// the sites whose trial was accepted, whose marks it clears.
__global__ void mixed_master_from_mirror(MixedDev c, Vec3D e, Vec3D eM, const double *mmom, int64_t n,
                                         uint8_t *moved) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    if (moved) {
        if (!moved[o]) return;
        moved[o] = 0;
    }
    const float4 v = c.mt[o];
    double x = v.x, y = v.y, z = v.z;
    const double sc = renorm_scale(fma(z, z, fma(y, y, x * x)) - 1.0);
    x *= sc;
    y *= sc;
    z *= sc;
    const double md = c.uni_m ? c.mmom_u : mmom[o];
    e.x[o] = x;
    e.y[o] = y;
    e.z[o] = z;
    eM.x[o] = md * x;
    eM.y[o] = md * y;
    eM.z[o] = md * z;
}

// Metropolis on the mirror (mc_evolve with flip_a, MonteCarlo/montecarlo.f90:44-273,
// montecarlo_common.f90:139-200): the trial of choose_random_flip (:25-79) from the same
// Philox words as the FP64 path, the energy change in FP32, acceptance when it is <= 0 or
// u < exp(-beta de); an accepted trial is written to the mirror and its site marked moved;
// after the sweeps mixed_master_from_mirror gives the moved sites the trial renormalised in
// FP64 (rejected sites keep their FP64 state as it was).
__global__ void __launch_bounds__(256) mixed_metropolis(HamDev h, MixedDev c, const int32_t *sites, int nsites,
                                                        float beta_mub, float delta, uint64_t seed, int64_t sweep) {
    const int N = h.natom;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nsites * h.mensemble) return;
    const int k = (int)(t / nsites);
    const int i = sites[t - (int64_t)k * nsites];
    const size_t o = (size_t)k * N + i;
    float4 *mt = c.mt;
    const float4 cur = mt[o];
    const Philox4 w = philox_draw(seed, i, k, sweep, kStreamMC);
    const float k32 = 2.3283064365386963e-10f;
    const float u0 = fmaf((float)w.x, k32, 0.5f * k32), u1 = fmaf((float)w.y, k32, 0.5f * k32);
    const float u2 = fmaf((float)w.z, k32, 0.5f * k32), u3 = fmaf((float)w.w, k32, 0.5f * k32);
    float nm[3];
    const int ftype = (int)floorf(3.0f * u0);
    if (ftype == 0) {  // uniform on the sphere
        const float ct = 1.0f - 2.0f * u2, st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
        float sp, cp;
        __sincosf(u1 * 2.0f * 3.14159265358979f, &sp, &cp);
        nm[0] = st * cp;
        nm[1] = st * sp;
        nm[2] = ct;
    } else if (ftype == 1) {  // Gaussian displacement of width delta, renormalised
        float g[3];
        normal3_f32_fast(seed, i, k, sweep, kStreamMCGauss, g);
        const float a0 = cur.x + g[0] * delta, a1 = cur.y + g[1] * delta, a2 = cur.z + g[2] * delta;
        const float il = rsqrtf(a0 * a0 + a1 * a1 + a2 * a2);
        nm[0] = a0 * il;
        nm[1] = a1 * il;
        nm[2] = a2 * il;
    } else {  // flip
        nm[0] = -cur.x;
        nm[1] = -cur.y;
        nm[2] = -cur.z;
    }
    const float de = delta_energy_f32(h, c, mt, i, k, nm);
    if (!(de <= 0.0f || u3 < __expf(-beta_mub * de))) return;
    mt[o] = make_float4(nm[0], nm[1], nm[2], cur.w);
    c.moved[o] = 1;
}

__global__ void mixed_mirror(Vec3D e, const double *mmom, float4 *mt, int64_t n) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) mt[t] = make_float4((float)e.x[t], (float)e.y[t], (float)e.z[t], (float)mmom[t]);
}

// precision 4: the double-single master from e (hi the mirror, lo the FP32 residual) and
// e / eM from the master
__global__ void mixed_mirror_ds(MixedDev c, Vec3D e, const double *mmom, int64_t n) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double x = e.x[t], y = e.y[t], z = e.z[t];
    const float hx = (float)x, hy = (float)y, hz = (float)z;
    c.mt[t] = make_float4(hx, hy, hz, (float)mmom[t]);
    c.lox[t] = (float)(x - (double)hx);
    c.loy[t] = (float)(y - (double)hy);
    c.loz[t] = (float)(z - (double)hz);
}

__global__ void mixed_ds_to_master(MixedDev c, Vec3D e, Vec3D eM, const double *mmom, int64_t n) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float4 h = c.mt[t];
    const double x = (double)h.x + (double)c.lox[t], y = (double)h.y + (double)c.loy[t],
                 z = (double)h.z + (double)c.loz[t];
    const double md = c.uni_m ? c.mmom_u : mmom[t];
    e.x[t] = x;
    e.y[t] = y;
    e.z[t] = z;
    eM.x[t] = md * x;
    eM.y[t] = md * y;
    eM.z[t] = md * z;
}

}  // namespace

namespace {
template <typename T>
bool fetch(std::vector<T> &h, const T *d, size_t n) {
    h.resize(n);
    return n == 0 || cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost) == cudaSuccess;
}
template <typename T>
bool store(T **d, const std::vector<T> &h) {
    cudaFree(*d);
    *d = nullptr;
    if (h.empty()) return true;
    return cudaMalloc(d, h.size() * sizeof(T)) == cudaSuccess &&
           cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess;
}

// Numbers fixed-width integer keys in order of first appearance (the site classes).
struct KeyInterner {
    size_t width, cap;
    std::vector<int32_t> keys;  // the distinct keys back to back
    std::unordered_map<uint64_t, std::vector<int>> byhash;
    int n = 0;
    KeyInterner(size_t w, size_t c) : width(w), cap(c) {}
    // the id of key k (a new one when unseen), -1 when a new one would exceed cap
    int id(const std::vector<int32_t> &k) {
        uint64_t hsh = 1469598103934665603ull;  // FNV-1a over the key words
        for (int32_t w : k) {
            hsh ^= (uint32_t)w;
            hsh *= 1099511628211ull;
        }
        std::vector<int> &cand = byhash[hsh];
        for (int c : cand)
            if (std::equal(k.begin(), k.end(), keys.begin() + (size_t)c * width)) return c;
        if ((size_t)n == cap) return -1;
        cand.push_back(n);
        keys.insert(keys.end(), k.begin(), k.end());
        return n++;
    }
    const int32_t *key(int c) const { return keys.data() + (size_t)c * width; }
};

// The class tables from the interned keys, laid out [K0 .. K0+4] = (coupling row,
// anisotropy row, anisotropy type, nn, nd), then mnn exchange and mdm DM offsets.
bool store_classes(MixedDev &m, const KeyInterner &ki, size_t k0, size_t mnn, size_t mdm,
                   const std::vector<int32_t> &cls) {
    const size_t ncls = ki.n;
    std::vector<int4> info(ncls);
    std::vector<int32_t> cnb(ncls * std::max<size_t>(mnn, 1)), cdm(ncls * std::max<size_t>(mdm, 1));
    for (size_t c = 0; c < ncls; ++c) {
        const int32_t *k = ki.key((int)c) + k0;
        info[c] = make_int4(k[3] | (k[4] << 16), k[0], k[1], k[2]);
        for (size_t q = 0; q < mnn; ++q) cnb[c * mnn + q] = k[5 + q];
        for (size_t q = 0; q < mdm; ++q) cdm[c * mdm + q] = k[5 + mnn + q];
    }
    const bool ok = store(&m.cls, cls) && store(&m.cinfo, info) && store(&m.cnb, cnb) && store(&m.cdm, cdm);
    m.ncls = ok ? (int)ncls : 0;
    return ok;
}

void drop_classes(MixedDev &m) {
    for (void *q : {(void *)m.cls, (void *)m.cinfo, (void *)m.cnb, (void *)m.cdm}) cudaFree(q);
    m.cls = nullptr;
    m.cinfo = nullptr;
    m.cnb = m.cdm = nullptr;
    m.ncls = 0;
}
}  // namespace

bool mixed_site_classes(Sim &s, const std::vector<int32_t> &row);
bool mixed_species_classes(Sim &s);
bool mixed_uniforms(Sim &s);

// (Re)builds the FP32 copies of the couplings from the FP64 Hamiltonian on the device,
// one row per distinct coupling row (compared bit for bit in FP32) and one anisotropy
// row per distinct (axis, K1, K2, sb).
int mixed_coefficients(Sim &s) {
    const HamDev &h = s.ham;
    const size_t N = h.natom, M = h.mensemble, nh = h.nham, mnn = std::max(h.mnn, 1), mdm = h.do_dm ? h.mnn_dm : 0;
    MixedDev &m = s.mix;
    m.nsp = 0;
    std::vector<double> d, dx, dy, dz, jtd;
    std::vector<int32_t> aham;
    bool ok = cudaStreamSynchronize(s.stream) == cudaSuccess;
    ok = ok && fetch(d, h.ncoup, mnn * nh) && fetch(aham, h.aham, N);
    if (ok && h.do_dm) ok = fetch(dx, h.dmx, mdm * nh) && fetch(dy, h.dmy, mdm * nh) && fetch(dz, h.dmz, mdm * nh);
    if (ok && h.do_jtensor) ok = fetch(jtd, h.jt, mnn * nh * 9);
    // the FP32 content of Hamiltonian row ih, as bits, for the comparison
    const size_t width = mnn + 3 * mdm + (h.do_jtensor ? 9 * mnn : 0);
    auto key = [&](size_t ih) {
        std::vector<uint32_t> k(width);
        size_t q = 0;
        auto put = [&](double v) {
            float f = (float)v;
            std::memcpy(&k[q++], &f, 4);
        };
        for (size_t sl = 0; sl < mnn; ++sl) put(d[sl * nh + ih]);
        for (size_t sl = 0; sl < mdm; ++sl) {
            put(dx[sl * nh + ih]);
            put(dy[sl * nh + ih]);
            put(dz[sl * nh + ih]);
        }
        if (h.do_jtensor)
            for (size_t sl = 0; sl < mnn; ++sl)
                for (int a = 0; a < 9; ++a) put(jtd[(sl * nh + ih) * 9 + a]);
        return k;
    };
    std::map<std::vector<uint32_t>, int> seen;
    std::vector<int> urow(nh), first;
    for (size_t ih = 0; ih < nh && ok; ++ih) {
        auto it = seen.emplace(key(ih), (int)first.size());
        if (it.second) first.push_back((int)ih);
        urow[ih] = it.first->second;
    }
    const size_t nr = first.size();
    m.nrow = (int)nr;
    std::vector<int32_t> row(N);
    for (size_t i = 0; i < N; ++i) row[i] = urow[aham[i]];
    std::vector<float> nc(mnn * nr);
    for (size_t sl = 0; sl < mnn; ++sl)
        for (size_t r = 0; r < nr; ++r) nc[sl * nr + r] = (float)d[sl * nh + first[r]];
    ok = ok && store(&m.row, row) && store(&m.nc, nc);
    if (ok && h.do_dm) {
        std::vector<float4> v(mdm * nr);
        for (size_t sl = 0; sl < mdm; ++sl)
            for (size_t r = 0; r < nr; ++r) {
                const size_t q = sl * nh + first[r];
                v[sl * nr + r] = make_float4((float)dx[q], (float)dy[q], (float)dz[q], 0.f);
            }
        ok = store(&m.dm, v);
    }
    if (ok && h.do_jtensor) {
        std::vector<float> v(mnn * nr * 9);
        for (size_t sl = 0; sl < mnn; ++sl)
            for (size_t r = 0; r < nr; ++r)
                for (int a = 0; a < 9; ++a) v[(sl * nr + r) * 9 + a] = (float)jtd[(sl * nh + first[r]) * 9 + a];
        ok = store(&m.jt, v);
    } else if (ok) {
        ok = store(&m.jt, std::vector<float>());
    }
    if (ok && h.do_aniso) {
        std::vector<double> k1, k2, sb;
        ok = fetch(dx, h.eax, N) && fetch(dy, h.eay, N) && fetch(dz, h.eaz, N) && fetch(k1, h.k1, N) &&
             fetch(k2, h.k2, N) && fetch(sb, h.sb, N);
        std::map<std::vector<uint32_t>, int> aseen;
        std::vector<float4> a;
        std::vector<float2> a2;
        std::vector<int32_t> arow(N);
        for (size_t i = 0; i < N && ok; ++i) {
            const float f[6] = {(float)dx[i], (float)dy[i], (float)dz[i], (float)k1[i], (float)k2[i], (float)sb[i]};
            std::vector<uint32_t> k(6);
            std::memcpy(k.data(), f, sizeof f);
            auto it = aseen.emplace(k, (int)a.size());
            if (it.second) {
                a.push_back(make_float4(f[0], f[1], f[2], f[3]));
                a2.push_back(make_float2(f[4], f[5]));
            }
            arow[i] = it.first->second;
        }
        ok = ok && store(&m.an, a) && store(&m.an2, a2) && store(&m.arow, arow);
    }
    if (ok) {
        ok = fetch(dx, h.ext.x, N * M) && fetch(dy, h.ext.y, N * M) && fetch(dz, h.ext.z, N * M);
        std::vector<float4> v(N * M);
        bool uniform = true;
        for (size_t q = 0; q < N * M && ok; ++q) {
            v[q] = make_float4((float)dx[q], (float)dy[q], (float)dz[q], 0.f);
            uniform = uniform && v[q].x == v[0].x && v[q].y == v[0].y && v[q].z == v[0].z;
        }
        m.ext_uniform = uniform ? 1 : 0;
        if (uniform) v.resize(1);
        ok = ok && store(&m.ext, v);
    }
    if (ok) ok = mixed_site_classes(s, row);
    // per-site lists (too many distinct rows, e.g. a random alloy): try classes that key
    // on the site's own chemical type and look each neighbour's coupling up by its type
    if (ok && m.ncls == 0 && m.spc && !h.do_jtensor) ok = mixed_species_classes(s);
    if (ok) ok = mixed_uniforms(s);
    if (!ok) {
        set_error("precision 3: copying the couplings to FP32 failed");
        return UPPASD_GPU_ECUDA;
    }
    return UPPASD_GPU_OK;
}

// Site classes (see MixedDev): the key of site i is its coupling row, anisotropy row and
// type, list sizes and neighbour offsets j - i.  Kept only when there are at most
// natom / 4 classes (else the per-site lists are the smaller form).
bool mixed_site_classes(Sim &s, const std::vector<int32_t> &row) {
    const HamDev &h = s.ham;
    MixedDev &m = s.mix;
    const size_t N = h.natom, mnn = h.mnn, mdm = h.do_dm ? h.mnn_dm : 0;
    std::vector<int32_t> nl, ns, dl, ds, ta, ar;
    bool ok = fetch(nl, h.nlist, mnn * N) && fetch(ns, h.nsize, N);
    if (ok && h.do_dm) ok = fetch(dl, h.dmlist, mdm * N) && fetch(ds, h.dmsize, N);
    if (ok && h.do_aniso) ok = fetch(ta, h.taniso, N) && fetch(ar, m.arow, N);
    if (!ok) return false;
    const size_t width = 5 + mnn + mdm;
    KeyInterner ki(width, std::max<size_t>(1, N / 4));
    std::vector<int32_t> cls(N), key(width);
    for (size_t i = 0; i < N; ++i) {
        std::fill(key.begin(), key.end(), 0);
        const int nn = ns[i], nd = h.do_dm ? ds[i] : 0;
        key[0] = row[i];
        key[1] = h.do_aniso ? ar[i] : 0;
        key[2] = h.do_aniso ? ta[i] : 0;
        key[3] = nn;
        key[4] = nd;
        for (int q = 0; q < nn; ++q) key[5 + q] = nl[(size_t)q * N + i] - (int32_t)i;
        for (int q = 0; q < nd; ++q) key[5 + mnn + q] = dl[(size_t)q * N + i] - (int32_t)i;
        const int id = ki.id(key);
        if (id < 0) {
            // too many distinct sites: keep reading the per-site lists
            drop_classes(m);
            return true;
        }
        cls[i] = id;
    }
    return store_classes(m, ki, 0, mnn, mdm, cls);
}

// Chemical classes (see MixedDev::nsp): the key of site i is its own chemical type, its
// DM row, anisotropy row and type, list sizes and neighbour offsets j - i, and the
// exchange coupling of each slot must then be a function of the chemical type of that
// slot's neighbour (bit for bit in FP32): a random alloy whose couplings come from a
// (type_i, type_j, shell) table, as the reference's chemical-type-resolved exchange of
// random alloys builds them.  A site that breaks this, or more than natom / (4 nsp)
// classes, leaves the per-site lists in place.
bool mixed_species_classes(Sim &s) {
    const HamDev &h = s.ham;
    MixedDev &m = s.mix;
    const size_t N = h.natom, nh = h.nham, mnn = h.mnn, mdm = h.do_dm ? h.mnn_dm : 0;
    std::vector<int8_t> sp;
    std::vector<double> d, dx, dy, dz;
    std::vector<int32_t> aham, nl, ns, dl, ds, ta, ar;
    bool ok = fetch(sp, m.spc, N) && fetch(d, h.ncoup, std::max<size_t>(mnn, 1) * nh) && fetch(aham, h.aham, N) &&
              fetch(nl, h.nlist, mnn * N) && fetch(ns, h.nsize, N);
    if (ok && h.do_dm)
        ok = fetch(dx, h.dmx, mdm * nh) && fetch(dy, h.dmy, mdm * nh) && fetch(dz, h.dmz, mdm * nh) &&
             fetch(dl, h.dmlist, mdm * N) && fetch(ds, h.dmsize, N);
    if (ok && h.do_aniso) ok = fetch(ta, h.taniso, N) && fetch(ar, m.arow, N);
    if (!ok) return false;
    int nsp = 1;
    for (int8_t v : sp) nsp = std::max(nsp, v + 1);
    // distinct DM rows (FP32 bits) of the Hamiltonian rows
    std::vector<int32_t> dmrow(nh, 0);
    if (mdm) {
        KeyInterner dk(3 * mdm, nh);
        std::vector<int32_t> k(3 * mdm);
        for (size_t ih = 0; ih < nh; ++ih) {
            for (size_t sl = 0; sl < mdm; ++sl) {
                const float f[3] = {(float)dx[sl * nh + ih], (float)dy[sl * nh + ih], (float)dz[sl * nh + ih]};
                std::memcpy(&k[3 * sl], f, sizeof f);
            }
            dmrow[ih] = dk.id(k);
        }
    }
    // key: (chemical type, DM row), then the class tables' layout
    const size_t width = 7 + mnn + mdm;
    KeyInterner ki(width, std::max<size_t>(1, N / (4 * (size_t)nsp)));
    std::vector<int32_t> cls(N), key(width);
    for (size_t i = 0; i < N; ++i) {
        std::fill(key.begin(), key.end(), 0);
        const int nn = ns[i], nd = h.do_dm ? ds[i] : 0;
        key[0] = sp[i];
        key[1] = dmrow[aham[i]];
        key[2] = 0;  // coupling row: the class itself (filled below)
        key[3] = h.do_aniso ? ar[i] : 0;
        key[4] = h.do_aniso ? ta[i] : 0;
        key[5] = nn;
        key[6] = nd;
        for (int q = 0; q < nn; ++q) key[7 + q] = nl[(size_t)q * N + i] - (int32_t)i;
        for (int q = 0; q < nd; ++q) key[7 + mnn + q] = dl[(size_t)q * N + i] - (int32_t)i;
        const int id = ki.id(key);
        if (id < 0) return true;
        cls[i] = id;
    }
    const size_t G = ki.n;
    for (size_t g = 0; g < G; ++g) ki.keys[g * width + 2] = (int32_t)g;
    // the coupling of (slot, class, neighbour type), checked against every site
    const size_t stride = nsp;
    std::vector<float> nc(std::max<size_t>(mnn, 1) * G * stride, 0.f);
    std::vector<uint8_t> have(nc.size(), 0);
    std::vector<int32_t> rep(G, -1);
    for (size_t i = 0; i < N; ++i) {
        const size_t g = cls[i], ih = aham[i];
        if (rep[g] < 0) rep[g] = (int32_t)ih;
        for (int q = 0; q < ns[i]; ++q) {
            const int j = nl[(size_t)q * N + i];
            const size_t x = ((size_t)q * G + g) * stride + sp[j];
            const float v = (float)d[(size_t)q * nh + ih];
            if (!have[x]) {
                nc[x] = v;
                have[x] = 1;
            } else if (std::memcmp(&nc[x], &v, 4) != 0) {
                return true;  // not a function of the neighbour's type: per-site lists
            }
        }
    }
    std::vector<int32_t> row(N);
    for (size_t i = 0; i < N; ++i) row[i] = cls[i];
    ok = store(&m.row, row) && store(&m.nc, nc);
    if (ok && h.do_dm) {
        std::vector<float4> v(mdm * G);
        for (size_t sl = 0; sl < mdm; ++sl)
            for (size_t g = 0; g < G; ++g) {
                const size_t q = sl * nh + rep[g];
                v[sl * G + g] = make_float4((float)dx[q], (float)dy[q], (float)dz[q], 0.f);
            }
        ok = store(&m.dm, v);
    }
    ok = ok && store_classes(m, ki, 2, mnn, mdm, cls);
    m.nrow = (int)G;
    m.nsp = ok ? nsp : 0;
    return ok;
}

// Damping, Lande factor, temperature and moment passed as scalars when they are the
// same for every site (and ensemble); again after set_temperature.
bool mixed_uniforms(Sim &s) {
    const HamDev &h = s.ham;
    MixedDev &m = s.mix;
    const size_t N = h.natom, M = h.mensemble;
    std::vector<double> v;
    auto uniform = [&](const double *d, size_t n, int &flag, double &val) {
        if (!fetch(v, d, n)) return false;
        flag = 1;
        for (size_t q = 1; q < n && flag; ++q) flag = v[q] == v[0];
        val = v.empty() ? 0.0 : v[0];
        return true;
    };
    double lam, g, T, mm;
    if (!(uniform(s.llg.lambda, N, m.uni_lam, lam) && uniform(s.llg.landeg, N, m.uni_g, g) &&
          uniform(s.llg.temp, N, m.uni_T, T) && uniform(s.llg.mmom, N * M, m.uni_m, mm)))
        return false;
    m.lam_u = (float)lam;
    m.g_u = (float)g;
    m.T_u = (float)T;
    m.mmom_u = mm;
    return true;
}

// set_temperature on precision 3: the uniform-temperature scalar follows the new array.
void mixed_temperature(Sim &s, const double *temp_array) {
    MixedDev &m = s.mix;
    const int N = s.ham.natom;
    m.uni_T = 1;
    for (int i = 1; i < N && m.uni_T; ++i) m.uni_T = temp_array[i] == temp_array[0];
    m.T_u = (float)temp_array[0];
}

int mixed_init(Sim &s, const int32_t *species) {
    if (!(s.llg.sdealgh == 1 || s.llg.sdealgh == 4 || s.llg.sdealgh == 5 || s.llg.sdealgh == 6 ||
          s.llg.sdealgh == 7 || s.llg.sdealgh == 11)) {
        set_error("precision 3 (FP32 gather, FP64 master): unknown SDEalgh");
        return UPPASD_GPU_EUNSUPPORTED;
    }
    const bool ds = s.precision == 4;
    const size_t n = (size_t)s.ham.natom * s.ham.mensemble;
    MixedDev &m = s.mix;
    m.ds = ds ? 1 : 0;
    cudaError_t e = cudaMalloc(&m.mt, n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&m.mp, n * sizeof(float4));
    for (float **q : {&m.b2x, &m.b2y, &m.b2z})
        if (e == cudaSuccess) e = cudaMalloc(q, n * sizeof(float));
    if (ds)
        for (float **q : {&m.lox, &m.loy, &m.loz})
            if (e == cudaSuccess) e = cudaMalloc(q, n * sizeof(float));
    if (e != cudaSuccess) {
        set_error(std::string("precision 3 set-up: ") + cudaGetErrorString(e));
        return UPPASD_GPU_ENOMEM;
    }
    s.bytes_allocated += n * (2 * sizeof(float4) + 3 * sizeof(float));
    m.valid = 0;
    // the caller's chemical types (0..15) for chemically resolved couplings;
    // UPPASD_CHEMICAL_CLASSES=0 keeps the per-site lists (for comparisons)
    const char *cc = getenv("UPPASD_CHEMICAL_CLASSES");
    if (species && !(cc && cc[0] == '0')) {
        const size_t N = s.ham.natom;
        std::vector<int8_t> sp(N);
        bool in_range = true;
        for (size_t i = 0; i < N && in_range; ++i) {
            in_range = species[i] >= 0 && species[i] < 16;
            sp[i] = (int8_t)species[i];
        }
        if (in_range && !store(&m.spc, sp)) {
            set_error("precision 3 set-up: chemical types");
            return UPPASD_GPU_ENOMEM;
        }
    }
    return mixed_coefficients(s);
}

void mixed_free(Sim &s) {
    MixedDev &m = s.mix;
    for (void *q : {(void *)m.mt, (void *)m.mp, (void *)m.b2x, (void *)m.b2y, (void *)m.b2z, (void *)m.nc,
                    (void *)m.dm, (void *)m.jt, (void *)m.an, (void *)m.an2, (void *)m.ext, (void *)m.row,
                    (void *)m.arow, (void *)m.cls, (void *)m.cinfo, (void *)m.cnb, (void *)m.cdm, (void *)m.moved,
                    (void *)m.lox, (void *)m.loy, (void *)m.loz, (void *)m.spc})
        cudaFree(q);
    m = MixedDev{};
}

// precision 4: e / eM from the double-single master when the steps have moved it
int mixed_sync(Sim &s) {
    if (!s.mix.ds || !s.mix.e_stale) return UPPASD_GPU_OK;
    const int64_t n = (int64_t)s.ham.natom * s.ham.mensemble;
    mixed_ds_to_master<<<(unsigned)((n + 255) / 256), 256, 0, s.stream>>>(s.mix, s.e, s.eM, s.llg.mmom, n);
    UPPASD_CUDA_TRY(cudaGetLastError());
    s.mix.e_stale = 0;
    return UPPASD_GPU_OK;
}

// The mirror (and the double-single master) from e when something else wrote e
// (put_moments, Monte Carlo).
int mixed_ready(Sim &s) {
    if (s.mix.valid) return UPPASD_GPU_OK;
    // the mirror was marked stale while the double-single master was ahead of e (by a
    // caller that did not write e): e from the master first, so that nothing is lost
    if (const int rc = mixed_sync(s)) return rc;
    const int64_t n = (int64_t)s.ham.natom * s.ham.mensemble;
    if (s.mix.ds)
        mixed_mirror_ds<<<(unsigned)((n + 255) / 256), 256, 0, s.stream>>>(s.mix, s.e, s.llg.mmom, n);
    else
        mixed_mirror<<<(unsigned)((n + 255) / 256), 256, 0, s.stream>>>(s.e, s.llg.mmom, s.mix.mt, n);
    UPPASD_CUDA_TRY(cudaGetLastError());
    s.mix.valid = 1;
    return UPPASD_GPU_OK;
}

// precision 3 heat-bath sweeps (mc_run mode 'H')
int mixed_metropolis_sweeps(Sim &s, double temperature, int64_t nsweeps) {
    if (s.ncolour <= 0) {
        set_error("no colouring available for Monte Carlo");
        return UPPASD_GPU_ESTATE;
    }
    int rc = mixed_sync(s);  // sites the sweeps reject keep their FP64 state
    if (!rc) rc = mixed_ready(s);
    if (rc) return rc;
    s.sqm_valid = 0;  // the square path's mirror does not follow these updates
    // flip_a's beta = 1 / (k_B (T + 1e-15)) and the Gaussian width (2/25)(k_B T / mu_B)^0.2
    // (montecarlo.f90:142, a REAL(4) constant), as the FP64 path forms them
    const float beta_mub = (float)(s.ham.mub / s.ham.kbolt / (1.0 * temperature + 1.0e-15));
    const float delta = (float)((double)(2.0f / 25.0f) * pow(s.ham.kbolt * temperature / s.ham.mub, 0.20));
    const int64_t nm = (int64_t)s.ham.natom * s.ham.mensemble;
    if (!s.mix.moved) {
        // the moved marks, cleared once; the pass after the sweeps clears what it uses
        uint8_t *mv = nullptr;
        UPPASD_CUDA_TRY(cudaMalloc(&mv, (size_t)nm));
        const cudaError_t e = cudaMemsetAsync(mv, 0, (size_t)nm, s.stream);
        if (e != cudaSuccess) {
            cudaFree(mv);
            set_error(std::string("mc_run (precision 3): ") + cudaGetErrorString(e));
            return UPPASD_GPU_ECUDA;
        }
        s.mix.moved = mv;
    }
    for (int64_t sw = 0; sw < nsweeps; ++sw) {
        for (int c = 0; c < s.ncolour; ++c) {
            const int beg = s.colour_start_h[c], n = s.colour_start_h[c + 1] - beg;
            if (n == 0) continue;
            const int64_t tot = (int64_t)n * s.ham.mensemble;
            mixed_metropolis<<<(unsigned)((tot + 255) / 256), 256, 0, s.stream>>>(
                s.ham, s.mix, s.colour_sites + beg, n, beta_mub, delta, s.llg.seed, s.mc_sweep);
        }
        s.mc_sweep += 1;
    }
    if (nsweeps > 0) {
        mixed_master_from_mirror<<<(unsigned)((nm + 255) / 256), 256, 0, s.stream>>>(s.mix, s.e, s.eM, s.llg.mmom,
                                                                                   nm, s.mix.moved);
        if (s.mix.ds) s.mix.valid = 0;  // the double-single residuals are made again from e
    }
    UPPASD_CUDA_TRY(cudaGetLastError());
    return UPPASD_GPU_OK;
}

int mixed_heat_bath_sweeps(Sim &s, double temperature, int64_t nsweeps, const float *betak) {
    if (s.ncolour <= 0) {
        set_error("no colouring available for Monte Carlo");
        return UPPASD_GPU_ESTATE;
    }
    int rc = mixed_sync(s);
    if (!rc) rc = mixed_ready(s);
    if (rc) return rc;
    s.sqm_valid = 0;  // the square path's mirror does not follow these updates
    const float beta_mub = betak ? 0.f : (float)(s.ham.mub / (s.ham.kbolt * temperature));
    for (int64_t sw = 0; sw < nsweeps; ++sw) {
        for (int c = 0; c < s.ncolour; ++c) {
            const int beg = s.colour_start_h[c], n = s.colour_start_h[c + 1] - beg;
            if (n == 0) continue;
            const int64_t tot = (int64_t)n * s.ham.mensemble;
            mixed_heat_bath<<<(unsigned)((tot + 255) / 256), 256, 0, s.stream>>>(
                s.ham, s.mix, s.colour_sites + beg, n, beta_mub, betak, s.llg.seed, s.mc_sweep);
        }
        s.mc_sweep += 1;
    }
    if (nsweeps > 0) {
        const int64_t nm = (int64_t)s.ham.natom * s.ham.mensemble;
        mixed_master_from_mirror<<<(unsigned)((nm + 255) / 256), 256, 0, s.stream>>>(s.mix, s.e, s.eM, s.llg.mmom,
                                                                                   nm, nullptr);
        if (s.mix.ds) s.mix.valid = 0;
    }
    UPPASD_CUDA_TRY(cudaGetLastError());
    return UPPASD_GPU_OK;
}

int mixed_step(Sim &s, int64_t step_offset, int phase) {
    MixArgs a;
    a.h = s.ham;
    a.lambda = s.llg.lambda;
    a.temp = s.llg.temp;
    a.landeg = s.llg.landeg;
    a.mmom = s.llg.mmom;
    const double gama = s.ham.gama, kbolt = s.ham.kbolt, mub = s.ham.mub;
    a.dt_dep = (float)(s.llg.delta_t * gama);
    a.dt_mid = (float)(s.llg.delta_t * s.llg.bn * gama);
    a.c_dp = (float)(2.0 * kbolt / (s.llg.delta_t * gama * mub));
    a.c_dk = (float)(kbolt / (mub * s.llg.bn));
    a.c_heun = (float)(s.llg.delta_t * gama * kbolt / mub);
    a.tau_dt = (float)(s.llg.relaxtime / s.llg.delta_t);
    a.dtg_llgi = (float)(-s.llg.delta_t * gama);
    a.perp = s.llg.perp;
    a.mpast = s.mpast;
    a.temprescale = (float)s.llg.temprescale;
    a.noise_on = s.llg.noise_on;
    a.nz.mode = s.llg.noise_mode;
    a.nz.seed = s.llg.seed;
    a.nz.inj = s.llg.inj;
    a.nz.inj_first = s.llg.inj_first;
    a.d_step = s.llg.d_step;
    a.step_off = step_offset;
    a.e = s.e;
    a.eM = s.eM;
    a.c = s.mix;
    const int64_t n = (int64_t)s.ham.natom * s.ham.mensemble;
    const int grid = (int)((n + 255) / 256);
    auto run = [&](auto alg) {
        constexpr int ALG = decltype(alg)::value;
        if (phase & 1) mixed_predict<ALG><<<grid, 256, 0, s.stream>>>(a);
        if (phase & 2) {
            if (s.mix.ds) mixed_correct<ALG, true><<<grid, 256, 0, s.stream>>>(a);
            else mixed_correct<ALG, false><<<grid, 256, 0, s.stream>>>(a);
        }
    };
    if ((phase & 2) && s.mix.ds) s.mix.e_stale = 1;
    switch (s.llg.sdealgh) {
    case 1: run(std::integral_constant<int, 1>{}); break;
    case 4: run(std::integral_constant<int, 4>{}); break;
    case 5: run(std::integral_constant<int, 5>{}); break;
    case 6: run(std::integral_constant<int, 6>{}); break;
    case 7: run(std::integral_constant<int, 7>{}); break;
    case 11: run(std::integral_constant<int, 11>{}); break;
    default: set_error("unsupported SDEalgh"); return UPPASD_GPU_EUNSUPPORTED;
    }
    UPPASD_CUDA_TRY(cudaGetLastError());
    return UPPASD_GPU_OK;
}

}  // namespace uppasd
