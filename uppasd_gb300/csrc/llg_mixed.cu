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
#include "common.cuh"
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
    float temprescale;
    int noise_on;
    NoiseArgs nz;          // Philox (FP32 Box-Muller here), injected normals, or none
    const int64_t *d_step;
    int64_t step_off;
    Vec3D e, eM;           // FP64 master
    float4 *mt, *mp;       // mirror at t, predictor
    float *b2x, *b2y, *b2z;
};

// FP32 effective field of site i from full moments m.w * m.xyz, in the FP64 field's
// term order (exchange or tensor, DMI, anisotropy, Zeeman).
__device__ __forceinline__ void field_f32(const HamDev &h, const float4 *m, int i, int k, float B[3]) {
    const int N = h.natom;
    const size_t off = (size_t)k * N;
    const int ih = h.aham[i];
    const int nn = h.nsize[i];
    float bs[3] = {0.f, 0.f, 0.f}, bq[3] = {0.f, 0.f, 0.f};
    if (h.do_jtensor) {
        for (int s = 0; s < nn; ++s) {
            const int j = __ldg(&h.nlist[(size_t)s * N + i]);
            const float4 v = m[off + j];
            const float m1 = v.w * v.x, m2 = v.w * v.y, m3 = v.w * v.z;
            const double *J = h.jt + ((size_t)s * h.nham + ih) * 9;
#pragma unroll
            for (int a = 0; a < 3; ++a)
                bs[a] += (float)__ldg(&J[3 * a]) * m1 + (float)__ldg(&J[3 * a + 1]) * m2 +
                         (float)__ldg(&J[3 * a + 2]) * m3;
        }
    } else {
        for (int s = 0; s < nn; ++s) {
            const int j = __ldg(&h.nlist[(size_t)s * N + i]);
            const float4 v = m[off + j];
            const float c = (float)__ldg(&h.ncoup[(size_t)s * h.nham + ih]) * v.w;
            bs[0] = fmaf(c, v.x, bs[0]);
            bs[1] = fmaf(c, v.y, bs[1]);
            bs[2] = fmaf(c, v.z, bs[2]);
        }
    }
    if (h.do_dm) {
        const int nd = h.dmsize[i];
        for (int s = 0; s < nd; ++s) {
            const int j = __ldg(&h.dmlist[(size_t)s * N + i]);
            const size_t d = (size_t)s * h.nham + ih;
            const float d0 = (float)h.dmx[d], d1 = (float)h.dmy[d], d2 = (float)h.dmz[d];
            const float4 v = m[off + j];
            const float m1 = v.w * v.x, m2 = v.w * v.y, m3 = v.w * v.z;
            bs[0] += d2 * m2 - d1 * m3;
            bs[1] += d0 * m3 - d2 * m1;
            bs[2] += d1 * m1 - d0 * m2;
        }
    }
    if (h.do_aniso) {
        const float4 me = m[off + i];
        const float m1 = me.w * me.x, m2 = me.w * me.y, m3 = me.w * me.z;
        const int ta = h.taniso[i];
        const float e0 = (float)h.eax[i], e1 = (float)h.eay[i], e2 = (float)h.eaz[i];
        const float ka0 = (float)h.k1[i], ka1 = (float)h.k2[i];
        if (ta == 1 || ta == 7) {
            const float tt1 = m1 * e0 + m2 * e1 + m3 * e2;
            const float tt3 = 2.0f * tt1 * (ka0 + 2.0f * ka1 * (1.0f - tt1 * tt1));
            bs[0] -= tt3 * e0;
            bs[1] -= tt3 * e1;
            bs[2] -= tt3 * e2;
        }
        if (ta == 2 || ta == 7) {
            const float t0 = 2.0f * ka0 * m1 * (m2 * m2 + m3 * m3) + 2.0f * ka1 * m1 * (m2 * m2 * (m3 * m3));
            const float t1 = 2.0f * ka0 * m2 * (m3 * m3 + m1 * m1) + 2.0f * ka1 * m2 * (m3 * m3 * (m1 * m1));
            const float t2 = 2.0f * ka0 * m3 * (m1 * m1 + m2 * m2) + 2.0f * ka1 * m3 * (m1 * m1 * (m2 * m2));
            const float sc = ta == 2 ? 1.0f : (float)h.sb[i];
            float *dst = ta == 2 ? bs : bq;
            dst[0] += t0 * sc;
            dst[1] += t1 * sc;
            dst[2] += t2 * sc;
        }
    }
    B[0] = bs[0] + (bq[0] + (float)h.ext.x[off + i]);
    B[1] = bs[1] + (bq[1] + (float)h.ext.y[off + i]);
    B[2] = bs[2] + (bq[2] + (float)h.ext.z[off + i]);
}

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

// thermal field / midpoint noise of site i at `step` (regenerated by the corrector)
template <int ALG>
__device__ __forceinline__ void noise_f32(const MixArgs &a, int i, int k, int64_t step, float lam, float mm,
                                          float out[3]) {
    float z[3];
    if (ALG == 1 && !a.noise_on) {
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
    const float T = (float)a.temp[i] * a.temprescale;
    float sigma;
    if (ALG == 5) {
        sigma = sqrtf(a.c_dp * lam * T / mm);
    } else {
        sigma = sqrtf(2.0f * (a.c_dk * lam / (1.0f + lam * lam)) * T / mm);
    }
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
    field_f32(a.h, a.mt, i, k, B);
    const float4 me = a.mt[o];
    const float e[3] = {me.x, me.y, me.z};
    const float lam = (float)a.lambda[i], mm = me.w;
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
        a.b2x[o] = bd[0];
        a.b2y[o] = bd[1];
        a.b2z[o] = bd[2];
    } else {
        const float dt = a.dt_mid / (1.0f + lam * lam);
        const float g = (float)a.landeg[i];
        const float dtg = dt * g, sqrtdtg = sqrtf(dt) * g;
        float A[3], et[3];
        midpoint_A_f32(lam, dtg, sqrtdtg, e, B, r, A);
        cayley_f32(A, e, et);
        p[0] = 0.5f * (e[0] + et[0]);
        p[1] = 0.5f * (e[1] + et[1]);
        p[2] = 0.5f * (e[2] + et[2]);
    }
    a.mp[o] = make_float4(p[0], p[1], p[2], mm);
}

template <int ALG>
__global__ void __launch_bounds__(256) mixed_correct(MixArgs a) {
    const int N = a.h.natom, M = a.h.mensemble;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)N * M) return;
    const int k = (int)(t / N), i = (int)(t - (int64_t)k * N);
    const size_t o = (size_t)k * N + i;
    const int64_t step = *a.d_step + a.step_off;
    float B[3];
    field_f32(a.h, a.mp, i, k, B);
    const float4 me = a.mt[o], mpv = a.mp[o];
    const float e[3] = {me.x, me.y, me.z}, pr[3] = {mpv.x, mpv.y, mpv.z};
    const float lam = (float)a.lambda[i], mm = me.w;
    float r[3];
    noise_f32<ALG>(a, i, k, step, lam, mm, r);
    float d[3];
    if (ALG == 5) {
        const float bl[3] = {B[0] + r[0], B[1] + r[1], B[2] + r[2]};
        float bd[3] = {bl[0] + lam * (pr[1] * bl[2] - pr[2] * bl[1]), bl[1] + lam * (pr[2] * bl[0] - pr[0] * bl[2]),
                       bl[2] + lam * (pr[0] * bl[1] - pr[1] * bl[0])};
        bd[0] = 0.5f * bd[0] + 0.5f * a.b2x[o];
        bd[1] = 0.5f * bd[1] + 0.5f * a.b2y[o];
        bd[2] = 0.5f * bd[2] + 0.5f * a.b2z[o];
        rotation_delta_f32(bd, e, a.dt_dep / (1.0f + lam * lam), d);
    } else {
        const float dt = a.dt_mid / (1.0f + lam * lam);
        const float g = (float)a.landeg[i];
        const float dtg = dt * g, sqrtdtg = sqrtf(dt) * g;
        float A[3], et[3];
        midpoint_A_f32(lam, dtg, sqrtdtg, pr, B, r, A);
        cayley_f32(A, e, et);
        d[0] = et[0] - e[0];
        d[1] = et[1] - e[1];
        d[2] = et[2] - e[2];
    }
    // FP64 master: add the change, renormalise, refresh the mirror
    double e0 = a.e.x[o] + (double)d[0], e1 = a.e.y[o] + (double)d[1], e2 = a.e.z[o] + (double)d[2];
    const double xx = fma(e2, e2, fma(e1, e1, e0 * e0)) - 1.0;
    const double sc = fma(xx, fma(0.375, xx, -0.5), 1.0);  // 1/sqrt(1+x) to second order, |x| ~ 1e-7
    e0 *= sc;
    e1 *= sc;
    e2 *= sc;
    const double mmd = a.mmom[o];
    a.e.x[o] = e0;
    a.e.y[o] = e1;
    a.e.z[o] = e2;
    a.eM.x[o] = mmd * e0;
    a.eM.y[o] = mmd * e1;
    a.eM.z[o] = mmd * e2;
    a.mt[o] = make_float4((float)e0, (float)e1, (float)e2, mm);
}

__global__ void mixed_mirror(Vec3D e, const double *mmom, float4 *mt, int64_t n) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) mt[t] = make_float4((float)e.x[t], (float)e.y[t], (float)e.z[t], (float)mmom[t]);
}

}  // namespace

int mixed_init(Sim &s) {
    if (!(s.llg.sdealgh == 1 || s.llg.sdealgh == 5)) {
        set_error("precision 3 (FP32 gather, FP64 master) implements SDEalgh 1 and 5");
        return UPPASD_GPU_EUNSUPPORTED;
    }
    const size_t n = (size_t)s.ham.natom * s.ham.mensemble;
    MixedDev &m = s.mix;
    cudaError_t e = cudaMalloc(&m.mt, n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&m.mp, n * sizeof(float4));
    for (float **q : {&m.b2x, &m.b2y, &m.b2z})
        if (e == cudaSuccess) e = cudaMalloc(q, n * sizeof(float));
    if (e != cudaSuccess) {
        set_error(std::string("precision 3 set-up: ") + cudaGetErrorString(e));
        return UPPASD_GPU_ENOMEM;
    }
    s.bytes_allocated += n * (2 * sizeof(float4) + 3 * sizeof(float));
    m.valid = 0;
    return UPPASD_GPU_OK;
}

void mixed_free(Sim &s) {
    MixedDev &m = s.mix;
    for (void *q : {(void *)m.mt, (void *)m.mp, (void *)m.b2x, (void *)m.b2y, (void *)m.b2z}) cudaFree(q);
    m = MixedDev{};
}

// The mirror from the master when something else wrote e (put_moments, Monte Carlo).
int mixed_ready(Sim &s) {
    if (s.mix.valid) return UPPASD_GPU_OK;
    const int64_t n = (int64_t)s.ham.natom * s.ham.mensemble;
    mixed_mirror<<<(unsigned)((n + 255) / 256), 256, 0, s.stream>>>(s.e, s.llg.mmom, s.mix.mt, n);
    UPPASD_CUDA_TRY(cudaGetLastError());
    s.mix.valid = 1;
    return UPPASD_GPU_OK;
}

int mixed_step(Sim &s, int64_t step_offset, int phase) {
    MixArgs a;
    a.h = s.ham;
    a.lambda = s.llg.lambda;
    a.temp = s.llg.temp;
    a.landeg = s.llg.landeg;
    a.mmom = s.llg.mmom;
    a.dt_dep = (float)(s.llg.delta_t * kGama);
    a.dt_mid = (float)(s.llg.delta_t * s.llg.bn * kGama);
    a.c_dp = (float)(2.0 * kKbolt / (s.llg.delta_t * kGama * kMub));
    a.c_dk = (float)(kKbolt / (kMub * s.llg.bn));
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
    a.mt = s.mix.mt;
    a.mp = s.mix.mp;
    a.b2x = s.mix.b2x;
    a.b2y = s.mix.b2y;
    a.b2z = s.mix.b2z;
    const int64_t n = (int64_t)s.ham.natom * s.ham.mensemble;
    const int grid = (int)((n + 255) / 256);
    if (s.llg.sdealgh == 5) {
        if (phase & 1) mixed_predict<5><<<grid, 256, 0, s.stream>>>(a);
        if (phase & 2) mixed_correct<5><<<grid, 256, 0, s.stream>>>(a);
    } else {
        if (phase & 1) mixed_predict<1><<<grid, 256, 0, s.stream>>>(a);
        if (phase & 2) mixed_correct<1><<<grid, 256, 0, s.stream>>>(a);
    }
    UPPASD_CUDA_TRY(cudaGetLastError());
    return UPPASD_GPU_OK;
}

}  // namespace uppasd
