// llg_generic.cu -- FP64 LLG step on an arbitrary neighbour list (the parity path).
//
// One thread per (site, ensemble).  Two fused kernels per step:
//   llg_predict : effective field at m(t) + evolve_first  (writes p, pM[, b2])
//   llg_correct : effective field at the predictor + evolve_second + moment_update
// The arithmetic follows the reference's Fortran expression order term by term
// and this file is compiled with --fmad=false, so on the same inputs the result
// differs from the FP64 CPU restatement only through the last-ulp behaviour of
// sin/cos/log.  Reference routines:
//   field      Hamiltonian/hamiltonianactions.f90:183-249 (heisenberg :431-466,
//              DM :546-580, uniaxial :842-879, cubic :883-919)
//   Depondt    Evolution/depondt.f90:136-191 and 284-329
//   midpoint   Evolution/midpoint.f90:123-177 and 274-318, noise rannum
//              RNG/randomnumbers.f90:660-745
//   Heun       Evolution/heun_proper.f90:28-161, 261-530
//   SIB        Evolution/sphmidpoint.f90:36-477
//   LLGI       Evolution/llgi.f90:18-278 (SDEalgh 11, inertial LLG)
//   moments    Evolution/updatemoments.f90:48-77
#include "common.cuh"
#include "field_fp64.cuh"
#include "sim.h"

namespace uppasd {

__device__ __forceinline__ void rodrigues(const double bdup[3], const double e[3], double dt, double gama,
                                          double lldamp, double mr[3]) {
    double Bnorm = bdup[0] * bdup[0] + bdup[1] * bdup[1] + bdup[2] * bdup[2];
    Bnorm = sqrt(Bnorm) + 1.0e-15;
    double hx = bdup[0] / Bnorm, hy = bdup[1] / Bnorm, hz = bdup[2] / Bnorm;
    double v = Bnorm * dt * gama * lldamp;
    double cosv = cos(v), sinv = sin(v), u = 1.0 - cosv;
    mr[0] = hx * hx * u * e[0] + cosv * e[0] + hx * hy * u * e[1] - hz * sinv * e[1] + hx * hz * u * e[2] + hy * sinv * e[2];
    mr[1] = hy * hx * u * e[0] + hz * sinv * e[0] + hy * hy * u * e[1] + cosv * e[1] + hy * hz * u * e[2] - hx * sinv * e[2];
    mr[2] = hx * hz * u * e[0] - hy * sinv * e[0] + hz * hy * u * e[1] + hx * sinv * e[1] + hz * hz * u * e[2] + cosv * e[2];
}

__device__ __forceinline__ void damped_field(const double bloc[3], const double e[3], double lam, double bdup[3]) {
    bdup[0] = 0.0 + bloc[0] + lam * e[1] * bloc[2] - lam * e[2] * bloc[1];
    bdup[1] = 0.0 + bloc[1] + lam * e[2] * bloc[0] - lam * e[0] * bloc[2];
    bdup[2] = 0.0 + bloc[2] + lam * e[0] * bloc[1] - lam * e[1] * bloc[0];
}

__device__ __forceinline__ void cayley(const double A[3], const double e[3], double et[3], double &detAi) {
    detAi = 1.0 / (1.0 + (A[0] * A[0] + A[1] * A[1] + A[2] * A[2]));
    double a0 = e[0] + e[1] * A[2] - e[2] * A[1];
    double a1 = e[1] + e[2] * A[0] - e[0] * A[2];
    double a2 = e[2] + e[0] * A[1] - e[1] * A[0];
    et[0] = a0 * (1.0 + A[0] * A[0]) + a1 * (A[0] * A[1] + A[2]) + a2 * (A[0] * A[2] - A[1]);
    et[1] = a0 * (A[1] * A[0] - A[2]) + a1 * (1.0 + A[1] * A[1]) + a2 * (A[1] * A[2] + A[0]);
    et[2] = a0 * (A[2] * A[0] + A[1]) + a1 * (A[2] * A[1] - A[0]) + a2 * (1.0 + A[2] * A[2]);
}

__device__ __forceinline__ void midpoint_A(double lam, double dtg, double sqrtdtg, const double e[3],
                                           const double b[3], const double r[3], double A[3]) {
    double a1[3], s1[3];
    a1[0] = -0.0 - b[0] - lam * (e[1] * b[2] - e[2] * b[1]);
    a1[1] = -0.0 - b[1] - lam * (e[2] * b[0] - e[0] * b[2]);
    a1[2] = -0.0 - b[2] - lam * (e[0] * b[1] - e[1] * b[0]);
    s1[0] = -r[0] - lam * (e[1] * r[2] - e[2] * r[1]);
    s1[1] = -r[1] - lam * (e[2] * r[0] - e[0] * r[2]);
    s1[2] = -r[2] - lam * (e[0] * r[1] - e[1] * r[0]);
#pragma unroll
    for (int c = 0; c < 3; ++c) A[c] = 0.5 * dtg * a1[c] + 0.5 * sqrtdtg * s1[c];
}

__device__ __forceinline__ void sib_a1s1(double lam, const double e[3], const double b[3], const double f[3],
                                         double a1[3], double s1[3]) {
    a1[0] = -b[0] - lam * (e[1] * b[2] - e[2] * b[1]);
    a1[1] = -b[1] - lam * (e[2] * b[0] - e[0] * b[2]);
    a1[2] = -b[2] - lam * (e[0] * b[1] - e[1] * b[0]);
    s1[0] = -f[0] - lam * (e[1] * f[2] - e[2] * f[1]);
    s1[1] = -f[1] - lam * (e[2] * f[0] - e[0] * f[2]);
    s1[2] = -f[2] - lam * (e[0] * f[1] - e[1] * f[0]);
}

__device__ __forceinline__ void sib_fixed_point(const double e1[3], const double a1[3], const double s1[3],
                                                double dtg, double sqrtdtg, double efp[3]) {
    const double epsilona = (double)1e-12f;  // REAL(4) literal in sphmidpoint.f90:165
    double f0[3] = {e1[0], e1[1], e1[2]};
    for (int it = 1; it <= 100; ++it) {
        double f1[3], fd[3], fs[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            f1[c] = 0.5 * (e1[c] + f0[c]);
            fd[c] = dtg * f1[c];
            fs[c] = sqrtdtg * f1[c];
        }
        efp[0] = e1[0] + fd[1] * a1[2] - fd[2] * a1[1] + fs[1] * s1[2] - fs[2] * s1[1];
        efp[1] = e1[1] + fd[2] * a1[0] - fd[0] * a1[2] + fs[2] * s1[0] - fs[0] * s1[2];
        efp[2] = e1[2] + fd[0] * a1[1] - fd[1] * a1[0] + fs[0] * s1[1] - fs[1] * s1[0];
        double dx = sqrt((f0[0] - efp[0]) * (f0[0] - efp[0]));
        double dy = sqrt((f0[1] - efp[1]) * (f0[1] - efp[1]));
        double dz = sqrt((f0[2] - efp[2]) * (f0[2] - efp[2]));
        if (dx < epsilona && dy < epsilona && dz < epsilona) break;
        f0[0] = efp[0];
        f0[1] = efp[1];
        f0[2] = efp[2];
    }
}

// sispht / sisphf (Evolution/sphmidpoint.f90:485-923, SDEalgh 7): the SIB iteration with
// the midpoint direction normalised, u = (e1 + efp0) / |e1 + efp0|.  efp is the last
// iterate; f0 the one before it when the tolerance ended the loop (else the last one).
__device__ __forceinline__ void sisph_fixed_point(const double e1[3], const double a1[3], const double s1[3],
                                                  double dtg, double sqrtdtg, double efp[3], double f0[3]) {
    const double epsilona = (double)1e-12f;  // REAL(4) literal in sphmidpoint.f90
    f0[0] = e1[0];
    f0[1] = e1[1];
    f0[2] = e1[2];
    for (int it = 1; it <= 100; ++it) {
        const double unorm = sqrt((e1[0] + f0[0]) * (e1[0] + f0[0]) + (e1[1] + f0[1]) * (e1[1] + f0[1]) +
                                  (e1[2] + f0[2]) * (e1[2] + f0[2]));
        double fd[3], fs[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double u = (e1[c] + f0[c]) / unorm;
            fd[c] = dtg * u;
            fs[c] = sqrtdtg * u;
        }
        efp[0] = e1[0] + fd[1] * a1[2] - fd[2] * a1[1] + fs[1] * s1[2] - fs[2] * s1[1];
        efp[1] = e1[1] + fd[2] * a1[0] - fd[0] * a1[2] + fs[2] * s1[0] - fs[0] * s1[2];
        efp[2] = e1[2] + fd[0] * a1[1] - fd[1] * a1[0] + fs[0] * s1[1] - fs[1] * s1[0];
        double dx = sqrt((f0[0] - efp[0]) * (f0[0] - efp[0]));
        double dy = sqrt((f0[1] - efp[1]) * (f0[1] - efp[1]));
        double dz = sqrt((f0[2] - efp[2]) * (f0[2] - efp[2]));
        if (dx < epsilona && dy < epsilona && dz < epsilona) break;
        f0[0] = efp[0];
        f0[1] = efp[1];
        f0[2] = efp[2];
    }
}

// llgiheun (Evolution/llgi.f90:178-278): m_new = A^-1 B, A = I + beta [e1]x, from
// m(t) = e1, m(t - dt) = et and the field h.
__device__ __forceinline__ void llgi_heun(double lam, double delta_t, double gama, double relaxtime,
                                          const double et[3], const double e1[3], const double h[3], double out[3]) {
    const double alfa = lam;
    const double beta = -alfa * (1.0 + relaxtime / delta_t);
    const double zeta = -alfa * (relaxtime / delta_t);
    const double dtg = -delta_t * gama;
    const double A12 = -beta * e1[2], A13 = beta * e1[1];
    const double A21 = beta * e1[2], A23 = -beta * e1[0];
    const double A31 = -beta * e1[1], A32 = beta * e1[0];
    double det = 1.0 - A23 * A32 - A12 * A21 - A13 * A31;
    det = 1.0 / det;
    const double I11 = (1.0 - A32 * A23) * det, I12 = (A13 * A32 - A12) * det, I13 = (A12 * A23 - A13) * det;
    const double I21 = (A23 * A31 - A21) * det, I22 = (1.0 - A31 * A13) * det, I23 = (A13 * A21 - A23) * det;
    const double I31 = (A21 * A32 - A31) * det, I32 = (A12 * A31 - A32) * det, I33 = (1.0 - A21 * A12) * det;
    const double B1 = e1[0] + dtg * (e1[1] * h[2] - e1[2] * h[1]) + zeta * (e1[2] * et[1] - e1[1] * et[2]);
    const double B2 = e1[1] + dtg * (e1[2] * h[0] - e1[0] * h[2]) + zeta * (e1[0] * et[2] - e1[2] * et[0]);
    const double B3 = e1[2] + dtg * (e1[0] * h[1] - e1[1] * h[0]) + zeta * (e1[1] * et[0] - e1[0] * et[1]);
    out[0] = I11 * B1 + I12 * B2 + I13 * B3;
    out[1] = I21 * B1 + I22 * B2 + I23 * B3;
    out[2] = I31 * B1 + I32 * B2 + I33 * B3;
}

// perp = 'Y' (Evolution/evolution.f90:104-112, :327-335): B <- B - e (B . e)
__device__ __forceinline__ void perp_project(double B[3], const double e[3]) {
    const double d = B[0] * e[0] + B[1] * e[1] + B[2] * e[2];
    B[0] = B[0] - e[0] * d;
    B[1] = B[1] - e[1] * d;
    B[2] = B[2] - e[2] * d;
}

struct StepArgs {
    HamDev h;
    NoiseArgs nz;
    const double *lambda, *temp, *landeg, *mmom;
    double delta_t, bn, temprescale, relaxtime;
    int noise_on;
    int perp;  // midpoint/SIB: rannum only when min(lambda) > 1e-12
    const int64_t *d_step;
    int64_t step_off;
    Vec3D e, eM, p, pM, b2, mpast;
};

template <int ALG>
__global__ void __launch_bounds__(256) llg_predict(StepArgs a) {
    const int N = a.h.natom, M = a.h.mensemble;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)N * M) return;
    const int k = (int)(t / N), i = (int)(t - (int64_t)k * N);
    const size_t o = (size_t)k * N + i;
    const int64_t step = *a.d_step + a.step_off;
    double B[3];
    site_field(a.h, a.eM, i, k, B);
    const double lam = a.lambda[i];
    const double mm = a.mmom[o];
    double e[3] = {a.e.x[o], a.e.y[o], a.e.z[o]};
    if (a.perp) perp_project(B, e);  // emom is m(t) before every solver's first half-step
    double z[3];
    if (ALG == 5) {
        noise3(a.nz, i, k, N, M, step, z);
        double Dp = (2.0 * lam * a.h.kbolt) / (a.delta_t * a.h.gama * a.h.mub);
        double sigma = sqrt(Dp * a.temprescale * a.temp[i] / mm);
        double bloc[3], bdup[3], mr[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) bloc[c] = B[c] + z[c] * sigma;
        damped_field(bloc, e, lam, bdup);
        rodrigues(bdup, e, a.delta_t, a.h.gama, 1.0 / (1.0 + lam * lam), mr);
        a.p.x[o] = mr[0];
        a.p.y[o] = mr[1];
        a.p.z[o] = mr[2];
        a.pM.x[o] = mr[0] * mm;
        a.pM.y[o] = mr[1] * mm;
        a.pM.z[o] = mr[2] * mm;
        a.b2.x[o] = bdup[0];
        a.b2.y[o] = bdup[1];
        a.b2.z[o] = bdup[2];
    } else if (ALG == 1 || ALG == 6 || ALG == 7) {
        double r[3] = {0.0, 0.0, 0.0};
        if (a.noise_on) {
            noise3(a.nz, i, k, N, M, step, z);
            double Dk = (((lam / (1.0 + lam * lam)) * a.h.kbolt) / a.h.gama / a.h.mub) * (a.h.gama / a.bn);
            double D = Dk * (1.0 / mm) * a.temp[i] * a.temprescale;
            double sigma = sqrt(2.00 * D);
            r[0] = z[0] * sigma;
            r[1] = z[1] * sigma;
            r[2] = z[2] * sigma;
        }
        double lldamp = 1.0 / (1.0 + lam * lam);
        double dt = a.delta_t * a.bn * a.h.gama * lldamp;
        double g = a.landeg[i];
        double dtg = dt * g, sqrtdtg = sqrt(dt) * g;
        double v[3];
        if (ALG == 1) {
            double A[3], et[3], detAi;
            midpoint_A(lam, dtg, sqrtdtg, e, B, r, A);
            cayley(A, e, et, detAi);
#pragma unroll
            for (int c = 0; c < 3; ++c) v[c] = 0.5 * (e[c] + et[c] * detAi);
        } else if (ALG == 6) {
            double a1[3], s1[3], efp[3];
            sib_a1s1(lam, e, B, r, a1, s1);
            sib_fixed_point(e, a1, s1, dtg, sqrtdtg, efp);
#pragma unroll
            for (int c = 0; c < 3; ++c) v[c] = 0.5 * (e[c] + efp[c]);
        } else {  // sispht: the normalised midpoint of e and the iterate it continues from
            double a1[3], s1[3], efp[3], f0[3];
            sib_a1s1(lam, e, B, r, a1, s1);
            sisph_fixed_point(e, a1, s1, dtg, sqrtdtg, efp, f0);
            const double unorm = sqrt((e[0] + f0[0]) * (e[0] + f0[0]) + (e[1] + f0[1]) * (e[1] + f0[1]) +
                                      (e[2] + f0[2]) * (e[2] + f0[2]));
#pragma unroll
            for (int c = 0; c < 3; ++c) v[c] = (e[c] + f0[c]) / unorm;
        }
        a.p.x[o] = v[0];
        a.p.y[o] = v[1];
        a.p.z[o] = v[2];
        a.pM.x[o] = v[0] * mm;
        a.pM.y[o] = v[1] * mm;
        a.pM.z[o] = v[2] * mm;
    } else if (ALG == 4) {
        noise3(a.nz, i, k, N, M, step, z);
        double dt = a.delta_t * a.h.gama;
        double Dk = lam / (1.0 + lam * lam) * a.h.kbolt / a.h.mub;
        double D = Dk * (1.0 / mm) * a.temp[i] * a.temprescale;
        double sigma = sqrt(dt * 2.0 * D);
        double g = a.landeg[i];
        double dtg = dt * g * (1.0 / (1.0 + lam * lam));
        double dwx = z[0] * sigma * g, dwy = z[1] * sigma * g, dwz = z[2] * sigma * g;
        double e1x = e[0], e1y = e[1], e1z = e[2];
        double hesx = B[0], hesy = B[1], hesz = B[2];
        double hlpx = lam * hesx, hlpy = lam * hesy, hlpz = lam * hesz;
        double prot = e1x * hlpx + e1y * hlpy + e1z * hlpz;
        double a1x = hlpx + e1z * (hesy + 0.0) - e1y * (hesz + 0.0) - e1x * prot;
        double a1y = hlpy - e1z * (hesx + 0.0) + e1x * (hesz + 0.0) - e1y * prot;
        double a1z = hlpz + e1y * (hesx + 0.0) - e1x * (hesy + 0.0) - e1z * prot;
        double b1xx = lam - e1x * e1x * lam, b1xy = e1z - e1x * e1y * lam, b1xz = -e1y - e1x * e1z * lam;
        double b1yx = -e1z - e1y * e1x * lam, b1yy = lam - e1y * e1y * lam, b1yz = e1x - e1y * e1z * lam;
        double b1zx = e1y - e1z * e1x * lam, b1zy = -e1x - e1z * e1y * lam, b1zz = lam - e1z * e1z * lam;
        double etx = e1x + a1x * dtg + b1xx * dwx + b1xy * dwy + b1xz * dwz;
        double ety = e1y + a1y * dtg + b1yx * dwx + b1yy * dwy + b1yz * dwz;
        double etz = e1z + a1z * dtg + b1zx * dwx + b1zy * dwy + b1zz * dwz;
        a.b2.x[o] = B[0];
        a.b2.y[o] = B[1];
        a.b2.z[o] = B[2];
        a.p.x[o] = etx;
        a.p.y[o] = ety;
        a.p.z[o] = etz;
        a.pM.x[o] = etx * mm;
        a.pM.y[o] = ety * mm;
        a.pM.z[o] = etz * mm;
    } else if (ALG == 11) {
        // llgi_evolve_first: thermfield (Depondt amplitude), bdup = beff + btherm
        noise3(a.nz, i, k, N, M, step, z);
        double Dp = (2.0 * lam * a.h.kbolt) / (a.delta_t * a.h.gama * a.h.mub);
        double sigma = sqrt(Dp * a.temprescale * a.temp[i] / mm);
        double bdup[3], et[3] = {a.mpast.x[o], a.mpast.y[o], a.mpast.z[o]}, mt[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) bdup[c] = B[c] + z[c] * sigma;
        llgi_heun(lam, a.delta_t, a.h.gama, a.relaxtime, et, e, bdup, mt);
        a.p.x[o] = mt[0];
        a.p.y[o] = mt[1];
        a.p.z[o] = mt[2];
        a.pM.x[o] = mt[0] * mm;
        a.pM.y[o] = mt[1] * mm;
        a.pM.z[o] = mt[2] * mm;
        a.b2.x[o] = bdup[0];
        a.b2.y[o] = bdup[1];
        a.b2.z[o] = bdup[2];
    }
}

template <int ALG>
__global__ void __launch_bounds__(256) llg_correct(StepArgs a) {
    const int N = a.h.natom, M = a.h.mensemble;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)N * M) return;
    const int k = (int)(t / N), i = (int)(t - (int64_t)k * N);
    const size_t o = (size_t)k * N + i;
    const int64_t step = *a.d_step + a.step_off;
    double B[3];
    site_field(a.h, a.pM, i, k, B);
    const double lam = a.lambda[i];
    const double mm = a.mmom[o];
    double e[3] = {a.e.x[o], a.e.y[o], a.e.z[o]};
    double pr[3] = {a.p.x[o], a.p.y[o], a.p.z[o]};
    // after the first half-step emom is m(t) for midpoint and SIB, the predictor for
    // Heun, Depondt and LLGI
    if (a.perp) perp_project(B, (ALG == 1 || ALG == 6 || ALG == 7) ? e : pr);
    double out[3];
    double z[3];
    if (ALG == 5) {
        noise3(a.nz, i, k, N, M, step, z);
        double Dp = (2.0 * lam * a.h.kbolt) / (a.delta_t * a.h.gama * a.h.mub);
        double sigma = sqrt(Dp * a.temprescale * a.temp[i] / mm);
        double bloc[3], bdup[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) bloc[c] = B[c] + z[c] * sigma;
        damped_field(bloc, pr, lam, bdup);
        bdup[0] = 0.50 * bdup[0] + 0.50 * a.b2.x[o];
        bdup[1] = 0.50 * bdup[1] + 0.50 * a.b2.y[o];
        bdup[2] = 0.50 * bdup[2] + 0.50 * a.b2.z[o];
        rodrigues(bdup, e, a.delta_t, a.h.gama, 1.0 / (1.0 + lam * lam), out);
    } else if (ALG == 1 || ALG == 6 || ALG == 7) {
        double r[3] = {0.0, 0.0, 0.0};
        if (a.noise_on) {
            noise3(a.nz, i, k, N, M, step, z);
            double Dk = (((lam / (1.0 + lam * lam)) * a.h.kbolt) / a.h.gama / a.h.mub) * (a.h.gama / a.bn);
            double D = Dk * (1.0 / mm) * a.temp[i] * a.temprescale;
            double sigma = sqrt(2.00 * D);
            r[0] = z[0] * sigma;
            r[1] = z[1] * sigma;
            r[2] = z[2] * sigma;
        }
        double lldamp = 1.0 / (1.0 + lam * lam);
        double dt = a.delta_t * a.bn * a.h.gama * lldamp;
        double g = a.landeg[i];
        double dtg = dt * g, sqrtdtg = sqrt(dt) * g;
        if (ALG == 1) {
            double A[3], et[3], detAi;
            midpoint_A(lam, dtg, sqrtdtg, pr, B, r, A);
            cayley(A, e, et, detAi);
#pragma unroll
            for (int c = 0; c < 3; ++c) out[c] = et[c] * detAi;
        } else if (ALG == 6) {
            double a1[3], s1[3];
            sib_a1s1(lam, pr, B, r, a1, s1);
            sib_fixed_point(e, a1, s1, dtg, sqrtdtg, out);
        } else {  // sisphf keeps the last iterate
            double a1[3], s1[3], f0[3];
            sib_a1s1(lam, pr, B, r, a1, s1);
            sisph_fixed_point(e, a1, s1, dtg, sqrtdtg, out, f0);
        }
    } else if (ALG == 11) {
        // llgi_evolve_second: the same btherm as the predictor (same counter), averaged
        // field, corrector from (m(t - dt), m(t)); m(t) becomes the new m(t - dt)
        noise3(a.nz, i, k, N, M, step, z);
        double Dp = (2.0 * lam * a.h.kbolt) / (a.delta_t * a.h.gama * a.h.mub);
        double sigma = sqrt(Dp * a.temprescale * a.temp[i] / mm);
        double b2v[3] = {a.b2.x[o], a.b2.y[o], a.b2.z[o]};
        double bdup[3], et[3] = {a.mpast.x[o], a.mpast.y[o], a.mpast.z[o]}, mt[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) bdup[c] = 0.5 * (B[c] + z[c] * sigma) + 0.5 * b2v[c];
        llgi_heun(lam, a.delta_t, a.h.gama, a.relaxtime, et, e, bdup, mt);
        a.mpast.x[o] = e[0];
        a.mpast.y[o] = e[1];
        a.mpast.z[o] = e[2];
        double etot = 1.0 / sqrt(mt[0] * mt[0] + mt[1] * mt[1] + mt[2] * mt[2]);
        out[0] = mt[0] * etot;
        out[1] = mt[1] * etot;
        out[2] = mt[2] * etot;
    } else {  // ALG == 4
        noise3(a.nz, i, k, N, M, step, z);
        double dt = a.delta_t * a.h.gama;
        double Dk = lam / (1.0 + lam * lam) * a.h.kbolt / a.h.mub;
        double D = Dk * (1.0 / mm) * a.temp[i] * a.temprescale;
        double sigma = sqrt(dt * 2.0 * D);
        double g = a.landeg[i];
        double dtg = dt * g * (1.0 / (1.0 + lam * lam));
        double dwx = z[0] * sigma * g, dwy = z[1] * sigma * g, dwz = z[2] * sigma * g;
        double e1x = pr[0], e1y = pr[1], e1z = pr[2];
        double e2x = e[0], e2y = e[1], e2z = e[2];
        double h1esx = B[0], h1esy = B[1], h1esz = B[2];
        double h1px = lam * h1esx, h1py = lam * h1esy, h1pz = lam * h1esz;
        double h2esx = a.b2.x[o], h2esy = a.b2.y[o], h2esz = a.b2.z[o];
        double h2px = lam * h2esx, h2py = lam * h2esy, h2pz = lam * h2esz;
        double prot = e1x * h1px + e1y * h1py + e1z * h1pz;
        double a1x = h1px + e1z * (h1esy + 0.0) - e1y * (h1esz + 0.0) - e1x * prot;
        double a1y = h1py - e1z * (h1esx + 0.0) + e1x * (h1esz + 0.0) - e1y * prot;
        double a1z = h1pz + e1y * (h1esx + 0.0) - e1x * (h1esy + 0.0) - e1z * prot;
        double b1xx = lam - e1x * e1x * lam, b1xy = e1z - e1x * e1y * lam, b1xz = -e1y - e1x * e1z * lam;
        double b1yx = -e1z - e1y * e1x * lam, b1yy = lam - e1y * e1y * lam, b1yz = e1x - e1y * e1z * lam;
        double b1zx = e1y - e1z * e1x * lam, b1zy = -e1x - e1z * e1y * lam, b1zz = lam - e1z * e1z - lam;
        prot = e2x * h2px + e2y * h2py + e2z * h2pz;
        double a2x = h2px + e2z * h2esy - e2y * h2esz - e2x * prot;
        double a2y = h2py - e2z * h2esx + e2x * h2esz - e2y * prot;
        double a2z = h2pz + e2y * h2esx - e2x * h2esy - e2z * prot;
        double b2xx = lam - e2x * e2x * lam, b2xy = e2z - e2x * e2y * lam, b2xz = -e2y - e2x * e2z * lam;
        double b2yx = -e2z - e2y * e2x * lam, b2yy = lam - e2y * e2y * lam, b2yz = e2x - e2y * e2z * lam;
        double b2zx = e2y - e2z * e2x * lam, b2zy = -e2x - e2z * e2y * lam, b2zz = lam - e2z * e2z * lam;
        double ax = a1x + a2x, ay = a1y + a2y, az = a1z + a2z;
        double bxx = b1xx + b2xx, bxy = b1xy + b2xy, bxz = b1xz + b2xz;
        double byx = b1yx + b2yx, byy = b1yy + b2yy, byz = b1yz + b2yz;
        double bzx = b1zx + b2zx, bzy = b1zy + b2zy, bzz = b1zz + b2zz;
        double etx = ax * dtg + bxx * dwx + bxy * dwy + bxz * dwz;
        double ety = ay * dtg + byx * dwx + byy * dwy + byz * dwz;
        double etz = az * dtg + bzx * dwx + bzy * dwy + bzz * dwz;
        double nx = e2x + 0.5 * etx, ny = e2y + 0.5 * ety, nz = e2z + 0.5 * etz;
        double etot = 1.0 / sqrt(nx * nx + ny * ny + nz * nz);
        out[0] = nx * etot;
        out[1] = ny * etot;
        out[2] = nz * etot;
    }
    // moment_update / copym: emom <- emom2, emomM <- emom2 * mmom
    a.e.x[o] = out[0];
    a.e.y[o] = out[1];
    a.e.z[o] = out[2];
    a.eM.x[o] = out[0] * mm;
    a.eM.y[o] = out[1] * mm;
    a.eM.z[o] = out[2] * mm;
}

// with dipoles on, the dipolar field of the moments each half step reads is enqueued
// before it (the predictor's from emomM, the corrector's from the predictor's mpM)
template <int ALG>
static int launch_pair(Sim &s, const StepArgs &a, int grid, int block, int phase) {
    int rc;
    if (phase & 1) {
        if (s.ham.do_dip && (rc = dipole_field(s, s.eM))) return rc;
        llg_predict<ALG><<<grid, block, 0, s.stream>>>(a);
    }
    if (phase & 2) {
        if (s.ham.do_dip && (rc = dipole_field(s, s.pM))) return rc;
        llg_correct<ALG><<<grid, block, 0, s.stream>>>(a);
    }
    return UPPASD_GPU_OK;
}

// Threads per block: 64 below 1024 (site, ensemble) pairs per SM, 256 above.  A thread's
// work is one site's whole field and update, a long dependent FP64 chain, so a small
// system is latency-bound: small blocks spread it over every SM and balance the SMs'
// shares (bcc 20^3: 0.072 -> 0.045 ms per Depondt step; square 256^2: 0.131 -> 0.117 ms
// per midpoint step, measured on the GB300).
static int fp64_block(const Sim &s, int64_t n) {
    static int sms = 0;
    if (!sms && cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s.device) != cudaSuccess) sms = 152;
    return n < (int64_t)sms * 1024 ? 64 : 256;
}

int llg_generic_step(Sim &s, int64_t step_offset, int phase) {
    StepArgs a;
    a.h = s.ham;
    a.nz.mode = s.llg.noise_mode;
    a.nz.seed = s.llg.seed;
    a.nz.inj = s.llg.inj;
    a.nz.inj_first = s.llg.inj_first;
    a.lambda = s.llg.lambda;
    a.temp = s.llg.temp;
    a.landeg = s.llg.landeg;
    a.mmom = s.llg.mmom;
    a.delta_t = s.llg.delta_t;
    a.bn = s.llg.bn;
    a.temprescale = s.llg.temprescale;
    a.relaxtime = s.llg.relaxtime;
    a.perp = s.llg.perp;
    a.noise_on = s.llg.noise_on;
    a.d_step = s.llg.d_step;
    a.step_off = step_offset;
    a.e = s.e;
    a.eM = s.eM;
    a.p = s.p;
    a.pM = s.pM;
    a.b2 = s.b2;
    a.mpast = s.mpast;
    const int64_t n = (int64_t)s.ham.natom * s.ham.mensemble;
    const int block = fp64_block(s, n);
    const int grid = (int)((n + block - 1) / block);
    int rc;
    switch (s.llg.sdealgh) {
    case 1: rc = launch_pair<1>(s, a, grid, block, phase); break;
    case 4: rc = launch_pair<4>(s, a, grid, block, phase); break;
    case 5: rc = launch_pair<5>(s, a, grid, block, phase); break;
    case 6: rc = launch_pair<6>(s, a, grid, block, phase); break;
    case 7: rc = launch_pair<7>(s, a, grid, block, phase); break;
    case 11: rc = launch_pair<11>(s, a, grid, block, phase); break;
    default: set_error("unsupported SDEalgh"); return UPPASD_GPU_EUNSUPPORTED;
    }
    if (rc) return rc;
    UPPASD_CUDA_TRY(cudaGetLastError());
    return UPPASD_GPU_OK;
}

}  // namespace uppasd
