// field_f32.cuh -- FP32 building blocks shared by the FP32-gather paths
// (precision 3 LLG and heat bath, the structured square heat bath):
//   field_f32      effective field of one site from an FP32 float4 mirror (unit
//                  vector, moment in w) and FP32 copies of the couplings, same terms
//                  and order as the FP64 field (Hamiltonian/hamiltonianactions.f90:187-243)
//   heat_bath_f32  flip_h (MonteCarlo/montecarlo_common.f90:371-422) in FP32, with
//                  the field frame built from the field's own components
//   delta_energy_f32  calculate_energy's E(trial) - E(current) of one site in FP32
//                  (MonteCarlo/montecarlo_common.f90:431-865), the same terms and the
//                  same mixed unit / full-moment DM current-energy term as the FP64 path
#pragma once
#include "common.cuh"
#include "sim.h"

namespace uppasd {

// What a site's field needs besides the spins: its coupling row, list sizes, anisotropy
// row and type, and where its neighbour indices come from (the class tables, with
// offsets from i, or the caller's per-site lists, slot-major, absolute).
struct SiteView {
    int ih, nn, nd, ta, ar, base;
    const int32_t *nb, *dl;
    size_t nbs, dls;
    __device__ __forceinline__ int nbr(int s) const { return base + __ldg(&nb[s * nbs]); }
    __device__ __forceinline__ int dmn(int s) const { return base + __ldg(&dl[s * dls]); }
};

__device__ __forceinline__ SiteView site_view(const HamDev &h, const MixedDev &c, int i) {
    SiteView v;
    if (c.ncls) {
        const int cl = __ldg(&c.cls[i]);
        const int4 ci = __ldg(&c.cinfo[cl]);
        v.nn = ci.x & 0xffff;
        v.nd = (int)((unsigned)ci.x >> 16);
        v.ih = ci.y;
        v.ar = ci.z;
        v.ta = ci.w;
        v.nb = c.cnb + (size_t)cl * h.mnn;
        v.dl = c.cdm + (size_t)cl * h.mnn_dm;
        v.nbs = v.dls = 1;
        v.base = i;
    } else {
        v.ih = __ldg(&c.row[i]);
        v.nn = h.nsize[i];
        v.nd = h.do_dm ? h.dmsize[i] : 0;
        v.ta = h.do_aniso ? h.taniso[i] : 0;
        v.ar = h.do_aniso ? __ldg(&c.arow[i]) : 0;
        v.nb = h.nlist + i;
        v.dl = h.dmlist + i;
        v.nbs = v.dls = (size_t)h.natom;
        v.base = 0;
    }
    return v;
}

// Chemically resolved exchange coupling of slot s for class ih and neighbour j, indexed
// by the neighbour's type (a float4 of the couplings to up to four types, selected by
// the type, was 1.5x slower on a 2 M-site alloy: four times the L1 bytes per neighbour).
__device__ __forceinline__ float chem_coupling(const MixedDev &c, int s, int ih, int j) {
    return __ldg(&c.nc[((size_t)s * c.nrow + ih) * c.nsp + __ldg(&c.spc[j])]);
}

// FP32 effective field of site i from full moments m.w * m.xyz, in the FP64 field's
// term order (exchange or tensor, DMI, anisotropy, Zeeman), with the couplings from
// the FP32 copies in MixedDev.
__device__ __forceinline__ void field_f32(const HamDev &h, const MixedDev &c, const float4 *m, int i, int k,
                                          float B[3]) {
    const int N = h.natom;
    const size_t off = (size_t)k * N;
    const SiteView sv = site_view(h, c, i);
    const int ih = sv.ih;
    const int nn = sv.nn;
    float bs[3] = {0.f, 0.f, 0.f}, bq[3] = {0.f, 0.f, 0.f};
    if (h.do_jtensor) {
        for (int s = 0; s < nn; ++s) {
            const int j = sv.nbr(s);
            const float4 v = m[off + j];
            const float m1 = v.w * v.x, m2 = v.w * v.y, m3 = v.w * v.z;
            const float *J = c.jt + ((size_t)s * c.nrow + ih) * 9;
#pragma unroll
            for (int a = 0; a < 3; ++a)
                bs[a] += __ldg(&J[3 * a]) * m1 + __ldg(&J[3 * a + 1]) * m2 + __ldg(&J[3 * a + 2]) * m3;
        }
    } else if (c.nsp) {
        for (int s = 0; s < nn; ++s) {
            const int j = sv.nbr(s);
            const float4 v = m[off + j];
            const float cj = chem_coupling(c, s, ih, j) * v.w;
            bs[0] = fmaf(cj, v.x, bs[0]);
            bs[1] = fmaf(cj, v.y, bs[1]);
            bs[2] = fmaf(cj, v.z, bs[2]);
        }
    } else {
        for (int s = 0; s < nn; ++s) {
            const int j = sv.nbr(s);
            const float4 v = m[off + j];
            const float cj = __ldg(&c.nc[(size_t)s * c.nrow + ih]) * v.w;
            bs[0] = fmaf(cj, v.x, bs[0]);
            bs[1] = fmaf(cj, v.y, bs[1]);
            bs[2] = fmaf(cj, v.z, bs[2]);
        }
    }
    if (h.do_dm) {
        const int nd = sv.nd;
        for (int s = 0; s < nd; ++s) {
            const int j = sv.dmn(s);
            const float4 d = __ldg(&c.dm[(size_t)s * c.nrow + ih]);
            const float4 v = m[off + j];
            const float m1 = v.w * v.x, m2 = v.w * v.y, m3 = v.w * v.z;
            bs[0] += d.z * m2 - d.y * m3;
            bs[1] += d.x * m3 - d.z * m1;
            bs[2] += d.y * m1 - d.x * m2;
        }
    }
    if (h.do_aniso) {
        const float4 me = m[off + i];
        const float m1 = me.w * me.x, m2 = me.w * me.y, m3 = me.w * me.z;
        const int ta = sv.ta;
        const int ar = sv.ar;
        const float4 an = __ldg(&c.an[ar]);
        const float2 an2 = __ldg(&c.an2[ar]);
        const float e0 = an.x, e1 = an.y, e2 = an.z, ka0 = an.w, ka1 = an2.x;
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
            const float sc = ta == 2 ? 1.0f : an2.y;
            float *dst = ta == 2 ? bs : bq;
            dst[0] += t0 * sc;
            dst[1] += t1 * sc;
            dst[2] += t2 * sc;
        }
    }
    const float4 ex = __ldg(&c.ext[c.ext_uniform ? 0 : off + i]);
    B[0] = bs[0] + (bq[0] + ex.x);
    B[1] = bs[1] + (bq[1] + ex.y);
    B[2] = bs[2] + (bq[2] + ex.z);
}

// E(trial) - E(current) of site i for the trial unit vector nm (before the factor mub),
// exchange (scalar or tensor) and DMI from the neighbours on the mirror m, anisotropy and
// Zeeman; the DM current energy keeps the reference's unit-moment components
// (montecarlo_common.f90:609-617).
__device__ __forceinline__ float delta_energy_f32(const HamDev &h, const MixedDev &c, const float4 *m, int i, int k,
                                                  const float nm[3]) {
    const int N = h.natom;
    const size_t off = (size_t)k * N;
    const SiteView sv = site_view(h, c, i);
    const int ih = sv.ih;
    const float4 me = m[off + i];
    const float mm = me.w;
    const float ei[3] = {me.x, me.y, me.z};
    const float mi[3] = {mm * me.x, mm * me.y, mm * me.z};
    const float tm[3] = {mm * nm[0], mm * nm[1], mm * nm[2]};
    const float dm[3] = {tm[0] - mi[0], tm[1] - mi[1], tm[2] - mi[2]};
    float b[3] = {0.f, 0.f, 0.f};
    const int nn = sv.nn;
    if (h.do_jtensor) {
        for (int s = 0; s < nn; ++s) {
            const int j = sv.nbr(s);
            const float4 v = m[off + j];
            const float m1 = v.w * v.x, m2 = v.w * v.y, m3 = v.w * v.z;
            const float *J = c.jt + ((size_t)s * c.nrow + ih) * 9;
#pragma unroll
            for (int a = 0; a < 3; ++a)
                b[a] += __ldg(&J[3 * a]) * m1 + __ldg(&J[3 * a + 1]) * m2 + __ldg(&J[3 * a + 2]) * m3;
        }
    } else if (c.nsp) {
        for (int s = 0; s < nn; ++s) {
            const int j = sv.nbr(s);
            const float4 v = m[off + j];
            const float cj = chem_coupling(c, s, ih, j) * v.w;
            b[0] = fmaf(cj, v.x, b[0]);
            b[1] = fmaf(cj, v.y, b[1]);
            b[2] = fmaf(cj, v.z, b[2]);
        }
    } else {
        for (int s = 0; s < nn; ++s) {
            const int j = sv.nbr(s);
            const float4 v = m[off + j];
            const float cj = __ldg(&c.nc[(size_t)s * c.nrow + ih]) * v.w;
            b[0] = fmaf(cj, v.x, b[0]);
            b[1] = fmaf(cj, v.y, b[1]);
            b[2] = fmaf(cj, v.z, b[2]);
        }
    }
    // bilinear exchange: E_t - E_c = -(t - m_i) . b
    float de = -(dm[0] * b[0] + dm[1] * b[1] + dm[2] * b[2]);
    if (h.do_dm) {
        const int nd = sv.nd;
        for (int s = 0; s < nd; ++s) {
            const int j = sv.dmn(s);
            const float4 d = __ldg(&c.dm[(size_t)s * c.nrow + ih]);
            const float4 v = m[off + j];
            const float mj0 = v.w * v.x, mj1 = v.w * v.y, mj2 = v.w * v.z;
            const float et = d.x * (tm[1] * mj2 - tm[2] * mj1) + d.y * (tm[2] * mj0 - tm[0] * mj2) +
                             d.z * (tm[0] * mj1 - tm[1] * mj0);
            const float ec = d.x * (mi[1] * mj2 - ei[2] * mj1) + d.y * (mi[2] * mj0 - mi[0] * mj2) +
                             d.z * (ei[0] * mj1 - mi[1] * mj0);
            de -= et - ec;
        }
    }
    if (h.do_aniso) {
        const int ta = sv.ta;
        const int ar = sv.ar;
        const float4 an = __ldg(&c.an[ar]);
        const float2 an2 = __ldg(&c.an2[ar]);
        const float ka0 = an.w, ka1 = an2.x;
        if (ta == 1 || ta == 7) {
            const float tta = mi[0] * an.x + mi[1] * an.y + mi[2] * an.z;
            const float ttb = tm[0] * an.x + tm[1] * an.y + tm[2] * an.z;
            const float a2 = tta * tta, b2 = ttb * ttb;
            de += ka0 * (b2 - a2) + ka1 * (b2 * b2 - a2 * a2);
        }
        if (ta == 2 || ta == 7) {
            // cubic: -K (x2 y2 + y2 z2 + z2 x2) - K2 x2 y2 z2 (ta 2), +sb times that (ta 7)
            const float sgn = ta == 2 ? -1.0f : an2.y;
            float x2 = mi[0] * mi[0], y2 = mi[1] * mi[1], z2 = mi[2] * mi[2];
            const float cc = ka0 * (x2 * y2 + y2 * z2 + z2 * x2) + ka1 * (x2 * y2 * z2);
            x2 = tm[0] * tm[0];
            y2 = tm[1] * tm[1];
            z2 = tm[2] * tm[2];
            const float ct = ka0 * (x2 * y2 + y2 * z2 + z2 * x2) + ka1 * (x2 * y2 * z2);
            de += sgn * (ct - cc);
        }
    }
    const float4 ex = __ldg(&c.ext[c.ext_uniform ? 0 : off + i]);
    de -= ex.x * dm[0] + ex.y * dm[1] + ex.z * dm[2];
    return de;
}

// flip_h in FP32: x = beta_mu |h|; 1 - cos(theta) = -ln((1 - e^-2x) q + e^-2x + tol) / x
// formed directly, and the frame from (zx, zy) so it stays orthonormal in FP32.
__device__ __forceinline__ float3 heat_bath_f32(float3 h, float beta_mu, float q, float fp) {
    const float zx = beta_mu * h.x, zy = beta_mu * h.y, zz = beta_mu * h.z;
    const float rxy = sqrtf(zx * zx + zy * zy);
    const float zarg = sqrtf(fmaf(rxy, rxy, zz * zz));
    const float izarg = 1.0f / zarg;
    const float zct = zz * izarg, zst = rxy * izarg;
    const float zcp = rxy > 0.0f ? zx / rxy : 1.0f, zsp = rxy > 0.0f ? zy / rxy : 0.0f;
    const float e2 = __expf(-2.0f * zarg);
    const float omc = fminf(2.0f, fmaxf(0.0f, -__logf(fmaf(1.0f - e2, q, e2) + 1e-14f) * izarg));
    const float ct = 1.0f - omc, st = sqrtf(omc * (2.0f - omc));
    float sp, cp;
    __sincosf(3.14159265358979f * (2.0f * fp - 1.0f), &sp, &cp);
    const float s0 = st * cp, s1 = st * sp;
    const float nx = zcp * zct * s0 - zsp * s1 + zcp * zst * ct;
    const float ny = zsp * zct * s0 + zcp * s1 + zsp * zst * ct;
    const float nz = -zst * s0 + zct * ct;
    const float il = rsqrtf(nx * nx + ny * ny + nz * nz);
    return make_float3(nx * il, ny * il, nz * il);
}

}  // namespace uppasd
