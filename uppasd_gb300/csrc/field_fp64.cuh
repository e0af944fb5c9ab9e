// field_fp64.cuh -- FP64 effective field of one site and the LLG noise source,
// shared by the FP64 kernels (LLG, observables, Monte Carlo).  Files that
// include it are compiled with --fmad=false so every product and sum rounds
// separately, in the order of the reference's Fortran expressions:
//   heisenberg_field      Hamiltonian/hamiltonianactions.f90:431-466
//   tensor_field          Hamiltonian/hamiltonianactions.f90:499-542 (do_jtensor)
//   dzyaloshinskii_moriya Hamiltonian/hamiltonianactions.f90:546-580
//   uniaxial / cubic      Hamiltonian/hamiltonianactions.f90:842-919
//   assembly              Hamiltonian/hamiltonianactions.f90:187-243
#pragma once
#include "common.cuh"
#include "sim.h"

namespace uppasd {

struct NoiseArgs {
    int mode;  // 0 Philox, 1 injected, 2 none
    uint64_t seed;
    const double *inj;
    int64_t inj_first;
};

__device__ __forceinline__ void noise3(const NoiseArgs &nz, int i, int k, int N, int M, int64_t step, double z[3]) {
    if (nz.mode == 0) {
        normal3_f64(nz.seed, i, k, step, kStreamLLG, z);
    } else if (nz.mode == 1) {
        const double *b = nz.inj + (size_t)(step - nz.inj_first) * 3 * (size_t)N * M;
        size_t o = 3 * ((size_t)i + (size_t)N * k);
        z[0] = b[o];
        z[1] = b[o + 1];
        z[2] = b[o + 2];
    } else {
        z[0] = z[1] = z[2] = 0.0;
    }
}

__device__ __forceinline__ void aniso_field(const HamDev &h, int i, double m1, double m2, double m3, double bs[3],
                                            double bq[3]) {
    int ta = h.taniso[i];
    double e0 = h.eax[i], e1 = h.eay[i], e2 = h.eaz[i];
    double ka0 = h.k1[i], ka1 = h.k2[i];
    if (ta == 1 || ta == 7) {
        double tt1 = m1 * e0 + m2 * e1 + m3 * e2;
        double tt2 = ka0 + 2.0 * ka1 * (1.0 - tt1 * tt1);
        double tt3 = 2.0 * tt1 * tt2;
        bs[0] = bs[0] - tt3 * e0;
        bs[1] = bs[1] - tt3 * e1;
        bs[2] = bs[2] - tt3 * e2;
    }
    if (ta == 2 || ta == 7) {
        double t0 = 2.0 * ka0 * m1 * (m2 * m2 + m3 * m3) + 2.0 * ka1 * m1 * (m2 * m2 * (m3 * m3));
        double t1 = 2.0 * ka0 * m2 * (m3 * m3 + m1 * m1) + 2.0 * ka1 * m2 * (m3 * m3 * (m1 * m1));
        double t2 = 2.0 * ka0 * m3 * (m1 * m1 + m2 * m2) + 2.0 * ka1 * m3 * (m1 * m1 * (m2 * m2));
        if (ta == 2) {
            bs[0] = bs[0] + t0;
            bs[1] = bs[1] + t1;
            bs[2] = bs[2] + t2;
        } else {
            double s = h.sb[i];
            bq[0] = bq[0] + t0 * s;
            bq[1] = bq[1] + t1 * s;
            bq[2] = bq[2] + t2 * s;
        }
    }
}

// Tensor exchange field of site i: b_a += J_a1 m1 + J_a2 m2 + J_a3 m3 per neighbour,
// summed left to right as the reference's array expression is.  The tensor is read
// per Hamiltonian index aham(i), as the Monte Carlo energy (montecarlo_common.f90:502-510)
// does; tensor_field indexes it by the atom, which is the same for a full Hamiltonian.
__device__ __forceinline__ void tensor_exchange(const HamDev &h, const Vec3D &m, int i, int ih, size_t off,
                                                double b[3]) {
    const int N = h.natom;
    const int nn = h.nsize[i];
    for (int s = 0; s < nn; ++s) {
        int j = __ldg(&h.nlist[(size_t)s * N + i]);
        const double *J = h.jt + ((size_t)s * h.nham + ih) * 9;
        double m1 = __ldg(&m.x[off + j]), m2 = __ldg(&m.y[off + j]), m3 = __ldg(&m.z[off + j]);
        b[0] = b[0] + __ldg(&J[0]) * m1 + __ldg(&J[1]) * m2 + __ldg(&J[2]) * m3;
        b[1] = b[1] + __ldg(&J[3]) * m1 + __ldg(&J[4]) * m2 + __ldg(&J[5]) * m3;
        b[2] = b[2] + __ldg(&J[6]) * m1 + __ldg(&J[7]) * m2 + __ldg(&J[8]) * m3;
    }
}

// Total effective field of site i in ensemble k from the full moments m.
__device__ __forceinline__ void site_field(const HamDev &h, const Vec3D &m, int i, int k, double B[3]) {
    const int N = h.natom;
    const size_t off = (size_t)k * N;
    double bs[3] = {0.0, 0.0, 0.0}, bq[3] = {0.0, 0.0, 0.0};
    const int ih = h.aham[i];
    const int nn = h.nsize[i];
    if (h.do_jtensor) {
        tensor_exchange(h, m, i, ih, off, bs);
    } else {
        for (int s = 0; s < nn; ++s) {
            int j = __ldg(&h.nlist[(size_t)s * N + i]);
            double c = __ldg(&h.ncoup[(size_t)s * h.nham + ih]);
            bs[0] = bs[0] + c * __ldg(&m.x[off + j]);
            bs[1] = bs[1] + c * __ldg(&m.y[off + j]);
            bs[2] = bs[2] + c * __ldg(&m.z[off + j]);
        }
    }
    if (h.do_dm) {
        const int nd = h.dmsize[i];
        for (int s = 0; s < nd; ++s) {
            int j = __ldg(&h.dmlist[(size_t)s * N + i]);
            size_t d = (size_t)s * h.nham + ih;
            double d0 = h.dmx[d], d1 = h.dmy[d], d2 = h.dmz[d];
            double m1 = m.x[off + j], m2 = m.y[off + j], m3 = m.z[off + j];
            bs[0] = bs[0] + d2 * m2 - d1 * m3;
            bs[1] = bs[1] + d0 * m3 - d2 * m1;
            bs[2] = bs[2] + d1 * m1 - d0 * m2;
        }
    }
    if (h.do_aniso) aniso_field(h, i, m.x[off + i], m.y[off + i], m.z[off + i], bs, bq);
    // beff = beff1 + beff2 with the dipolar field first in beff1 (hamiltonianactions.f90:173-181)
    double bd[3] = {0.0, 0.0, 0.0};
    if (h.do_dip) {
        bd[0] = h.dip.x[off + i];
        bd[1] = h.dip.y[off + i];
        bd[2] = h.dip.z[off + i];
    }
    B[0] = bd[0] + bs[0] + (bq[0] + h.ext.x[off + i] + 0.0);
    B[1] = bd[1] + bs[1] + (bq[1] + h.ext.y[off + i] + 0.0);
    B[2] = bd[2] + bs[2] + (bq[2] + h.ext.z[off + i] + 0.0);
}

}  // namespace uppasd
