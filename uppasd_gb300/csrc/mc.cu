// mc.cu -- checkerboard Metropolis / heat-bath sweeps in FP64 (the parity path).
//
// The reference sweeps sites one at a time in a random permutation
// (MonteCarlo/montecarlo.f90:227-268).  Here sites are grouped into colours of
// an independent set of the coupling graph (built and verified at set-up), so
// all sites of one colour update concurrently without the data race of the
// reference's OpenMP loop.  The single-spin kernels are those of the reference:
//   trial moves    choose_random_flip   MonteCarlo/montecarlo_common.f90:25-79
//   energy change  calculate_energy     MonteCarlo/montecarlo_common.f90:431-865
//   acceptance     flip_a               MonteCarlo/montecarlo_common.f90:139-200
//   heat bath      flip_h               MonteCarlo/montecarlo_common.f90:371-422
// With the dipolar field on (dipole.cu), Metropolis adds the field of the sweep's start
// to the external field of the energy change and the heat bath has it, refreshed before
// each colour, in the site field.
// Random numbers come from Philox keyed by (site, ensemble, sweep): one draw
// of four uniforms per update, and a second (Gaussian) draw for the Gaussian
// trial move.  Compiled with --fmad=false.
#include "common.cuh"
#include "field_fp64.cuh"
#include "sim.h"

namespace uppasd {

// Parameters/parameters.f90:12 dbl_tolerance = 1e-14 is a REAL(4) literal.
__device__ __constant__ double kDblTol = (double)1e-14f;

__device__ __forceinline__ void choose_random_flip(const double e[3], double delta, const double rn[3],
                                                   const double gn[3], double nm[3]) {
    int ftype = (int)floor(3.0 * rn[0]);
    if (ftype == 0) {
        double phi = rn[1] * 2.0 * kPi;
        double theta = acos(1.0 - 2.0 * rn[2]);
        nm[0] = sin(theta) * cos(phi);
        nm[1] = sin(theta) * sin(phi);
        nm[2] = cos(theta);
    } else if (ftype == 1) {
        double g0 = gn[0] * delta, g1 = gn[1] * delta, g2 = gn[2] * delta;
        double l = sqrt((e[0] + g0) * (e[0] + g0) + (e[1] + g1) * (e[1] + g1) + (e[2] + g2) * (e[2] + g2));
        nm[0] = (e[0] + g0) / l;
        nm[1] = (e[1] + g1) / l;
        nm[2] = (e[2] + g2) / l;
    } else {
        nm[0] = -e[0];
        nm[1] = -e[1];
        nm[2] = -e[2];
    }
}

// de = mub * (E_trial - E_current) for site i; the DM current-energy term mixes
// unit and full moments exactly like the reference (montecarlo_common.f90:609-617).
__device__ double delta_energy(const HamDev &h, const Vec3D &eM, const Vec3D &e, double mm, int i, int k,
                               const double nm[3], const double ext[3]) {
    const int N = h.natom;
    const size_t off = (size_t)k * N;
    double e_c = 0.0, e_t = 0.0;
    double tm[3] = {nm[0] * mm, nm[1] * mm, nm[2] * mm};
    double mi[3] = {eM.x[off + i], eM.y[off + i], eM.z[off + i]};
    double ei[3] = {e.x[off + i], e.y[off + i], e.z[off + i]};
    const int ih = h.aham[i];
    if (h.do_jtensor) {
        // montecarlo_common.f90:502-510: the tensor field of the neighbours, then the dot products
        double bt[3] = {0.0, 0.0, 0.0};
        tensor_exchange(h, eM, i, ih, off, bt);
        e_c = e_c - (mi[0] * bt[0] + mi[1] * bt[1] + mi[2] * bt[2]);
        e_t = e_t - (tm[0] * bt[0] + tm[1] * bt[1] + tm[2] * bt[2]);
    } else {
        for (int s = 0; s < h.nsize[i]; ++s) {
            int j = h.nlist[(size_t)s * N + i];
            double c = h.ncoup[(size_t)s * h.nham + ih];
            double mj0 = eM.x[off + j], mj1 = eM.y[off + j], mj2 = eM.z[off + j];
            e_c = e_c - c * (mi[0] * mj0 + mi[1] * mj1 + mi[2] * mj2);
            e_t = e_t - c * (tm[0] * mj0 + tm[1] * mj1 + tm[2] * mj2);
        }
    }
    if (h.do_aniso) {
        int ta = h.taniso[i];
        double ea[3] = {h.eax[i], h.eay[i], h.eaz[i]};
        double ka0 = h.k1[i], ka1 = h.k2[i];
        if (ta == 1) {
            double tta = mi[0] * ea[0] + mi[1] * ea[1] + mi[2] * ea[2];
            double ttb = tm[0] * ea[0] + tm[1] * ea[1] + tm[2] * ea[2];
            e_c = e_c + ka0 * (tta * tta) + ka1 * (tta * tta * (tta * tta));
            e_t = e_t + ka0 * (ttb * ttb) + ka1 * (ttb * ttb * (ttb * ttb));
        } else if (ta == 2) {
            double x2 = mi[0] * mi[0], y2 = mi[1] * mi[1], z2 = mi[2] * mi[2];
            e_c = e_c - ka0 * (x2 * y2 + y2 * z2 + z2 * x2) - ka1 * (x2 * y2 * z2);
            x2 = tm[0] * tm[0];
            y2 = tm[1] * tm[1];
            z2 = tm[2] * tm[2];
            e_t = e_t - ka0 * (x2 * y2 + y2 * z2 + z2 * x2) - ka1 * (x2 * y2 * z2);
        }
        if (ta == 7) {
            double tta = mi[0] * ea[0] + mi[1] * ea[1] + mi[2] * ea[2];
            double ttb = tm[0] * ea[0] + tm[1] * ea[1] + tm[2] * ea[2];
            e_c = e_c + ka0 * (tta * tta) + ka1 * (tta * tta * (tta * tta));
            e_t = e_t + ka0 * (ttb * ttb) + ka1 * (ttb * ttb * (ttb * ttb));
            double aw1 = ka0 * h.sb[i], aw2 = ka1 * h.sb[i];
            double x2 = mi[0] * mi[0], y2 = mi[1] * mi[1], z2 = mi[2] * mi[2];
            e_c = e_c + aw1 * (x2 * y2 + y2 * z2 + z2 * x2) + aw2 * (x2 * y2 * z2);
            x2 = tm[0] * tm[0];
            y2 = tm[1] * tm[1];
            z2 = tm[2] * tm[2];
            e_t = e_t + aw1 * (x2 * y2 + y2 * z2 + z2 * x2) + aw2 * (x2 * y2 * z2);
        }
    }
    if (h.do_dm) {
        for (int s = 0; s < h.dmsize[i]; ++s) {
            int j = h.dmlist[(size_t)s * N + i];
            size_t d = (size_t)s * h.nham + ih;
            double d0 = h.dmx[d], d1 = h.dmy[d], d2 = h.dmz[d];
            double mj0 = eM.x[off + j], mj1 = eM.y[off + j], mj2 = eM.z[off + j];
            e_c = e_c - d0 * (mi[1] * mj2 - ei[2] * mj1) - d1 * (mi[2] * mj0 - mi[0] * mj2) -
                  d2 * (ei[0] * mj1 - mi[1] * mj0);
            e_t = e_t - d0 * (tm[1] * mj2 - tm[2] * mj1) - d1 * (tm[2] * mj0 - tm[0] * mj2) -
                  d2 * (tm[0] * mj1 - tm[1] * mj0);
        }
    }
    e_c = e_c - ext[0] * mi[0] - ext[1] * mi[1] - ext[2] * mi[2];
    e_t = e_t - ext[0] * tm[0] - ext[1] * tm[1] - ext[2] * tm[2];
    return h.mub * (e_t - e_c);
}

__device__ __forceinline__ void heat_bath(const HamDev &h, double mm, double temperature, double flipprob,
                                          const double tf[3], double q, double out[3]) {
    double beta = 1.0 / h.kbolt / (1.0 * temperature);
    double zfc[3] = {beta * tf[0] * h.mub * mm, beta * tf[1] * h.mub * mm, beta * tf[2] * h.mub * mm};
    double zarg = sqrt(zfc[0] * zfc[0] + zfc[1] * zfc[1] + zfc[2] * zfc[2]);
    double zctheta = zfc[2] / zarg;
    double zstheta = sqrt(1.0 - zctheta * zctheta) + kDblTol;
    double zcphi = zfc[0] / (zarg * zstheta);
    double zsphi = zfc[1] / (zarg * zstheta);
    double ctheta = 1.0 + (1.0 / zarg) * log((1.0 - exp(-2.0 * zarg)) * q + exp(-2.0 * zarg) + kDblTol);
    double stheta = sqrt(1.0 - ctheta * ctheta);
    double phi = kPi * (2.0 * flipprob - 1.0);
    double st0 = stheta * cos(phi), st1 = stheta * sin(phi), st2 = ctheta;
    out[0] = zcphi * zctheta * st0 - zsphi * st1 + zcphi * zstheta * st2;
    out[1] = zsphi * zctheta * st0 + zcphi * st1 + zsphi * zstheta * st2;
    out[2] = -zstheta * st0 + zctheta * st2;
}

__global__ void __launch_bounds__(256) mc_colour_kernel(HamDev h, Vec3D e, Vec3D eM, const double *mmom,
                                                        const int32_t *sites, int nsites, int heatbath,
                                                        double temperature, double delta, const double *tk,
                                                        uint64_t seed, int64_t sweep) {
    const int N = h.natom;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nsites * h.mensemble) return;
    const int k = (int)(t / nsites);
    const int i = sites[t - (int64_t)k * nsites];
    if (tk) {  // one temperature per ensemble (replicas of pt_iphase)
        temperature = tk[k];
        if (!heatbath) delta = (double)(2.0f / 25.0f) * pow(h.kbolt * temperature / h.mub, 0.20);
    }
    const size_t o = (size_t)k * N + i;
    Philox4 w = philox_draw(seed, i, k, sweep, kStreamMC);
    double u[4] = {u01_open(w.x), u01_open(w.y), u01_open(w.z), u01_open(w.w)};
    const double mm = mmom[o];
    double nm[3];
    if (heatbath) {
        double tf[3];
        site_field(h, eM, i, k, tf);
        heat_bath(h, mm, temperature, u[1], tf, u[0], nm);
    } else {
        double ecur[3] = {e.x[o], e.y[o], e.z[o]};
        double rn[3] = {u[0], u[1], u[2]};
        double gn[3] = {0.0, 0.0, 0.0};
        if ((int)floor(3.0 * rn[0]) == 1) normal3_f64(seed, i, k, sweep, kStreamMCGauss, gn);
        choose_random_flip(ecur, delta, rn, gn, nm);
        // loc_mag_fld = extfield + beff + loc_demag_fld (montecarlo.f90:231): beff is the
        // dipolar field of the sweep's start when dipoles are on, zero otherwise
        double bd[3] = {0.0, 0.0, 0.0};
        if (h.do_dip) {
            bd[0] = h.dip.x[o];
            bd[1] = h.dip.y[o];
            bd[2] = h.dip.z[o];
        }
        double ext[3] = {(h.ext.x[o] + bd[0]) + 0.0, (h.ext.y[o] + bd[1]) + 0.0, (h.ext.z[o] + bd[2]) + 0.0};
        double de = delta_energy(h, eM, e, mm, i, k, nm, ext);
        double beta = 1.0 / h.kbolt / (1.0 * temperature + 1.0e-15);
        if (!(de <= 0.0 || u[3] < exp(-beta * de))) return;
    }
    e.x[o] = nm[0];
    e.y[o] = nm[1];
    e.z[o] = nm[2];
    eM.x[o] = mm * nm[0];
    eM.y[o] = mm * nm[1];
    eM.z[o] = mm * nm[2];
}

int mc_checkerboard_sweeps(Sim &s, char mode, double temperature, int64_t nsweeps, const double *tk) {
    square_mirror_stale(s);
    if (s.ncolour <= 0) {
        set_error("no colouring available for Monte Carlo");
        return UPPASD_GPU_ESTATE;
    }
    // montecarlo.f90:142, (2.0/25.0) is a REAL(4) constant
    const double delta = (double)(2.0f / 25.0f) * pow(s.ham.kbolt * temperature / s.ham.mub, 0.20);
    const int hb = mode == 'H' ? 1 : 0;
    int rc;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s.device);
    for (int64_t sw = 0; sw < nsweeps; ++sw) {
        // dipoles: Metropolis takes the field of the sweep's start as an extra external
        // field (montecarlo.f90:216-231); the heat bath has it in the site field
        // (effective_field_hb), evaluated before each colour: within a colour only the
        // colour's own sites change, and the long-range field of those changes is the
        // one term the colouring cannot keep exact
        if (s.ham.do_dip && !hb && (rc = dipole_field(s, s.eM))) return rc;
        for (int c = 0; c < s.ncolour; ++c) {
            int beg = s.colour_start_h[c], end = s.colour_start_h[c + 1];
            int n = end - beg;
            if (n == 0) continue;
            if (s.ham.do_dip && hb && (rc = dipole_field(s, s.eM))) return rc;
            int64_t tot = (int64_t)n * s.ham.mensemble;
            // small colours in 64-thread blocks, spread over more SMs (one site's energy
            // change and draw is a long dependent FP64 chain), as the FP64 LLG steps do
            const int block = tot < (int64_t)sms * 1024 ? 64 : 256;
            mc_colour_kernel<<<(unsigned)((tot + block - 1) / block), block, 0, s.stream>>>(
                s.ham, s.e, s.eM, s.llg.mmom, s.colour_sites + beg, n, hb, temperature, delta, tk, s.llg.seed,
                s.mc_sweep);
        }
        s.mc_sweep += 1;
    }
    UPPASD_CUDA_TRY(cudaGetLastError());
    return UPPASD_GPU_OK;
}

}  // namespace uppasd
