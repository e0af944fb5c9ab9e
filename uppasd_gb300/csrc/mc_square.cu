// mc_square.cu -- structured heat bath for uniform square-lattice Hamiltonians
// (exchange and interfacial DMI on the four nearest neighbours, uniform moment
// and Zeeman field), all ensembles of a simulation in one launch per colour.
//
// The reference's general path (mc.cu) gathers through the neighbour list in
// FP64; here the neighbours are x +- 1, y +- 1 of site i = x + L y, the
// couplings are per-direction constants recognised once from the caller's
// nlist/ncoup/dmlist/dm_vect, and the heat-bath draw (flip_h,
// MonteCarlo/montecarlo_common.f90:371-422) runs in FP32 on the FP64 spin state.
// Neighbours are read from an FP32 mirror of the state (the values the draw uses
// anyway), and every new spin is written to the mirror, from which e / eM are made
// once after the call's sweeps: four 16-byte loads per site instead of twelve 8-byte
// loads and conversions from e, and one 16-byte store per update.
// The chain is the checkerboard chain of mc.cu (colours x + y even, then odd)
// with the same Philox counters (site, ensemble, sweep), so it agrees with the
// FP64 path to FP32 rounding.
#include <cmath>
#include <string>
#include <vector>

#include "common.cuh"
#include "field_f32.cuh"
#include "sim.h"

namespace uppasd {
namespace {

struct SqArgs {
    int L, N, mensemble, colour;
    float c[4], d[4][3], ext[3], beta_mu, mom;
    uint64_t seed;
    long long sweep;
};

// betak: muB / (kB T) per ensemble (one temperature per ensemble), or null (a.beta_mu).
// The draw goes to the FP32 mirror only; e / eM, which hold exactly the draw (and the
// uniform moment times it), are made from the mirror once after the sweeps
// (sq_master_from_mirror) instead of on every update of every other site.
__global__ void __launch_bounds__(256) sq_heat_bath(SqArgs a, float4 *m, const float *betak) {
    const int half = a.L >> 1;
    const long long per = (long long)a.L * half;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= per * a.mensemble) return;
    const int k = (int)(t / per);
    const int idx = (int)(t - (long long)k * per);
    const int y = idx / half;
    const int x = 2 * (idx - y * half) + ((y + a.colour) & 1);
    const int L = a.L;
    const int xp = x + 1 == L ? 0 : x + 1, xm = x == 0 ? L - 1 : x - 1;
    const int yp = y + 1 == L ? 0 : y + 1, ym = y == 0 ? L - 1 : y - 1;
    const size_t off = (size_t)k * a.N;
    const int nb[4] = {xp + L * y, xm + L * y, x + L * yp, x + L * ym};
    float hx = a.ext[0], hy = a.ext[1], hz = a.ext[2];
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        const float4 v = m[off + nb[d]];
        const float ex = v.x, ey = v.y, ez = v.z;
        // exchange c e_j plus DMI e_j x d
        hx += a.c[d] * ex + (ey * a.d[d][2] - ez * a.d[d][1]);
        hy += a.c[d] * ey + (ez * a.d[d][0] - ex * a.d[d][2]);
        hz += a.c[d] * ez + (ex * a.d[d][1] - ey * a.d[d][0]);
    }
    const int i = x + L * y;
    const Philox4 w = philox_draw(a.seed, i, k, a.sweep, kStreamMC);
    const float k32 = 2.3283064365386963e-10f;
    const float q = fmaf((float)w.x, k32, 0.5f * k32), fp = fmaf((float)w.y, k32, 0.5f * k32);
    const float3 n = heat_bath_f32(make_float3(hx, hy, hz), betak ? betak[k] * a.mom : a.beta_mu, q, fp);
    m[off + i] = make_float4(n.x, n.y, n.z, 0.f);
}

__global__ void sq_master_from_mirror(const float4 *m, Vec3D e, Vec3D eM, float mom, long long n) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    const float4 v = m[o];
    e.x[o] = v.x;
    e.y[o] = v.y;
    e.z[o] = v.z;
    eM.x[o] = (double)mom * v.x;
    eM.y[o] = (double)mom * v.y;
    eM.z[o] = (double)mom * v.z;
}

__global__ void to_mirror(Vec3D e, float4 *m, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) m[t] = make_float4((float)e.x[t], (float)e.y[t], (float)e.z[t], 0.f);
}

template <typename T>
int to_host(std::vector<T> &h, const T *d, size_t n) {
    h.resize(n);
    return cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost) == cudaSuccess ? 0 : 1;
}

}  // namespace

// Recognise a uniform square-lattice Hamiltonian of edge L; fills s.sq or returns an error.
int square_recognise(Sim &s, int L) {
    const HamDev &h = s.ham;
    const int N = h.natom;
    auto fail = [&](const std::string &why) {
        set_error("structured heat bath: " + why);
        return UPPASD_GPU_EUNSUPPORTED;
    };
    if (L < 2 || (L & 1) || N != L * L) return fail("natom must equal L^2 with L even");
    if (h.do_jtensor) return fail("the exchange is a tensor; the structured path covers scalar exchange");
    std::vector<int32_t> nlist, nsize, aham, dml, dms, ta;
    std::vector<double> nc, dx, dy, dz, mm, ex, ey, ez, k1, k2;
    int bad = to_host(nlist, h.nlist, (size_t)h.mnn * N) | to_host(nsize, h.nsize, N) | to_host(aham, h.aham, N) |
              to_host(nc, h.ncoup, (size_t)h.mnn * h.nham) | to_host(mm, s.llg.mmom, (size_t)N * h.mensemble) |
              to_host(ex, h.ext.x, (size_t)N * h.mensemble) | to_host(ey, h.ext.y, (size_t)N * h.mensemble) |
              to_host(ez, h.ext.z, (size_t)N * h.mensemble);
    if (h.do_dm)
        bad |= to_host(dml, h.dmlist, (size_t)h.mnn_dm * N) | to_host(dms, h.dmsize, N) |
               to_host(dx, h.dmx, (size_t)h.mnn_dm * h.nham) | to_host(dy, h.dmy, (size_t)h.mnn_dm * h.nham) |
               to_host(dz, h.dmz, (size_t)h.mnn_dm * h.nham);
    if (h.do_aniso) bad |= to_host(k1, h.k1, N) | to_host(k2, h.k2, N) | to_host(ta, h.taniso, N);
    if (bad) {
        set_error("structured heat bath: device copy failed");
        return UPPASD_GPU_ECUDA;
    }
    auto dir_of = [&](int i, int j) {
        const int x = i % L, y = i / L, jx = j % L, jy = j / L;
        const int dx_ = (jx - x + L) % L, dy_ = (jy - y + L) % L;
        if (dx_ == 1 && dy_ == 0) return 0;
        if (dx_ == L - 1 && dy_ == 0) return 1;
        if (dx_ == 0 && dy_ == 1) return 2;
        if (dx_ == 0 && dy_ == L - 1) return 3;
        return -1;
    };
    double cdir[4];
    double ddir[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    bool seen[4] = {false, false, false, false}, dseen[4] = {false, false, false, false};
    for (int i = 0; i < N; ++i) {
        if (nsize[i] != 4) return fail("every site needs exactly 4 exchange neighbours");
        for (int q = 0; q < 4; ++q) {
            const int d = dir_of(i, nlist[(size_t)q * N + i]);
            if (d < 0) return fail("neighbours must be x +- 1, y +- 1 (periodic)");
            const double c = nc[(size_t)q * h.nham + aham[i]];
            if (!seen[d]) {
                cdir[d] = c;
                seen[d] = true;
            } else if (c != cdir[d]) {
                return fail("exchange must be uniform per direction");
            }
        }
        if (h.do_dm) {
            if (dms[i] != 4 && dms[i] != 0) return fail("DMI must act on the 4 nearest neighbours");
            for (int q = 0; q < dms[i]; ++q) {
                const int d = dir_of(i, dml[(size_t)q * N + i]);
                if (d < 0) return fail("DMI neighbours must be x +- 1, y +- 1");
                const size_t o = (size_t)q * h.nham + aham[i];
                const double v[3] = {dx[o], dy[o], dz[o]};
                if (!dseen[d]) {
                    for (int c = 0; c < 3; ++c) ddir[d][c] = v[c];
                    dseen[d] = true;
                } else if (v[0] != ddir[d][0] || v[1] != ddir[d][1] || v[2] != ddir[d][2]) {
                    return fail("DMI vectors must be uniform per direction");
                }
            }
        }
        if (h.do_aniso && ta[i] != 0 && (k1[i] != 0.0 || k2[i] != 0.0))
            return fail("anisotropy is not supported (the heat bath of a quadratic term is not exact)");
    }
    for (size_t q = 1; q < mm.size(); ++q)
        if (mm[q] != mm[0]) return fail("moments must be uniform");
    for (size_t q = 1; q < ex.size(); ++q)
        if (ex[q] != ex[0] || ey[q] != ey[0] || ez[q] != ez[0]) return fail("the Zeeman field must be uniform");
    SquareMC &sq = s.sq;
    sq.mom = (float)mm[0];
    for (int d = 0; d < 4; ++d) {
        sq.c[d] = (float)(cdir[d] * mm[0]);
        for (int c = 0; c < 3; ++c) sq.d[d][c] = (float)(ddir[d][c] * mm[0]);
    }
    sq.ext[0] = (float)ex[0];
    sq.ext[1] = (float)ey[0];
    sq.ext[2] = (float)ez[0];
    sq.L = L;
    return UPPASD_GPU_OK;
}

int square_mirror_ready(Sim &s) {
    if (s.sqm_valid) return UPPASD_GPU_OK;
    const long long n = (long long)s.ham.natom * s.ham.mensemble;
    if (!s.sqm) {
        UPPASD_CUDA_TRY(cudaMalloc(&s.sqm, (size_t)n * sizeof(float4)));
        s.bytes_allocated += (size_t)n * sizeof(float4);
    }
    to_mirror<<<(unsigned)((n + 255) / 256), 256, 0, s.stream>>>(s.e, s.sqm, n);
    UPPASD_CUDA_TRY(cudaGetLastError());
    s.sqm_valid = 1;
    return UPPASD_GPU_OK;
}

}  // namespace uppasd

namespace uppasd {

// Structured heat-bath sweeps; betak (muB / (kB T) per ensemble, on the device) or
// null for the single `temperature`.
int square_sweeps(Sim &s, int L, double temperature, const float *betak, int64_t nsweeps) {
    if (s.ham.do_dip) {
        set_error("mc_run_square: the dipolar field is not taken; set_dipole(0) first, or use mc_run");
        return UPPASD_GPU_EUNSUPPORTED;
    }
    if (structured(s)) {
        set_error("mc_run_square: needs the FP64 state (precision 0, 3 or 4)");
        return UPPASD_GPU_EUNSUPPORTED;
    }
    if (const int rc = sync_state(s)) return rc;  // precision 4: e from its master first
    s.mix.valid = 0;  // the precision-3 / 4 LLG mirror does not follow these updates
    if (s.sq.L != L) {
        const int rc = square_recognise(s, L);
        if (rc) return rc;
    }
    if (const int rc = square_mirror_ready(s)) return rc;
    SqArgs a{};
    a.L = L;
    a.N = s.ham.natom;
    a.mensemble = s.ham.mensemble;
    for (int d = 0; d < 4; ++d) {
        a.c[d] = s.sq.c[d];
        for (int c = 0; c < 3; ++c) a.d[d][c] = s.sq.d[d][c];
    }
    for (int c = 0; c < 3; ++c) a.ext[c] = s.sq.ext[c];
    a.mom = s.sq.mom;
    a.beta_mu = betak ? 0.f : (float)(s.ham.mub * s.sq.mom / (s.ham.kbolt * temperature));
    a.seed = s.llg.seed;
    const long long per = (long long)L * (L / 2) * a.mensemble;
    const unsigned blocks = (unsigned)((per + 255) / 256);
    for (int64_t sw = 0; sw < nsweeps; ++sw) {
        a.sweep = s.mc_sweep;
        for (int c = 0; c < 2; ++c) {
            a.colour = c;
            sq_heat_bath<<<blocks, 256, 0, s.stream>>>(a, s.sqm, betak);
        }
        s.mc_sweep += 1;
    }
    if (nsweeps > 0) {
        const long long nm = (long long)s.ham.natom * s.ham.mensemble;
        sq_master_from_mirror<<<(unsigned)((nm + 255) / 256), 256, 0, s.stream>>>(s.sqm, s.e, s.eM, a.mom, nm);
    }
    UPPASD_CUDA_TRY(cudaGetLastError());
    return UPPASD_GPU_OK;
}

}  // namespace uppasd

extern "C" int uppasd_gpu_mc_run_square(uppasd_gpu_sim *w, int32_t L, double temperature, int64_t nsweeps) {
    using namespace uppasd;
    if (!w || nsweeps < 0 || !(temperature > 0.0) || L < 2) {
        set_error("mc_run_square: temperature > 0, nsweeps >= 0, L >= 2");
        return UPPASD_GPU_EINVAL;
    }
    return square_sweeps(w->s, L, temperature, nullptr, nsweeps);
}

extern "C" int uppasd_gpu_mc_run_square_temps(uppasd_gpu_sim *w, int32_t L, const double *temps, int64_t nsweeps) {
    using namespace uppasd;
    if (!w || !temps || nsweeps < 0 || L < 2) {
        set_error("mc_run_square_temps: temperatures, nsweeps >= 0, L >= 2");
        return UPPASD_GPU_EINVAL;
    }
    const int rc = set_ensemble_temps(w->s, temps);
    if (rc) return rc;
    return square_sweeps(w->s, L, 0.0, w->s.betak, nsweeps);
}
