// llg_stencil.cu -- structured-lattice mixed-precision LLG (precision 1 and 2).
//
// Scope: periodic bcc lattices (2-atom conventional cell) with up to four
// exchange shells and up to two chemical species, uniform damping and
// temperature, Depondt solver (Evolution/depondt.f90:50-333), exchange plus a
// uniform Zeeman field.  init verifies that the caller's nlist/ncoup are
// exactly this structure (every neighbour and every FP64 coupling) and refuses
// otherwise, so the generic FP64 path stays the fallback.
//
// What changes against the FP64 path:
//  * neighbour indices are not stored: each sublattice is kept in a
//    ghost-padded array, so a neighbour is the site's own address plus a
//    block-uniform offset (no wrap logic, no per-neighbour index loads);
//  * couplings come from a (shell, species_i, species_j) table: with the
//    neighbour's species s_j in {0,1} carried in the float4's w, the coupling
//    is c_A + s_j (c_B - c_A), one FMA;
//  * the field gather, thermal field, damping term and Rodrigues rotation run in
//    FP32 on a float4 mirror (unit spin xyz + species in w);
//  * the spin state itself is kept in higher precision and renormalised every
//    step: FP64 (precision 1) or double-single hi+lo float pairs (precision 2,
//    hi = the FP32 mirror itself, lo = a residual array).  GB300's FP64 pipe
//    runs at ~1/70 of FP32, which is why the double-single master exists.
//
// HBM layout.  Mirrors (float4): per (ensemble k, basis b) a padded box of
// P3 x P2 x P1 cells, interior cell (x,y,z) at ((z+2)*P2 + (y+2))*P1 + (x+XOFF);
// the 2-cell ghost shell holds periodic copies written by the producing kernel.
// Other per-site arrays (b2eff, residual / FP64 master) are unpadded:
// ((k*2 + b)*L3 + z)*L2*L1 + y*L1 + x.
// Threads: block (TXB, TYB) covers TXB consecutive x of TYB rows at one z, one
// basis and one ensemble per block.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <utility>
#include <vector>

#include "common.cuh"
#include "sim.h"
#include "tc_gemm.cuh"
#include "tc_host.h"

namespace uppasd {

namespace {

constexpr int XOFF = 8;  // left x padding: keeps interior rows 128-byte aligned

// bcc neighbour stencil: (dx, dy, dz, target basis, shell) in cell units, for
// basis 0 (corner) and basis 1 (body centre); shells 1..4 = 8, 6, 12, 24 sites.
struct St {
    int8_t dx, dy, dz, bj, sh;
};

__host__ __device__ constexpr St stencil_entry(int b, int s) {
    // shell 1 : s in [0,8)   other basis, offsets {-1,0}^3 (b=0) or {0,1}^3 (b=1)
    // shell 2 : s in [8,14)  same basis, +-unit axis
    // shell 3 : s in [14,26) same basis, (+-1,+-1,0) permutations
    // shell 4 : s in [26,50) other basis, one axis {-2,+1} (b=0) / {-1,+2} (b=1), others as shell 1
    if (s < 8) {
        int o0 = b == 0 ? -1 : 0;
        return St{(int8_t)(o0 + ((s >> 0) & 1)), (int8_t)(o0 + ((s >> 1) & 1)), (int8_t)(o0 + ((s >> 2) & 1)),
                  (int8_t)(1 - b), 1};
    }
    if (s < 14) {
        int q = s - 8, ax = q >> 1, sg = (q & 1) ? -1 : 1;
        return St{(int8_t)(ax == 0 ? sg : 0), (int8_t)(ax == 1 ? sg : 0), (int8_t)(ax == 2 ? sg : 0), (int8_t)b, 2};
    }
    if (s < 26) {
        int q = s - 14, pr = q >> 2, sa = (q & 1) ? -1 : 1, sb = (q & 2) ? -1 : 1;
        int a0 = pr == 2 ? 1 : 0, a1 = pr == 0 ? 1 : 2;
        int d[3] = {0, 0, 0};
        d[a0] = sa;
        d[a1] = sb;
        return St{(int8_t)d[0], (int8_t)d[1], (int8_t)d[2], (int8_t)b, 3};
    }
    int q = s - 26, ax = q >> 3, far = (q >> 2) & 1, p1 = q & 1, p2 = (q >> 1) & 1;
    int o0 = b == 0 ? -1 : 0;
    int fa = b == 0 ? (far ? -2 : 1) : (far ? -1 : 2);
    int d[3] = {0, 0, 0};
    d[ax] = fa;
    int oa = ax == 0 ? 1 : 0, ob = ax == 2 ? 1 : 2;
    d[oa] = o0 + p1;
    d[ob] = o0 + p2;
    return St{(int8_t)d[0], (int8_t)d[1], (int8_t)d[2], (int8_t)(1 - b), 4};
}

constexpr int nb_of_shells(int nsh) { return nsh >= 4 ? 50 : nsh == 3 ? 26 : nsh == 2 ? 14 : 8; }

struct SParams {
    int L1, L2, L3, nens;
    int k0, kn;                 // the ensembles a launch covers: k0 .. k0 + kn - 1 (all by default)
    int P1, P2;                 // padded row and plane pitch (cells)
    long long pbox;             // cells per padded sublattice box = P2 * (L3 + 4)
    long long nsite;            // sites per ensemble (2 L1 L2 L3)
    float4 *mt, *mp;            // padded mirrors at t and at the predictor
    // the predictor's damped field b2eff plus the corrector's thermal term (see predict_update)
    float *b2x, *b2y, *b2z;
    float *lox, *loy, *loz;     // double-single residuals (precision 2)
    double *mx, *my, *mz;       // FP64 master (precision 1)
    float cA[4][2], cD[4][2];   // coupling on unit vectors: cA[sh][s_i] + s_j * cD[sh][s_i]
    float sigma[2];             // thermal-field amplitude per species (Depondt, depondt.f90:143-144)
    float lam, dtg;             // damping, delta_t*gama/(1+lambda^2)
    float ext[3];
    uint64_t seed;
    const int64_t *d_step;
    long long step_off;
    int *err;                   // set when a plane wait of the staged kernels ran past its limit
};

// Padded pitches of a cubic L^3 lattice; LC = 0 selects the runtime pitches.
__host__ __device__ constexpr int pitch1(int L) { return ((L + XOFF + 2) + 7) / 8 * 8; }
__host__ __device__ constexpr int pitch2(int L) { return pitch1(L) * (L + 4); }

// Lattice edges and pitches: compile-time for the compiled cubic sizes (LC > 0), so the
// index arithmetic folds into immediates; from the parameters otherwise.
template <int LC> __device__ __forceinline__ int gl1(const SParams &p) { if constexpr (LC) return LC; else return p.L1; }
template <int LC> __device__ __forceinline__ int gl2(const SParams &p) { if constexpr (LC) return LC; else return p.L2; }
template <int LC> __device__ __forceinline__ int gl3(const SParams &p) { if constexpr (LC) return LC; else return p.L3; }
template <int LC> __device__ __forceinline__ int gp1(const SParams &p) {
    if constexpr (LC) return pitch1(LC); else return p.P1;
}
template <int LC> __device__ __forceinline__ long long gp2(const SParams &p) {
    if constexpr (LC) return pitch2(LC); else return p.P2;
}
template <int LC> __device__ __forceinline__ long long gpbox(const SParams &p) {
    if constexpr (LC) return (long long)pitch2(LC) * (LC + 4); else return p.pbox;
}

template <int LC = 0>
__device__ __forceinline__ long long pidx(const SParams &p, int k, int b, int x, int y, int z) {
    return (long long)(k * 2 + b) * gpbox<LC>(p) +
           ((long long)(z + 2) * gp2<LC>(p) + (long long)(y + 2) * gp1<LC>(p) + (x + XOFF));
}
template <int LC = 0>
__device__ __forceinline__ long long uidx(const SParams &p, int k, int b, int x, int y, int z) {
    return (((long long)(k * 2 + b) * gl3<LC>(p) + z) * gl2<LC>(p) + y) * (long long)gl1<LC>(p) + x;
}
// Reference numbering i = I0 + NA*(I1 + N1*(I2 + N2*I3)) (0-based) for the Philox
// counter, so the structured and the generic path draw the same thermal-field stream.
template <int LC = 0>
__device__ __forceinline__ long long ref_site(const SParams &p, int b, int x, int y, int z) {
    return b + 2LL * (x + (long long)gl1<LC>(p) * (y + (long long)gl2<LC>(p) * z));
}

// Store a site's mirror value and its periodic ghost copies.
template <int LC = 0>
__device__ __forceinline__ void store_mirror(const SParams &p, float4 *m, int k, int b, int x, int y, int z,
                                             float4 v) {
    const int L1 = gl1<LC>(p), L2 = gl2<LC>(p), L3 = gl3<LC>(p);
    float4 *bx = m + (long long)(k * 2 + b) * gpbox<LC>(p);
    const int gx0 = x + XOFF, gy0 = y + 2, gz0 = z + 2;
    // second (ghost) coordinate per axis, -1 when the site is not within 2 cells of that face
    const int gx1 = x < 2 ? gx0 + L1 : (x >= L1 - 2 ? gx0 - L1 : -1);
    const int gy1 = y < 2 ? gy0 + L2 : (y >= L2 - 2 ? gy0 - L2 : -1);
    const int gz1 = z < 2 ? gz0 + L3 : (z >= L3 - 2 ? gz0 - L3 : -1);
    const long long py0 = (long long)gy0 * gp1<LC>(p), pz0 = (long long)gz0 * gp2<LC>(p);
    bx[pz0 + py0 + gx0] = v;
    if (gx1 < 0 && gy1 < 0 && gz1 < 0) return;
    const long long py1 = (long long)gy1 * gp1<LC>(p), pz1 = (long long)gz1 * gp2<LC>(p);
    if (gx1 >= 0) bx[pz0 + py0 + gx1] = v;
    if (gy1 >= 0) {
        bx[pz0 + py1 + gx0] = v;
        if (gx1 >= 0) bx[pz0 + py1 + gx1] = v;
    }
    if (gz1 >= 0) {
        bx[pz1 + py0 + gx0] = v;
        if (gx1 >= 0) bx[pz1 + py0 + gx1] = v;
        if (gy1 >= 0) {
            bx[pz1 + py1 + gx0] = v;
            if (gx1 >= 0) bx[pz1 + py1 + gx1] = v;
        }
    }
}


template <int NSH, int b, int LC>
__device__ __forceinline__ void gather_b(const SParams &p, const float4 *__restrict__ m, int k, int x, int y, int z,
                                         int si, float B[3]) {
    constexpr int NB = nb_of_shells(NSH);
    // with LC fixed at compile time every neighbour offset is an immediate in the load
    const int P1 = LC ? pitch1(LC) : p.P1;
    const int P2 = LC ? pitch2(LC) : p.P2;
    const long long own = (long long)(z + 2) * P2 + (long long)(y + 2) * P1 + (x + XOFF);
    const float4 *base0 = m + (long long)(k * 2 + 0) * p.pbox + own;
    const float4 *base1 = m + (long long)(k * 2 + 1) * p.pbox + own;
    float cA[4], cD[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        cA[s] = si ? p.cA[s][1] : p.cA[s][0];
        cD[s] = si ? p.cD[s][1] : p.cD[s][0];
    }
    float bx = 0.f, by = 0.f, bz = 0.f;
#pragma unroll
    for (int s = 0; s < NB; ++s) {
        const St e = stencil_entry(b, s);
        const int off = e.dz * P2 + e.dy * P1 + e.dx;  // block-uniform (immediate when LC > 0)
        const float4 v = __ldg((e.bj ? base1 : base0) + off);
        const float c = fmaf(v.w, cD[e.sh - 1], cA[e.sh - 1]);
        bx = fmaf(c, v.x, bx);
        by = fmaf(c, v.y, by);
        bz = fmaf(c, v.z, bz);
    }
    B[0] = bx + p.ext[0];
    B[1] = by + p.ext[1];
    B[2] = bz + p.ext[2];
}

// Depondt's effective field including damping: bdup = bloc + lambda * e x bloc
__device__ __forceinline__ void depondt_bdup(float lam, const float e[3], const float bl[3], float o[3]) {
    o[0] = bl[0] + lam * (e[1] * bl[2] - e[2] * bl[1]);
    o[1] = bl[1] + lam * (e[2] * bl[0] - e[0] * bl[2]);
    o[2] = bl[2] + lam * (e[0] * bl[1] - e[1] * bl[0]);
}

// Rodrigues rotation increment: R e - e = (1-cos v)[(h.e)h - e] + sin v (h x e),
// with h = bdup/|bdup| and v = |bdup| dt gama/(1+lambda^2)  (depondt.f90:156-179).
__device__ __forceinline__ void rotation_delta(const float bd[3], const float e[3], float dtg, float d[3]) {
    // |bd| and 1/|bd| from one reciprocal square root; the tiny addend keeps a zero field
    // at zero rotation, as the reference's + 1e-15 on the norm does (depondt.f90:159)
    const float n2 = bd[0] * bd[0] + bd[1] * bd[1] + bd[2] * bd[2];
    const float inv = rsqrtf(n2 + 1e-30f);
    const float bn = n2 * inv;
    float hx = bd[0] * inv, hy = bd[1] * inv, hz = bd[2] * inv;
    float v = bn * dtg;
    float sv, u;
    if (v < 0.25f) {
        // Taylor series to v^7 / v^8: truncation below 1e-11 for v < 0.25, i.e. at
        // FP32 rounding, and far cheaper than the accurate library sincosf
        float v2 = v * v;
        sv = v * fmaf(v2, fmaf(v2, fmaf(v2, -1.0f / 5040.0f, 1.0f / 120.0f), -1.0f / 6.0f), 1.0f);
        u = v2 * fmaf(v2, fmaf(v2, fmaf(v2, -1.0f / 40320.0f, 1.0f / 720.0f), -1.0f / 24.0f), 0.5f);
    } else {
        float cv;
        sincosf(v, &sv, &cv);
        float sh = sinf(0.5f * v);
        u = 2.0f * sh * sh;  // 1 - cos v without cancellation
    }
    float he = hx * e[0] + hy * e[1] + hz * e[2];
    d[0] = u * (he * hx - e[0]) + sv * (hy * e[2] - hz * e[1]);
    d[1] = u * (he * hy - e[1]) + sv * (hz * e[0] - hx * e[2]);
    d[2] = u * (he * hz - e[2]) + sv * (hx * e[1] - hy * e[0]);
}

struct Site {
    int x, y, z, b, k;
};

__device__ __forceinline__ bool site_of_thread(const SParams &p, Site &s) {
    const int nyt = (p.L2 + blockDim.y - 1) / blockDim.y;
    s.x = threadIdx.x;
    s.y = (blockIdx.x % nyt) * blockDim.y + threadIdx.y;
    s.z = blockIdx.x / nyt;
    s.b = blockIdx.y;
    s.k = blockIdx.z + p.k0;
    return s.x < p.L1 && s.y < p.L2;
}

// Predictor update of one site from its field B: thermal field, Depondt damped
// field, Rodrigues rotation; writes m_pred (with ghosts) and one 3-vector for the
// corrector.  The corrector's damped field at the predicted spin ep splits as
//   bdup(ep, B(ep) + th) = bdup(ep, B(ep)) + [th + lambda ep x th],
// and the bracket is known here (ep is this thread's own result), so the predictor
// stores b2eff + th + lambda ep x th (depondt.f90:152-154, 290-301) and the thermal field
// itself is neither stored nor drawn again.
template <int LC = 0>
__device__ __forceinline__ void predict_update(const SParams &p, int k, int b, int x, int y, int z, const float4 &me,
                                               const float B[3]) {
    const int si = me.w != 0.f ? 1 : 0;
    const long long step = *p.d_step + p.step_off;
    float zr[3];
    normal3_f32_fast(p.seed, ref_site<LC>(p, b, x, y, z), k, step, kStreamLLG, zr);
    const float sg = p.sigma[si];
    const float e[3] = {me.x, me.y, me.z};
    const float th[3] = {zr[0] * sg, zr[1] * sg, zr[2] * sg};
    float bl[3] = {B[0] + th[0], B[1] + th[1], B[2] + th[2]};
    float bd[3], d[3];
    depondt_bdup(p.lam, e, bl, bd);
    rotation_delta(bd, e, p.dtg, d);
    const float ep[3] = {e[0] + d[0], e[1] + d[1], e[2] + d[2]};
    store_mirror<LC>(p, p.mp, k, b, x, y, z, make_float4(ep[0], ep[1], ep[2], me.w));
    float tc[3];
    depondt_bdup(p.lam, ep, th, tc);
    const long long u = uidx<LC>(p, k, b, x, y, z);
    p.b2x[u] = bd[0] + tc[0];
    p.b2y[u] = bd[1] + tc[1];
    p.b2z[u] = bd[2] + tc[2];
}

template <int NSH, int b, int LC>
__device__ __forceinline__ void predict_site(const SParams &p, const Site &s) {
    const float4 me = p.mt[pidx(p, s.k, b, s.x, s.y, s.z)];
    float B[3];
    gather_b<NSH, b, LC>(p, p.mt, s.k, s.x, s.y, s.z, me.w != 0.f ? 1 : 0, B);
    predict_update(p, s.k, b, s.x, s.y, s.z, me, B);
}

template <int NSH, int LC>
__global__ void __launch_bounds__(256) stencil_predict(SParams p) {
    Site s;
    if (!site_of_thread(p, s)) return;
    if (s.b == 0) predict_site<NSH, 0, LC>(p, s);
    else predict_site<NSH, 1, LC>(p, s);
}

// Corrector update of one site from the field B at the predictor: Depondt
// average with b2eff, rotation of m(t), master update and renormalisation.
// What the corrector of one site reads besides the gather: m(t) (the mirror), the
// predictor's stored field, and the master (FP64, or the double-single residual).
// Loaded before the gather so that these DRAM reads overlap it.
template <int MASTER>
struct CorrIn {
    float4 mt;
    float b2[3];
    float lo[3];    // MASTER 2
    double m[3];    // MASTER 1
};

template <int MASTER, int LC = 0>
__device__ __forceinline__ void correct_load(const SParams &p, int k, int b, int x, int y, int z, CorrIn<MASTER> &c) {
    const long long u = uidx<LC>(p, k, b, x, y, z);
    c.mt = p.mt[pidx<LC>(p, k, b, x, y, z)];
    c.b2[0] = p.b2x[u];
    c.b2[1] = p.b2y[u];
    c.b2[2] = p.b2z[u];
    if constexpr (MASTER == 1) {
        c.m[0] = p.mx[u];
        c.m[1] = p.my[u];
        c.m[2] = p.mz[u];
    } else {
        c.lo[0] = p.lox[u];
        c.lo[1] = p.loy[u];
        c.lo[2] = p.loz[u];
    }
}

template <int MASTER, int LC = 0>  // MASTER 1: FP64, 2: double-single
__device__ __forceinline__ void correct_finish(const SParams &p, int k, int b, int x, int y, int z, const float4 &mp,
                                               const float B[3], const CorrIn<MASTER> &ci) {
    const long long u = uidx<LC>(p, k, b, x, y, z);
    const float ep[3] = {mp.x, mp.y, mp.z};
    float bd[3];
    depondt_bdup(p.lam, ep, B, bd);   // the thermal term is in b2 (predict_update)
    bd[0] = 0.5f * bd[0] + 0.5f * ci.b2[0];
    bd[1] = 0.5f * bd[1] + 0.5f * ci.b2[1];
    bd[2] = 0.5f * bd[2] + 0.5f * ci.b2[2];
    const float4 mt = ci.mt;
    const float eh[3] = {mt.x, mt.y, mt.z};
    float d[3];
    rotation_delta(bd, eh, p.dtg, d);
    float4 out;
    if (MASTER == 1) {
        double e0 = ci.m[0] + (double)d[0], e1 = ci.m[1] + (double)d[1], e2 = ci.m[2] + (double)d[2];
        double n2 = fma(e2, e2, fma(e1, e1, e0 * e0));
        double xx = n2 - 1.0;
        double sc = fma(xx, fma(0.375, xx, -0.5), 1.0);  // 1/sqrt(1+x) to second order, |x| ~ 1e-7
        e0 *= sc;
        e1 *= sc;
        e2 *= sc;
        p.mx[u] = e0;
        p.my[u] = e1;
        p.mz[u] = e2;
        out = make_float4((float)e0, (float)e1, (float)e2, mt.w);
    } else {
        float lo[3] = {ci.lo[0], ci.lo[1], ci.lo[2]};
        float hi[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            float sm, er;
            two_sum(eh[c], d[c], sm, er);
            quick_two_sum(sm, er + lo[c], hi[c], lo[c]);
        }
        // |e|^2 - 1 in double-single: sum of hi^2 (exact products) plus 2 hi lo
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
        float xx = xs + (xe + n2l);                // |e|^2 - 1: the FP32 rounding of one step's rotation
        float sm1 = xx * fmaf(0.375f, xx, -0.5f);  // 1/sqrt(1+x) - 1
        // e (1 + sm1): the correction hi sm1 is ~|xx| hi, far below half an ulp of hi, so it
        // joins the low word (lo sm1, below 1e-15 of e, is dropped); the next step's update
        // renormalises the pair
#pragma unroll
        for (int c = 0; c < 3; ++c) lo[c] = fmaf(hi[c], sm1, lo[c]);
        p.lox[u] = lo[0];
        p.loy[u] = lo[1];
        p.loz[u] = lo[2];
        out = make_float4(hi[0], hi[1], hi[2], mt.w);
    }
    store_mirror<LC>(p, p.mt, k, b, x, y, z, out);
}

template <int MASTER>
__device__ __forceinline__ void correct_update(const SParams &p, int k, int b, int x, int y, int z, const float4 &mp,
                                               const float B[3]) {
    CorrIn<MASTER> ci;
    correct_load<MASTER>(p, k, b, x, y, z, ci);
    correct_finish<MASTER>(p, k, b, x, y, z, mp, B, ci);
}

template <int NSH, int MASTER, int b, int LC>
__device__ __forceinline__ void correct_site(const SParams &p, const Site &s) {
    const float4 mp = p.mp[pidx(p, s.k, b, s.x, s.y, s.z)];
    float B[3];
    gather_b<NSH, b, LC>(p, p.mp, s.k, s.x, s.y, s.z, mp.w != 0.f ? 1 : 0, B);
    correct_update<MASTER>(p, s.k, b, s.x, s.y, s.z, mp, B);
}

template <int NSH, int MASTER, int LC>
__global__ void __launch_bounds__(256) stencil_correct(SParams p) {
    Site s;
    if (!site_of_thread(p, s)) return;
    if (s.b == 0) correct_site<NSH, MASTER, 0, LC>(p, s);
    else correct_site<NSH, MASTER, 1, LC>(p, s);
}

// ---------------------------------------------------------------------------
// z-blocked gather: a thread produces NZ sites of one sublattice stacked in z.
// Neighbour points shared by several of its sites are loaded once (about 28
// loads per site instead of 50 for the four-shell stencil, NZ = 4).  The point
// list and the (site, shell) pairs each point feeds are built by the constexpr
// evaluator and expanded with integer sequences, so every offset, coupling
// register and accumulator index is a compile-time constant.
struct ZbPt {
    int8_t bj, dx, dy, dz;
    uint8_t first, count;
};
struct ZbPair {
    int8_t q, sh;
};
struct ZbTables {
    ZbPt pts[256];
    ZbPair pairs[256];
    int npts, npairs;
};

__host__ __device__ constexpr ZbTables make_zb(int nsh, int b, int nz) {
    ZbTables t{};
    int np = 0, nq = 0;
    for (int bj = 0; bj < 2; ++bj)
        for (int zz = -2; zz <= nz + 1; ++zz)
            for (int dy = -2; dy <= 2; ++dy)
                for (int dx = -2; dx <= 2; ++dx) {
                    const int first = nq;
                    for (int q = 0; q < nz; ++q)
                        for (int s = 0; s < nb_of_shells(nsh); ++s) {
                            const St e = stencil_entry(b, s);
                            if (e.bj == bj && e.dx == dx && e.dy == dy && q + e.dz == zz)
                                t.pairs[nq++] = ZbPair{(int8_t)q, e.sh};
                        }
                    if (nq > first)
                        t.pts[np++] = ZbPt{(int8_t)bj, (int8_t)dx, (int8_t)dy, (int8_t)zz, (uint8_t)first,
                                           (uint8_t)(nq - first)};
                }
    t.npts = np;
    t.npairs = nq;
    return t;
}

template <int NSH, int B, int NZ>
struct ZB {
    static constexpr ZbTables t = make_zb(NSH, B, NZ);
};

template <int NSH, int B, int NZ, int I>
__device__ __forceinline__ void zb_pair(const float4 &v, const float (&cA)[NZ][4], const float (&cD)[NZ][4],
                                        float (&acc)[NZ][3]) {
    constexpr ZbPair pr = ZB<NSH, B, NZ>::t.pairs[I];
    const float c = fmaf(v.w, cD[pr.q][pr.sh - 1], cA[pr.q][pr.sh - 1]);
    acc[pr.q][0] = fmaf(c, v.x, acc[pr.q][0]);
    acc[pr.q][1] = fmaf(c, v.y, acc[pr.q][1]);
    acc[pr.q][2] = fmaf(c, v.z, acc[pr.q][2]);
}

template <int NSH, int B, int NZ, int FIRST, int... R>
__device__ __forceinline__ void zb_pairs(const float4 &v, const float (&cA)[NZ][4], const float (&cD)[NZ][4],
                                         float (&acc)[NZ][3], std::integer_sequence<int, R...>) {
    (zb_pair<NSH, B, NZ, FIRST + R>(v, cA, cD, acc), ...);
}

template <int NSH, int B, int NZ, int LC, int Q>
__device__ __forceinline__ void zb_point(const float4 *base0, const float4 *base1, const float (&cA)[NZ][4],
                                         const float (&cD)[NZ][4], float (&acc)[NZ][3]) {
    constexpr ZbPt pt = ZB<NSH, B, NZ>::t.pts[Q];
    constexpr int off = pt.dz * pitch2(LC) + pt.dy * pitch1(LC) + pt.dx;
    const float4 v = __ldg((pt.bj ? base1 : base0) + off);
    zb_pairs<NSH, B, NZ, pt.first>(v, cA, cD, acc, std::make_integer_sequence<int, pt.count>{});
}

template <int NSH, int B, int NZ, int LC, int... Q>
__device__ __forceinline__ void zb_points(const float4 *base0, const float4 *base1, const float (&cA)[NZ][4],
                                          const float (&cD)[NZ][4], float (&acc)[NZ][3],
                                          std::integer_sequence<int, Q...>) {
    (zb_point<NSH, B, NZ, LC, Q>(base0, base1, cA, cD, acc), ...);
}

template <int NSH, int B, int NZ, int LC, int KIND, int MASTER>
__device__ __forceinline__ void zb_sites(const SParams &p, int k, int x, int y, int z0) {
    constexpr int P1 = pitch1(LC), P2 = pitch2(LC);
    const float4 *m = KIND == 0 ? p.mt : p.mp;
    const long long own = (long long)(z0 + 2) * P2 + (long long)(y + 2) * P1 + (x + XOFF);
    const float4 *base0 = m + (long long)(k * 2 + 0) * p.pbox + own;
    const float4 *base1 = m + (long long)(k * 2 + 1) * p.pbox + own;
    float4 me[NZ];
    float cA[NZ][4], cD[NZ][4], acc[NZ][3];
#pragma unroll
    for (int q = 0; q < NZ; ++q) {
        me[q] = (B ? base1 : base0)[q * P2];
        const int si = me[q].w != 0.f ? 1 : 0;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            cA[q][s] = si ? p.cA[s][1] : p.cA[s][0];
            cD[q][s] = si ? p.cD[s][1] : p.cD[s][0];
        }
        acc[q][0] = acc[q][1] = acc[q][2] = 0.f;
    }
    zb_points<NSH, B, NZ, LC>(base0, base1, cA, cD, acc, std::make_integer_sequence<int, ZB<NSH, B, NZ>::t.npts>{});
#pragma unroll
    for (int q = 0; q < NZ; ++q) {
        const float Bf[3] = {acc[q][0] + p.ext[0], acc[q][1] + p.ext[1], acc[q][2] + p.ext[2]};
        if (KIND == 0) predict_update(p, k, B, x, y, z0 + q, me[q], Bf);
        else correct_update<MASTER>(p, k, B, x, y, z0 + q, me[q], Bf);
    }
}

template <int NSH, int NZ, int LC, int KIND, int MASTER>
__global__ void __launch_bounds__(256) stencil_zblock(SParams p) {
    const int nyt = (p.L2 + blockDim.y - 1) / blockDim.y;
    const int x = threadIdx.x;
    const int y = (blockIdx.x % nyt) * blockDim.y + threadIdx.y;
    const int z0 = (blockIdx.x / nyt) * NZ;
    const int k = blockIdx.z + p.k0;
    if (x >= p.L1 || y >= p.L2) return;
    if (blockIdx.y == 0) zb_sites<NSH, 0, NZ, LC, KIND, MASTER>(p, k, x, y, z0);
    else zb_sites<NSH, 1, NZ, LC, KIND, MASTER>(p, k, x, y, z0);
}

// ---------------------------------------------------------------------------
// Cell-blocked gather: a thread produces both sites (corner b = 0 and centre
// b = 1) of NZ cells stacked in z.  The two sublattices' neighbourhoods overlap
// (the centre's corner neighbours include the corner's own same-sublattice
// neighbours and vice versa), so the union of the 4 NZ sites' 50-point stencils
// is 24 points per site for NZ = 2 (36 with one sublattice per thread, 50 with one
// site).  Points and (site, shell) pairs come from the constexpr evaluator as above;
// site index = b * NZ + q.
__host__ __device__ constexpr ZbTables make_cb(int nsh, int nz) {
    ZbTables t{};
    int np = 0, nq = 0;
    for (int bj = 0; bj < 2; ++bj)
        for (int zz = -2; zz <= nz + 1; ++zz)
            for (int dy = -2; dy <= 2; ++dy)
                for (int dx = -2; dx <= 2; ++dx) {
                    const int first = nq;
                    for (int b = 0; b < 2; ++b)
                        for (int q = 0; q < nz; ++q)
                            for (int s = 0; s < nb_of_shells(nsh); ++s) {
                                const St e = stencil_entry(b, s);
                                if (e.bj == bj && e.dx == dx && e.dy == dy && q + e.dz == zz)
                                    t.pairs[nq++] = ZbPair{(int8_t)(b * nz + q), e.sh};
                            }
                    if (nq > first)
                        t.pts[np++] = ZbPt{(int8_t)bj, (int8_t)dx, (int8_t)dy, (int8_t)zz, (uint8_t)first,
                                           (uint8_t)(nq - first)};
                }
    t.npts = np;
    t.npairs = nq;
    return t;
}

template <int NSH, int NZ>
struct CB {
    static constexpr ZbTables t = make_cb(NSH, NZ);
};

template <int NSH, int NZ, int I>
__device__ __forceinline__ void cb_pair(const float4 &v, const float (&cA)[2 * NZ][4], const float (&cD)[2 * NZ][4],
                                        float (&acc)[2 * NZ][3]) {
    constexpr ZbPair pr = CB<NSH, NZ>::t.pairs[I];
    const float c = fmaf(v.w, cD[pr.q][pr.sh - 1], cA[pr.q][pr.sh - 1]);
    acc[pr.q][0] = fmaf(c, v.x, acc[pr.q][0]);
    acc[pr.q][1] = fmaf(c, v.y, acc[pr.q][1]);
    acc[pr.q][2] = fmaf(c, v.z, acc[pr.q][2]);
}

template <int NSH, int NZ, int FIRST, int... R>
__device__ __forceinline__ void cb_pairs(const float4 &v, const float (&cA)[2 * NZ][4], const float (&cD)[2 * NZ][4],
                                         float (&acc)[2 * NZ][3], std::integer_sequence<int, R...>) {
    (cb_pair<NSH, NZ, FIRST + R>(v, cA, cD, acc), ...);
}

// Point source of the gather: the padded global mirror, read through the
// read-only data cache.  (bj, dx, dy, dz) are compile-time offsets from the
// thread's cell at its first z.
template <int LC>
struct GlobalSrc {
    const float4 *base0, *base1;
    template <int BJ, int DX, int DY, int DZ>
    __device__ __forceinline__ float4 get() const {
        constexpr int off = DZ * pitch2(LC) + DY * pitch1(LC) + DX;
        return __ldg((BJ ? base1 : base0) + off);
    }
};

template <int NSH, int NZ, class Src, int Q>
__device__ __forceinline__ void cb_point(const Src &src, const float (&cA)[2 * NZ][4], const float (&cD)[2 * NZ][4],
                                         float (&acc)[2 * NZ][3]) {
    constexpr ZbPt pt = CB<NSH, NZ>::t.pts[Q];
    const float4 v = src.template get<pt.bj, pt.dx, pt.dy, pt.dz>();
    cb_pairs<NSH, NZ, pt.first>(v, cA, cD, acc, std::make_integer_sequence<int, pt.count>{});
}

template <int NSH, int NZ, class Src, int... Q>
__device__ __forceinline__ void cb_points(const Src &src, const float (&cA)[2 * NZ][4], const float (&cD)[2 * NZ][4],
                                          float (&acc)[2 * NZ][3], std::integer_sequence<int, Q...>) {
    (cb_point<NSH, NZ, Src, Q>(src, cA, cD, acc), ...);
}

template <int NZ, class Src, int... I>
__device__ __forceinline__ void cb_own(const Src &src, float4 (&me)[2 * NZ], std::integer_sequence<int, I...>) {
    ((me[I] = src.template get<I / NZ, 0, 0, I % NZ>()), ...);
}

// Both sites of NZ cells: own values, the gather, then the predictor or corrector
// update of every site.
template <int NSH, int NZ, int LC, int KIND, int MASTER, class Src>
__device__ __forceinline__ void cb_sites(const SParams &p, const Src &src, int k, int x, int y, int z0) {
    float4 me[2 * NZ];
    float cA[2 * NZ][4], cD[2 * NZ][4], acc[2 * NZ][3];
    CorrIn<MASTER == 1 ? 1 : 2> ci[KIND == 1 ? 2 * NZ : 1];
    if constexpr (KIND == 1) {
        // the corrector's own-site DRAM reads first: they overlap the gather
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int q = 0; q < NZ; ++q) correct_load<MASTER == 1 ? 1 : 2, LC>(p, k, b, x, y, z0 + q, ci[b * NZ + q]);
    }
    cb_own<NZ>(src, me, std::make_integer_sequence<int, 2 * NZ>{});
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int q = 0; q < NZ; ++q) {
            const int i = b * NZ + q;
            const int si = me[i].w != 0.f ? 1 : 0;
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                cA[i][s] = si ? p.cA[s][1] : p.cA[s][0];
                cD[i][s] = si ? p.cD[s][1] : p.cD[s][0];
            }
            acc[i][0] = acc[i][1] = acc[i][2] = 0.f;
        }
    cb_points<NSH, NZ>(src, cA, cD, acc, std::make_integer_sequence<int, CB<NSH, NZ>::t.npts>{});
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int q = 0; q < NZ; ++q) {
            const int i = b * NZ + q;
            const float Bf[3] = {acc[i][0] + p.ext[0], acc[i][1] + p.ext[1], acc[i][2] + p.ext[2]};
            if constexpr (KIND == 0) predict_update<LC>(p, k, b, x, y, z0 + q, me[i], Bf);
            else correct_finish<MASTER == 1 ? 1 : 2, LC>(p, k, b, x, y, z0 + q, me[i], Bf, ci[i]);
        }
}

template <int NSH, int NZ, int LC, int KIND, int MASTER>
__global__ void __launch_bounds__(256) stencil_cells(SParams p) {
    const int nyt = (p.L2 + blockDim.y - 1) / blockDim.y;
    const int x = threadIdx.x;
    const int y = (blockIdx.x % nyt) * blockDim.y + threadIdx.y;
    const int z0 = (blockIdx.x / nyt) * NZ;
    const int k = blockIdx.z + p.k0;
    if (x >= p.L1 || y >= p.L2) return;
    const float4 *m = KIND == 0 ? p.mt : p.mp;
    const long long own = (long long)(z0 + 2) * pitch2(LC) + (long long)(y + 2) * pitch1(LC) + (x + XOFF);
    GlobalSrc<LC> src;
    src.base0 = m + (long long)(k * 2 + 0) * p.pbox + own;
    src.base1 = m + (long long)(k * 2 + 1) * p.pbox + own;
    cb_sites<NSH, NZ, LC, KIND, MASTER>(p, src, k, x, y, z0);
}


// ---------------------------------------------------------------------------
// Plane-staged gather (TMA).  A CTA owns a TX x TY tile of cells of one ensemble and
// a chunk of ZC planes, and marches up z two planes at a time.  The planes it reads
// arrive by TMA (cp.async.bulk.tensor, 5-D map over the padded mirror: float lane,
// x, y, z, ensemble x sublattice) into a ring of kRing slots in shared memory; slot
// u holds the (TX + 3) x (TY + 3) box of the centre sublattice at plane pz and of the
// corner sublattice at plane pz + 1 (pz = zs - 2 + u), which is exactly what output
// plane z needs from slots pz = z - 2 .. z + 1 (the corner sites' centre neighbours
// lie at dz in [-2, 1], the centre sites' corner neighbours at dz in [-1, 2]).  Each
// iteration computes both sites of two planes of the tile (cb_sites) from shared
// memory while the slots of the next iteration load; every neighbour is fetched from
// DRAM / L2 once per tile instead of once per reading site.
template <int TX, int TY, int R>
struct TileGeom {
    static constexpr int BW = TX + 3, BH = TY + 3;
    static constexpr uint32_t kBox = (uint32_t)BW * BH * 16;          // bytes the TMA box moves
    static constexpr uint32_t kBoxA = (kBox + 127) / 128 * 128;       // box stride in shared memory
    static constexpr uint32_t kSlot = 2 * kBoxA;
    static constexpr size_t kSmem = (size_t)R * kSlot + 128;          // + alignment slack
};

// Tile geometry of the plane-staged kernels per compiled size: the tile (TX, TY), the
// planes of a z chunk (ZC), the planes per iteration (NZ), the ring's slots (R) and the
// CTAs per SM the registers are sized for (MINB).
// V = 0: two planes per iteration, 7 slots, registers for 2 CTAs per SM; V = 1: one
// plane, 5 slots, registers for 3 CTAs per SM (more warps, more reads per site).
template <int LC, int V = 0>
struct TmaTile {
    static constexpr int TX = LC == 100 ? 50 : (LC == 64 ? 32 : LC);
    static constexpr int TY = LC == 100 ? 5 : (LC == 64 ? 8 : LC);
    static constexpr int ZC = LC == 100 ? 20 : (LC == 64 ? 16 : LC);
    static constexpr int NZ = V ? 1 : 2, R = V ? 5 : 7, MINB = V ? 3 : 2;
};

// Point source of the gather: this thread's cell in the NZ + 3 slots of the current
// iteration (slot of plane z - 2 + j at pj[j]).
template <int TX, int TY, int NZ, int R>
struct SmemSrc {
    const uint8_t *pj[NZ + 3];
    template <int BJ, int DX, int DY, int DZ>
    __device__ __forceinline__ float4 get() const {
        using G = TileGeom<TX, TY, R>;
        constexpr int j = DZ + 1 + BJ;
        constexpr int off = BJ * (int)G::kBoxA + 16 * ((DY + 1 + BJ) * G::BW + DX + 1 + BJ);
        static_assert(j >= 0 && j < NZ + 3, "plane outside the iteration's slots");
        return *reinterpret_cast<const float4 *>(pj[j] + off);
    }
};

__device__ __forceinline__ void tma_load_5d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1, int c2,
                                            int c3, int c4) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, %6, %7}], "
        "[%2];" ::"r"(tc::smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(tc::smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4)
        : "memory");
}

// Iteration i covers planes zs + NZ i .. + NZ - 1 and reads slots u = NZ i .. NZ i + NZ + 2;
// slot u may be (re)filled once slot u - R is no longer read, i.e. u < NZ i + R at the
// top of iteration i.
template <int NSH, int LC, int TX, int TY, int ZC, int NZ, int R, int MINB, int KIND, int MASTER>
__global__ void __launch_bounds__(TX * TY, MINB) stencil_tma(const __grid_constant__ CUtensorMap mapm, SParams p,
                                                             int ntx, int nty) {
    using G = TileGeom<TX, TY, R>;
    static_assert(ZC % NZ == 0 && ZC / NZ >= 2, "whole iterations, at least two of them");
    static_assert(R >= NZ + 4, "one slot of look-ahead at least");
    constexpr int kSlots = ZC + 3;  // pz = zs - 2 .. zs + ZC
    extern __shared__ uint8_t tma_smem_raw[];
    uint8_t *ring = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(tma_smem_raw) + 127) & ~(uintptr_t)127);
    __shared__ __align__(8) uint64_t full[R];
    __shared__ int fail;
    const int t = threadIdx.x;
    const int bid = blockIdx.x;
    const int x0 = (bid % ntx) * TX, y0 = ((bid / ntx) % nty) * TY, zs = (bid / (ntx * nty)) * ZC;
    const int k = blockIdx.z + p.k0;
    const int tx = t % TX, ty = t / TX;
    const int x = x0 + tx, y = y0 + ty;
    const bool active = x < p.L1 && y < p.L2;
    if (t == 0) {
        for (int r = 0; r < R; ++r) tc::mbar_init(&full[r], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fail = 0;
    }
    __syncthreads();
    // slot u: corner plane pz + 1 and centre plane pz, pz = zs - 2 + u, padded z = pz + 2
    auto issue = [&](int u) {
        const int r = u % R, pz = zs - 2 + u;
        uint8_t *dst = ring + r * G::kSlot;
        tc::mbar_expect_tx(&full[r], 2 * G::kBox);
        tma_load_5d(dst, &mapm, &full[r], 0, x0 - 1 + XOFF, y0 + 1, pz + 3, 2 * k);
        tma_load_5d(dst + G::kBoxA, &mapm, &full[r], 0, x0 - 2 + XOFF, y0, pz + 2, 2 * k + 1);
    };
    int issued = 0;  // slots issued so far (thread 0)
    int waited = 0;  // slots this thread has seen complete
    if (t == 0)
        for (; issued < R && issued < kSlots; ++issued) issue(issued);
    const uint8_t *cell = ring + 16 * (ty * G::BW + tx);
    for (int i = 0; i < ZC / NZ; ++i) {
        if (i > 0) {
            __syncthreads();  // the previous iteration's reads of its oldest slots are done
            if (fail) break;
            if (t == 0)
                for (; issued < kSlots && issued < NZ * i + R; ++issued) issue(issued);
        }
        bool ok = true;
        for (; waited <= NZ * i + NZ + 2; ++waited) ok = ok && tc::mbar_wait(&full[waited % R], (waited / R) & 1);
        if (!ok) {
            fail = 1;
            atomicExch(p.err, 1);
            continue;
        }
        if (active) {
            SmemSrc<TX, TY, NZ, R> src;
#pragma unroll
            for (int j = 0; j < NZ + 3; ++j) src.pj[j] = cell + ((NZ * i + j) % R) * G::kSlot;
            cb_sites<NSH, NZ, LC, KIND, MASTER>(p, src, k, x, y, zs + NZ * i);
        }
    }
    __syncthreads();
    if (fail && t == 0) {
        // a wait ran out: let the copies still in flight land (each wait bounded too)
        // before the CTA's shared memory is given back
        for (int u = issued - R < 0 ? 0 : issued - R; u < issued; ++u) tc::mbar_wait(&full[u % R], (u / R) & 1);
    }
}

// Conversions between the generic FP64 state (s.e / s.eM, [k][i] reference order)
// and the structured state.
__global__ void to_structured(SParams p, const double *ex, const double *ey, const double *ez,
                              const int8_t *species, int master) {
    long long t = (long long)p.k0 * p.nsite + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long total = p.nsite * (p.k0 + p.kn);
    if (t >= total) return;
    int k = (int)(t / p.nsite);
    long long i = t - (long long)k * p.nsite;  // reference site index
    int b = (int)(i & 1);
    long long cell = i >> 1;
    int x = (int)(cell % p.L1), y = (int)((cell / p.L1) % p.L2), z = (int)(cell / ((long long)p.L1 * p.L2));
    long long u = uidx(p, k, b, x, y, z);
    double e0 = ex[t], e1 = ey[t], e2 = ez[t];
    float w = species ? (float)species[i] : 0.f;
    float h0 = (float)e0, h1 = (float)e1, h2 = (float)e2;
    store_mirror(p, p.mt, k, b, x, y, z, make_float4(h0, h1, h2, w));
    if (master == 1) {
        p.mx[u] = e0;
        p.my[u] = e1;
        p.mz[u] = e2;
    } else {
        p.lox[u] = (float)(e0 - (double)h0);
        p.loy[u] = (float)(e1 - (double)h1);
        p.loz[u] = (float)(e2 - (double)h2);
    }
}

__global__ void from_structured(SParams p, double *ex, double *ey, double *ez, double *mx, double *my, double *mz,
                                const double *mmom, int master) {
    long long t = (long long)p.k0 * p.nsite + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long total = p.nsite * (p.k0 + p.kn);
    if (t >= total) return;
    int k = (int)(t / p.nsite);
    long long i = t - (long long)k * p.nsite;
    int b = (int)(i & 1);
    long long cell = i >> 1;
    int x = (int)(cell % p.L1), y = (int)((cell / p.L1) % p.L2), z = (int)(cell / ((long long)p.L1 * p.L2));
    long long u = uidx(p, k, b, x, y, z);
    double e0, e1, e2;
    if (master == 1) {
        e0 = p.mx[u];
        e1 = p.my[u];
        e2 = p.mz[u];
    } else {
        float4 h = p.mt[pidx(p, k, b, x, y, z)];
        e0 = (double)h.x + (double)p.lox[u];
        e1 = (double)h.y + (double)p.loy[u];
        e2 = (double)h.z + (double)p.loz[u];
    }
    double m = mmom[t];
    ex[t] = e0;
    ey[t] = e1;
    ez[t] = e2;
    mx[t] = e0 * m;
    my[t] = e1 * m;
    mz[t] = e2 * m;
}

}  // namespace

struct StructuredFast {
    SParams p{};
    int nshell = 0, master = 1, lc = 0;
    // compiled sizes: 0 one sublattice per thread (stencil_zblock), 1 both sublattices
    // (stencil_cells), 2 both sublattices from TMA-staged planes (stencil_tma)
    int kernel = 2;
    CUtensorMap map_mt, map_mp;  // 5-D maps of the padded mirrors (kernel 2)
    dim3 grid, block;
    int8_t *species = nullptr;
    // what the thermal amplitude and the rotation scale are computed from
    double lam = 0.0, temp = 0.0, delta_t = 0.0, temprescale = 1.0, mom[2] = {1.0, 1.0};
};

// 5-D TMA map over a padded mirror array: (float lane, x, y, z, ensemble x sublattice)
// with the box of one plane of a TX x TY tile plus its three-cell halo.
static int mirror_map(CUtensorMap *m, const StructuredFast *f, const float4 *base, int tx, int ty) {
    const SParams &p = f->p;
    const uint64_t dims[5] = {4, (uint64_t)p.P1, (uint64_t)p.L2 + 4, (uint64_t)p.L3 + 4, (uint64_t)2 * p.nens};
    const uint64_t strides[4] = {16, (uint64_t)p.P1 * 16, (uint64_t)p.P2 * 16, (uint64_t)p.pbox * 16};
    const uint32_t box[5] = {4, (uint32_t)tx + 3, (uint32_t)ty + 3, 1, 1};
    return tc::encode_tiled(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, 5, base, dims, strides, box);
}

// Depondt thermal amplitude per species (depondt.f90:143-145) and rotation scale from the
// uniform damping and temperature and the simulation's physical constants; again after
// set_temperature and set_units.
static void structured_coefficients(const Sim &s, StructuredFast *f) {
    const HamDev &h = s.ham;
    for (int ti = 0; ti < 2; ++ti) {
        double Dp = (2.0 * f->lam * h.kbolt) / (f->delta_t * h.gama * h.mub);
        f->p.sigma[ti] = (float)sqrt(Dp * f->temprescale * f->temp / f->mom[ti]);
    }
    f->p.lam = (float)f->lam;
    f->p.dtg = (float)(f->delta_t * h.gama / (1.0 + f->lam * f->lam));
}

int structured_set_temperature(Sim &s, const double *temp_array) {
    for (int i = 1; i < s.ham.natom; ++i)
        if (temp_array[i] != temp_array[0]) {
            set_error("set_temperature: the structured path (precision 1, 2) needs a uniform temperature");
            return UPPASD_GPU_EUNSUPPORTED;
        }
    s.fast->temp = temp_array[0];
    structured_coefficients(s, s.fast);
    return UPPASD_GPU_OK;
}

void structured_refresh(Sim &s) {
    if (s.fast) structured_coefficients(s, s.fast);
}

static void fast_free(StructuredFast *f) {
    if (!f) return;
    void *ptrs[] = {f->p.mt, f->p.mp, f->p.b2x, f->p.b2y, f->p.b2z, f->p.lox, f->p.loy, f->p.loz,
                    f->p.mx, f->p.my, f->p.mz, f->species, f->p.err};
    for (void *q : ptrs) cudaFree(q);
    delete f;
}

void structured_free(Sim &s) {
    fast_free(s.fast);
    s.fast = nullptr;
}

int structured_init(Sim &s, const uppasd_gpu_consts *c, const uppasd_gpu_arrays *a) {
    auto no = [](const std::string &m) {
        set_error("structured path not applicable: " + m);
        return UPPASD_GPU_EUNSUPPORTED;
    };
    if (c->sdealgh != 5) return no("only the Depondt solver (SDEalgh 5) is implemented");
    if (c->do_dm || c->do_aniso) return no("DM and anisotropy terms use the generic path");
    if (c->na != 2 || c->n1 < 4 || c->n2 < 4 || c->n3 < 4) return no("needs a bcc cell grid (na = 2, n >= 4)");
    const int N = c->natom, M = c->mensemble, L1 = c->n1, L2 = c->n2, L3 = c->n3;
    if ((long long)2 * L1 * L2 * L3 != N) return no("natom != 2*n1*n2*n3");
    if (L1 > 1024) return no("n1 must be <= 1024");
    for (int i = 1; i < N; ++i)
        if (a->lambda1_array[i] != a->lambda1_array[0] || a->temp_array[i] != a->temp_array[0])
            return no("damping and temperature must be uniform");
    for (long long t = 1; t < (long long)N * M; ++t)
        if (a->external_field[3 * t] != a->external_field[0] || a->external_field[3 * t + 1] != a->external_field[1] ||
            a->external_field[3 * t + 2] != a->external_field[2])
            return no("external field must be uniform");
    std::vector<int8_t> sp(N, 0);
    if (a->species)
        for (int i = 0; i < N; ++i) {
            if (a->species[i] < 0 || a->species[i] > 1) return no("at most two species");
            sp[i] = (int8_t)a->species[i];
        }
    // moment per species (must be uniform within a species and across ensembles)
    double mom[2] = {-1.0, -1.0};
    for (long long t = 0; t < (long long)N * M; ++t) {
        int sI = sp[t % N];
        if (mom[sI] < 0) mom[sI] = a->mmom[t];
        else if (mom[sI] != a->mmom[t]) return no("moment must be uniform per species");
    }
    // identify shells and the coupling table, verifying every neighbour and coupling
    const int mnn = c->max_no_neigh;
    int nshell = 0;
    for (int sh : {1, 2, 3, 4})
        if (mnn == nb_of_shells(sh)) nshell = sh;
    if (!nshell) return no("neighbour count must be 8, 14, 26 or 50 (bcc shells 1..4)");
    const int NB = nb_of_shells(nshell);
    double tab[4][2][2];
    bool have[4][2][2] = {};
    std::vector<std::pair<int, int>> es(NB), gs(NB);
    for (int i = 0; i < N; ++i) {
        int ih = a->aham[i] - 1;
        if (a->nlistsize[ih] != NB) return no("every site must have the full shell set");
        int b = i & 1, cell = i >> 1;
        int x = cell % L1, y = (cell / L1) % L2, z = cell / (L1 * L2);
        for (int q = 0; q < NB; ++q) {
            St e = stencil_entry(b, q);
            int xx = ((x + e.dx) % L1 + L1) % L1, yy = ((y + e.dy) % L2 + L2) % L2, zz = ((z + e.dz) % L3 + L3) % L3;
            es[q] = {e.bj + 2 * (xx + L1 * (yy + L2 * zz)), e.sh};
            gs[q] = {a->nlist[q + (size_t)mnn * i] - 1, q};
        }
        std::sort(es.begin(), es.end());
        std::sort(gs.begin(), gs.end());
        for (int q = 0; q < NB; ++q) {
            if (es[q].first != gs[q].first) return no("neighbour list does not match the bcc shell stencil");
            if (q + 1 < NB && es[q].first == es[q + 1].first) return no("periodic images coincide (lattice too small)");
            int sh = es[q].second - 1;
            double cval = a->ncoup[gs[q].second + (size_t)mnn * ih];
            int tj = sp[es[q].first];
            if (!have[sh][sp[i]][tj]) {
                tab[sh][sp[i]][tj] = cval;
                have[sh][sp[i]][tj] = true;
            } else if (tab[sh][sp[i]][tj] != cval) {
                return no("couplings are not a function of (shell, species_i, species_j)");
            }
        }
    }
    StructuredFast *f = new (std::nothrow) StructuredFast();
    if (!f) return UPPASD_GPU_ENOMEM;
    f->nshell = nshell;
    f->master = c->precision;
    if (const char *kv = getenv("UPPASD_STENCIL_KERNEL")) f->kernel = atoi(kv);
    SParams &p = f->p;
    p.L1 = L1;
    p.L2 = L2;
    p.L3 = L3;
    p.nens = M;
    p.k0 = 0;
    p.kn = M;
    p.nsite = N;
    p.P1 = pitch1(L1);
    p.P2 = p.P1 * (L2 + 4);
    // cubic lattices of the sizes below get kernels with compile-time pitches
    f->lc = 0;
    if (L1 == L2 && L2 == L3)
        for (int lc : {6, 64, 100})
            if (L1 == lc && (nshell == 2 || nshell == 4)) f->lc = lc;
    p.pbox = (long long)p.P2 * (L3 + 4);
    for (int sh = 0; sh < 4; ++sh)
        for (int ti = 0; ti < 2; ++ti) {
            double v[2];
            for (int tj = 0; tj < 2; ++tj)
                v[tj] = (sh < nshell && have[sh][ti][tj]) ? tab[sh][ti][tj] * (mom[tj] > 0 ? mom[tj] : 0.0) : 0.0;
            if (!(sh < nshell && have[sh][ti][1])) v[1] = v[0];
            p.cA[sh][ti] = (float)v[0];
            p.cD[sh][ti] = (float)(v[1] - v[0]);
        }
    f->lam = a->lambda1_array[0];
    f->temp = a->temp_array[0];
    f->delta_t = c->delta_t;
    f->temprescale = c->temprescale;
    for (int ti = 0; ti < 2; ++ti) f->mom[ti] = mom[ti] > 0 ? mom[ti] : 1.0;
    structured_coefficients(s, f);
    for (int q = 0; q < 3; ++q) p.ext[q] = (float)a->external_field[q];
    p.seed = c->gpu_rng_seed;
    p.d_step = s.llg.d_step;
    const size_t n = (size_t)N * M;
    const size_t nbox = (size_t)p.pbox * 2 * M;
    cudaError_t e = cudaSuccess;
    auto al = [&](void **q, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(q, bytes);
        if (e == cudaSuccess) s.bytes_allocated += bytes;
    };
    al((void **)&p.mt, nbox * sizeof(float4));
    al((void **)&p.mp, nbox * sizeof(float4));
    if (e == cudaSuccess) e = cudaMemset(p.mt, 0, nbox * sizeof(float4));
    if (e == cudaSuccess) e = cudaMemset(p.mp, 0, nbox * sizeof(float4));
    al((void **)&p.b2x, n * sizeof(float));
    al((void **)&p.b2y, n * sizeof(float));
    al((void **)&p.b2z, n * sizeof(float));
    if (f->master == 1) {
        al((void **)&p.mx, n * sizeof(double));
        al((void **)&p.my, n * sizeof(double));
        al((void **)&p.mz, n * sizeof(double));
    } else {
        al((void **)&p.lox, n * sizeof(float));
        al((void **)&p.loy, n * sizeof(float));
        al((void **)&p.loz, n * sizeof(float));
    }
    al((void **)&f->species, N);
    al((void **)&p.err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(p.err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(f->species, sp.data(), N, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        fast_free(f);
        set_error(std::string("structured_init: ") + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? UPPASD_GPU_ENOMEM : UPPASD_GPU_ECUDA;
    }
    const int bx = L1 <= 256 ? L1 : 256;
    if (L1 > 256) {
        fast_free(f);
        return no("n1 must be <= 256 for the structured kernels");
    }
    const int by = std::max(1, 256 / bx);
    f->block = dim3(bx, by, 1);
    f->grid = dim3((unsigned)(((L2 + by - 1) / by) * L3), 2, (unsigned)M);
    if (f->lc == 0 && f->kernel != 0) f->kernel = 0;  // runtime pitches: one sublattice per thread
    if (f->kernel >= 2) {
        const int tx = f->lc == 100 ? TmaTile<100>::TX : (f->lc == 64 ? TmaTile<64>::TX : TmaTile<6>::TX);
        const int ty = f->lc == 100 ? TmaTile<100>::TY : (f->lc == 64 ? TmaTile<64>::TY : TmaTile<6>::TY);
        int rc = mirror_map(&f->map_mt, f, p.mt, tx, ty);
        if (!rc) rc = mirror_map(&f->map_mp, f, p.mp, tx, ty);
        if (rc) {
            fast_free(f);
            return rc;
        }
    }
    s.fast = f;
    return UPPASD_GPU_OK;
}

// The same conversions between the caller's (3, natom, mensemble) layout (a device copy
// of it) and the structured state, for the host blocks (abi.cu:sd_run_io): the generic
// e / eM are left as they are (the structured state owns the spins until the next sync).
// from_aos_structured writes what to_structured writes for e = aos; to_aos_structured
// writes what from_structured and soa_to_aos give for e (full = 0) or eM (full = 1).
__global__ void from_aos_structured(SParams p, const double *aos, const int8_t *species, int master) {
    long long t = (long long)p.k0 * p.nsite + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.nsite * (p.k0 + p.kn)) return;
    int k = (int)(t / p.nsite);
    long long i = t - (long long)k * p.nsite;
    int b = (int)(i & 1);
    long long cell = i >> 1;
    int x = (int)(cell % p.L1), y = (int)((cell / p.L1) % p.L2), z = (int)(cell / ((long long)p.L1 * p.L2));
    long long u = uidx(p, k, b, x, y, z);
    double e0 = aos[3 * t], e1 = aos[3 * t + 1], e2 = aos[3 * t + 2];
    float w = species ? (float)species[i] : 0.f;
    float h0 = (float)e0, h1 = (float)e1, h2 = (float)e2;
    store_mirror(p, p.mt, k, b, x, y, z, make_float4(h0, h1, h2, w));
    if (master == 1) {
        p.mx[u] = e0;
        p.my[u] = e1;
        p.mz[u] = e2;
    } else {
        p.lox[u] = (float)(e0 - (double)h0);
        p.loy[u] = (float)(e1 - (double)h1);
        p.loz[u] = (float)(e2 - (double)h2);
    }
}

__global__ void to_aos_structured(SParams p, double *aos, const double *mmom, int master, int full) {
    long long t = (long long)p.k0 * p.nsite + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.nsite * (p.k0 + p.kn)) return;
    int k = (int)(t / p.nsite);
    long long i = t - (long long)k * p.nsite;
    int b = (int)(i & 1);
    long long cell = i >> 1;
    int x = (int)(cell % p.L1), y = (int)((cell / p.L1) % p.L2), z = (int)(cell / ((long long)p.L1 * p.L2));
    long long u = uidx(p, k, b, x, y, z);
    double e0, e1, e2;
    if (master == 1) {
        e0 = p.mx[u];
        e1 = p.my[u];
        e2 = p.mz[u];
    } else {
        float4 h = p.mt[pidx(p, k, b, x, y, z)];
        e0 = (double)h.x + (double)p.lox[u];
        e1 = (double)h.y + (double)p.loy[u];
        e2 = (double)h.z + (double)p.loz[u];
    }
    if (full) {
        const double m = mmom[t];
        e0 *= m;
        e1 *= m;
        e2 *= m;
    }
    aos[3 * t] = e0;
    aos[3 * t + 1] = e1;
    aos[3 * t + 2] = e2;
}

int structured_load_state(Sim &s) {
    StructuredFast *f = s.fast;
    long long total = f->p.nsite * f->p.kn;
    to_structured<<<(unsigned)((total + 255) / 256), 256, 0, s.stream>>>(f->p, s.e.x, s.e.y, s.e.z, f->species,
                                                                         f->master);
    UPPASD_CUDA_TRY(cudaGetLastError());
    return UPPASD_GPU_OK;
}

int structured_sync_state(Sim &s) {
    square_mirror_stale(s);
    StructuredFast *f = s.fast;
    {
        // a plane wait of the staged kernels that ran past its limit (reset once reported)
        int herr = 0;
        UPPASD_CUDA_TRY(cudaMemcpyAsync(&herr, f->p.err, sizeof(int), cudaMemcpyDeviceToHost, s.stream));
        UPPASD_CUDA_TRY(cudaStreamSynchronize(s.stream));
        if (herr) {
            UPPASD_CUDA_TRY(cudaMemsetAsync(f->p.err, 0, sizeof(int), s.stream));
            set_error("structured LLG: a TMA plane wait ran past its limit");
            return UPPASD_GPU_ESTATE;
        }
    }
    long long total = f->p.nsite * f->p.kn;
    from_structured<<<(unsigned)((total + 255) / 256), 256, 0, s.stream>>>(f->p, s.e.x, s.e.y, s.e.z, s.eM.x, s.eM.y,
                                                                           s.eM.z, s.llg.mmom, f->master);
    UPPASD_CUDA_TRY(cudaGetLastError());
    return UPPASD_GPU_OK;
}

template <int NSH, int LC, int V, int KIND, int MASTER>
static void launch_tma_kernel(StructuredFast *f, cudaStream_t st) {
    using T = TmaTile<LC, V>;
    using G = TileGeom<T::TX, T::TY, T::R>;
    auto kern = stencil_tma<NSH, LC, T::TX, T::TY, T::ZC, T::NZ, T::R, T::MINB, KIND, MASTER>;
    static bool attr = false;  // per instantiation
    if (!attr) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::kSmem) != cudaSuccess)
            return;  // the launch below then fails and the step reports it
        attr = true;
    }
    const int ntx = (LC + T::TX - 1) / T::TX, nty = (LC + T::TY - 1) / T::TY;
    const dim3 g((unsigned)(ntx * nty * (LC / T::ZC)), 1, (unsigned)f->p.kn);
    kern<<<g, T::TX * T::TY, G::kSmem, st>>>(KIND == 0 ? f->map_mt : f->map_mp, f->p, ntx, nty);
}

template <int NSH, int LC, int V>
static void launch_tma_v(StructuredFast *f, cudaStream_t st, int phase) {
    if (phase & 1) launch_tma_kernel<NSH, LC, V, 0, 2>(f, st);
    if (phase & 2) {
        if (f->master == 1) launch_tma_kernel<NSH, LC, V, 1, 1>(f, st);
        else launch_tma_kernel<NSH, LC, V, 1, 2>(f, st);
    }
}

// Two planes per iteration (V = 0) is the faster schedule with the double-single master
// (fewer shared-memory reads per site); with the FP64 master the FP64 pipe holds the
// corrector back and the extra warps of V = 1 hide more of it (both measured on the
// 100^3 alloy).  kernel 3 forces V = 1 throughout.
template <int NSH, int LC>
static void launch_tma(StructuredFast *f, cudaStream_t st, int phase) {
    if constexpr (LC != 0) {
        if (f->kernel == 3 || f->master == 1) launch_tma_v<NSH, LC, 1>(f, st, phase);
        else launch_tma_v<NSH, LC, 0>(f, st, phase);
    }
}

template <int NSH, int LC>
static void launch_lc(StructuredFast *f, cudaStream_t st, int phase) {
    if constexpr (LC != 0) {
        // compiled cubic sizes: NZ sites per thread stacked in z (NZ divides LC).  Two
        // sites per thread in both kernels: on the 100^3 alloy NZ = 4 in the predictor
        // was 5-10 % slower (a larger unrolled body stalls on instruction fetch) and
        // NZ = 1 in either kernel 5-10 % slower (fewer shared neighbour loads).
        constexpr int NZP = 2;
        constexpr int NZC = 2;
        const unsigned nyt = (unsigned)((f->p.L2 + f->block.y - 1) / f->block.y);
        if (f->kernel >= 2) {
            launch_tma<NSH, LC>(f, st, phase);
            return;
        }
        if (f->kernel == 1) {
            const dim3 g(nyt * (LC / 2), 1, (unsigned)f->p.kn);
            if (phase & 1) stencil_cells<NSH, 2, LC, 0, 2><<<g, f->block, 0, st>>>(f->p);
            if (phase & 2) {
                if (f->master == 1) stencil_cells<NSH, 2, LC, 1, 1><<<g, f->block, 0, st>>>(f->p);
                else stencil_cells<NSH, 2, LC, 1, 2><<<g, f->block, 0, st>>>(f->p);
            }
            return;
        }
        if (phase & 1)
            stencil_zblock<NSH, NZP, LC, 0, 2>
                <<<dim3(nyt * (LC / NZP), 2, (unsigned)f->p.kn), f->block, 0, st>>>(f->p);
        if (phase & 2) {
            const dim3 g(nyt * (LC / NZC), 2, (unsigned)f->p.kn);
            if (f->master == 1) stencil_zblock<NSH, NZC, LC, 1, 1><<<g, f->block, 0, st>>>(f->p);
            else stencil_zblock<NSH, NZC, LC, 1, 2><<<g, f->block, 0, st>>>(f->p);
        }
        return;
    }
    const dim3 g(f->grid.x, f->grid.y, (unsigned)f->p.kn);
    if (phase & 1) stencil_predict<NSH, LC><<<g, f->block, 0, st>>>(f->p);
    if (phase & 2) {
        if (f->master == 1) stencil_correct<NSH, 1, LC><<<g, f->block, 0, st>>>(f->p);
        else stencil_correct<NSH, 2, LC><<<g, f->block, 0, st>>>(f->p);
    }
}

template <int NSH>
static void launch(StructuredFast *f, cudaStream_t st, int phase) {
    if (NSH == 2 || NSH == 4) {
        switch (f->lc) {
        case 6: launch_lc<NSH, 6>(f, st, phase); return;
        case 64: launch_lc<NSH, 64>(f, st, phase); return;
        case 100: launch_lc<NSH, 100>(f, st, phase); return;
        default: break;
        }
    }
    launch_lc<NSH, 0>(f, st, phase);
}

// One step (or half step) of the ensembles k0 .. k0 + kn - 1 on stream st; the launch
// parameters are taken by value, so the whole-range defaults are restored at once.
static int step_range(Sim &s, int64_t step_offset, int phase, int k0, int kn, cudaStream_t st) {
    StructuredFast *f = s.fast;
    f->p.step_off = step_offset;
    f->p.d_step = s.llg.d_step;
    f->p.k0 = k0;
    f->p.kn = kn;
    switch (f->nshell) {
    case 1: launch<1>(f, st, phase); break;
    case 2: launch<2>(f, st, phase); break;
    case 3: launch<3>(f, st, phase); break;
    default: launch<4>(f, st, phase); break;
    }
    f->p.k0 = 0;
    f->p.kn = f->p.nens;
    UPPASD_CUDA_TRY(cudaGetLastError());
    return UPPASD_GPU_OK;
}

int structured_step(Sim &s, int64_t step_offset, int phase) {
    return step_range(s, step_offset, phase, 0, s.fast->p.nens, s.stream);
}

// The ensemble-range forms the pipelined host run (abi.cu:sd_run_io) issues per group:
// conversions from and to the caller's layout and nsteps steps, all on stream st.  The
// steps read the device step counter, which the caller advances once all groups are done.
// aos: the device copy of the caller's (3, natom, mensemble) array
int structured_load_range(Sim &s, const double *aos, int k0, int kn, cudaStream_t st) {
    StructuredFast *f = s.fast;
    SParams p = f->p;
    p.k0 = k0;
    p.kn = kn;
    const long long total = p.nsite * kn;
    from_aos_structured<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(p, aos, f->species, f->master);
    UPPASD_CUDA_TRY(cudaGetLastError());
    return UPPASD_GPU_OK;
}

int structured_steps_range(Sim &s, int64_t nsteps, int k0, int kn, cudaStream_t st) {
    for (int64_t j = 0; j < nsteps; ++j) {
        int rc = step_range(s, j, 3, k0, kn, st);
        if (rc) return rc;
    }
    return UPPASD_GPU_OK;
}

// the unit (full = 0) or full (full = 1) moments into aos, the caller's layout
int structured_store_range(Sim &s, double *aos, int full, int k0, int kn, cudaStream_t st) {
    StructuredFast *f = s.fast;
    SParams p = f->p;
    p.k0 = k0;
    p.kn = kn;
    const long long total = p.nsite * kn;
    to_aos_structured<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(p, aos, s.llg.mmom, f->master, full);
    UPPASD_CUDA_TRY(cudaGetLastError());
    return UPPASD_GPU_OK;
}

// the plane-wait flag of the staged kernels, read after a pipelined run (reset once reported)
int structured_check_flag(Sim &s) {
    StructuredFast *f = s.fast;
    int herr = 0;
    UPPASD_CUDA_TRY(cudaMemcpyAsync(&herr, f->p.err, sizeof(int), cudaMemcpyDeviceToHost, s.stream));
    UPPASD_CUDA_TRY(cudaStreamSynchronize(s.stream));
    if (herr) {
        UPPASD_CUDA_TRY(cudaMemsetAsync(f->p.err, 0, sizeof(int), s.stream));
        set_error("structured LLG: a TMA plane wait ran past its limit");
        return UPPASD_GPU_ESTATE;
    }
    return UPPASD_GPU_OK;
}

}  // namespace uppasd
