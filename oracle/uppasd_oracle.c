/*
 * uppasd_oracle.c -- CPU restatement of UppASD's spin-update hot path.
 *
 * TEST INFRASTRUCTURE ONLY (correctness oracle and CPU baseline).  Nothing in
 * the product library links or calls this file.  Each routine cites the
 * reference Fortran it restates (paths relative to the UppASD source tree).
 * Expressions keep the Fortran left-to-right evaluation order; the file is
 * compiled with -ffp-contract=off.
 */
#include "uppasd_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Fortran default-real literals promoted to double (single precision first). */
#define F32(x) ((double)(float)(x))
/* Parameters/parameters.f90:12  dbl_tolerance=1e-14 (a REAL(4) literal) */
static const double DBL_TOLERANCE = (double)(float)1e-14;

double orc_gama = ORC_GAMA_SI, orc_kbolt = ORC_KBOLT_SI, orc_mub = ORC_MUB_SI, orc_mry = ORC_MRY_SI;
void orc_set_units(double gama, double kbolt, double mub, double mry) {
    orc_gama = gama;
    orc_kbolt = kbolt;
    orc_mub = mub;
    orc_mry = mry;
}

static int g_threads = 0;
void orc_set_threads(int n) { g_threads = n; }
int orc_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* Fortran index helpers (0-based storage of 1-based arrays) */
#define V3(a, c, i, k, N) ((a)[(c) + 3 * ((int64_t)(i) + (int64_t)(N) * (k))])
#define M2(a, i, k, N) ((a)[(int64_t)(i) + (int64_t)(N) * (k)])

/* ===================================================================== */
/* mtprng (RNG/mtprng.f90)                                               */
/* ===================================================================== */
#define MT_N 624
#define MT_M 397
static const uint64_t MT_MAG1 = (uint64_t)(int64_t)-1727483681LL;   /* mtprng.f90:200 */
static const uint64_t MT_UPPER = 2147483648ULL;                     /* :203 */
static const uint64_t MT_LOWER = 2147483647ULL;                     /* :204 */
static const uint64_t MT_TB = (uint64_t)(int64_t)-1658038656LL;     /* :207 */
static const uint64_t MT_TC = (uint64_t)(int64_t)-272236544LL;      /* :208 */
static const uint64_t MASK32 = 4294967295ULL;

/* mtprng_init (mtprng.f90:118-138) */
void orc_mt_init(orc_mt_state *s, int32_t seed) {
    s->mt[0] = (uint64_t)(int64_t)seed;
    for (int i = 1; i < MT_N; ++i) {
        uint64_t p = s->mt[i - 1];
        s->mt[i] = MASK32 & (1812433253ULL * (p ^ (p >> 30)) + (uint64_t)i);
    }
    s->mti = MT_N;
}

/* mtprng_rand64 (mtprng.f90:191-246): INT64 words, signed mag01; the upper
 * bits of a word can be set and leak into the first tempering shift. */
uint64_t orc_mt_rand64(orc_mt_state *s) {
    uint64_t r;
    if (s->mti >= MT_N) {
        if (s->mti == -1) orc_mt_init(s, 4357);
        int kk;
        for (kk = 0; kk <= MT_N - MT_M - 1; ++kk) {
            r = (s->mt[kk] & MT_UPPER) | (s->mt[kk + 1] & MT_LOWER);
            s->mt[kk] = (s->mt[kk + MT_M] ^ (r >> 1)) ^ ((r & 1ULL) ? MT_MAG1 : 0ULL);
        }
        for (kk = MT_N - MT_M; kk <= MT_N - 2; ++kk) {
            r = (s->mt[kk] & MT_UPPER) | (s->mt[kk + 1] & MT_LOWER);
            s->mt[kk] = (s->mt[kk + (MT_M - MT_N)] ^ (r >> 1)) ^ ((r & 1ULL) ? MT_MAG1 : 0ULL);
        }
        r = (s->mt[MT_N - 1] & MT_UPPER) | (s->mt[0] & MT_LOWER);
        s->mt[MT_N - 1] = (s->mt[MT_M - 1] ^ (r >> 1)) ^ ((r & 1ULL) ? MT_MAG1 : 0ULL);
        s->mti = 0;
    }
    r = s->mt[s->mti];
    s->mti += 1;
    r = r ^ (r >> 11);
    r = MASK32 & (r ^ ((r << 7) & MT_TB));
    r = MASK32 & (r ^ ((r << 15) & MT_TC));
    r = r ^ (r >> 18);
    return r;
}

/* mtprng_rand (mtprng.f90:250-270) */
int32_t orc_mt_rand(orc_mt_state *s) {
    int64_t x = (int64_t)orc_mt_rand64(s);
    if (x > 2147483647LL) return (int32_t)(x - 4294967296LL);
    return (int32_t)x;
}

/* mtprng_rand_real1 / real2 (mtprng.f90:292-325) */
double orc_mt_real1(orc_mt_state *s) {
    static const double factor = 1.0 / 4294967295.0;
    return (double)(int64_t)orc_mt_rand64(s) * factor;
}
double orc_mt_real2(orc_mt_state *s) {
    static const double factor = 1.0 / 4294967296.0;
    return (double)(int64_t)orc_mt_rand64(s) * factor;
}

/* ===================================================================== */
/* ziggurat (RNG/randomnumbers.f90:330-565)                              */
/* ===================================================================== */
static const double ZIG_R = 3.442620;   /* randomnumbers.f90:41 */

/* r4_nor_setup (randomnumbers.f90:441-509) */
void orc_zig_setup(orc_zig *g, int32_t seed) {
    const double m1 = 2147483648.0;
    const double vn = 9.91256303526217e-03;
    double dn = 3.442619855899, tn = 3.442619855899;
    orc_mt_init(&g->z, seed);
    double q = vn / exp(-0.5 * dn * dn);
    g->kn[0] = (int32_t)((dn / q) * m1);
    g->kn[1] = 0;
    g->wn[0] = q / m1;
    g->wn[127] = dn / m1;
    g->fn[0] = 1.0;
    g->fn[127] = exp(-0.5 * dn * dn);
    for (int i = 127; i >= 2; --i) {
        dn = sqrt(-2.0 * log(vn / dn + exp(-0.5 * dn * dn)));
        g->kn[i] = (int32_t)((dn / tn) * m1);   /* kn(i+1) */
        tn = dn;
        g->fn[i - 1] = exp(-0.5 * dn * dn);     /* fn(i) */
        g->wn[i - 1] = dn / m1;                 /* wn(i) */
    }
}

static inline int32_t iabs32(int32_t h) { return h == INT32_MIN ? INT32_MIN : (h < 0 ? -h : h); }

/* r4_nor (randomnumbers.f90:330-438).  log(real(u)) is a single-precision log. */
double orc_zig_nor(orc_zig *g) {
    int32_t hz = orc_mt_rand(&g->z);
    int32_t iz = hz & 127;
    double value, x, y;
    if (iabs32(hz) < g->kn[iz]) {
        value = (double)hz * g->wn[iz];
    } else {
        for (;;) {
            if (iz == 0) {
                for (;;) {
                    x = -0.2904764 * (double)logf((float)orc_mt_real1(&g->z));
                    y = (double)(-logf((float)orc_mt_real1(&g->z)));
                    if (x * x <= y + y) break;
                }
                if (hz <= 0) value = -ZIG_R - x;
                else value = ZIG_R + x;
                break;
            }
            x = (double)hz * g->wn[iz];
            if (g->fn[iz] + orc_mt_real1(&g->z) * (g->fn[iz - 1] - g->fn[iz]) < exp(-0.5 * x * x)) {
                value = x;
                break;
            }
            hz = orc_mt_rand(&g->z);
            iz = hz & 127;
            if (iabs32(hz) < g->kn[iz]) {
                value = (double)hz * g->wn[iz];
                break;
            }
        }
    }
    return value;
}

/* fill_rngarray (randomnumbers.f90:548-565) with rng_trans==1 */
void orc_zig_fill(orc_zig *g, double *out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = orc_zig_nor(g);
}

/* ===================================================================== */
/* Philox4x32-10 (Salmon et al., SC'11): the GPU path's counter RNG       */
/* ===================================================================== */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static void philox_words(uint64_t seed, int64_t site, int32_t ens, int64_t step, uint32_t stream,
                         uint32_t w[4]) {
    uint32_t ctr[4], key[2];
    ctr[0] = (uint32_t)site;
    ctr[1] = (uint32_t)ens;
    ctr[2] = (uint32_t)step;
    ctr[3] = ((uint32_t)((uint64_t)step >> 32) & 0xFFFFu) | (stream << 16);
    key[0] = (uint32_t)seed;
    key[1] = (uint32_t)(seed >> 32);
    orc_philox4x32_10(ctr, key, w);
}

static inline double u32_to_open01(uint32_t x) { return ((double)x + 0.5) * 2.3283064365386963e-10; }

void orc_philox_uniform4(uint64_t seed, int64_t site, int32_t ens, int64_t step, uint32_t stream,
                         double u[4]) {
    uint32_t w[4];
    philox_words(seed, site, ens, step, stream, w);
    for (int i = 0; i < 4; ++i) u[i] = u32_to_open01(w[i]);
}

void orc_philox_normal3(uint64_t seed, int64_t site, int32_t ens, int64_t step, uint32_t stream,
                        double z[3]) {
    double u[4];
    orc_philox_uniform4(seed, site, ens, step, stream, u);
    const double twopi = 2.0 * ORC_PI;
    double r0 = sqrt(-2.0 * log(u[0]));
    double t0 = twopi * u[1];
    double r1 = sqrt(-2.0 * log(u[2]));
    double t1 = twopi * u[3];
    z[0] = r0 * cos(t0);
    z[1] = r0 * sin(t0);
    z[2] = r1 * cos(t1);
}

/* ===================================================================== */
/* Effective field (Hamiltonian/hamiltonianactions.f90)                  */
/* ===================================================================== */
/* uniaxial_anisotropy_field (:842-879) and cubic_anisotropy_field (:883-919),
 * combined by taniso as effective_field_full does (:225-239). */
static void site_field_aniso(const orc_ham *h, const double *emomM, int i, int k, double bs[3], double bq[3]) {
    const int N = h->natom;
    if (h->do_aniso == 1) {
        int ta = h->taniso[i];
        const double *e = &h->eaniso[3 * (int64_t)i];
        const double *ka = &h->kaniso[2 * (int64_t)i];
        double m1 = V3(emomM, 0, i, k, N), m2 = V3(emomM, 1, i, k, N), m3 = V3(emomM, 2, i, k, N);
        if (ta == 1 || ta == 7) {
            double tt1 = m1 * e[0] + m2 * e[1] + m3 * e[2];
            double tt2 = ka[0] + 2.0 * ka[1] * (1.0 - tt1 * tt1);
            double tt3 = 2.0 * tt1 * tt2;
            bs[0] = bs[0] - tt3 * e[0];
            bs[1] = bs[1] - tt3 * e[1];
            bs[2] = bs[2] - tt3 * e[2];
        }
        if (ta == 2 || ta == 7) {
            double t[3];
            t[0] = 2.0 * ka[0] * m1 * (m2 * m2 + m3 * m3) + 2.0 * ka[1] * m1 * (m2 * m2 * (m3 * m3));
            t[1] = 2.0 * ka[0] * m2 * (m3 * m3 + m1 * m1) + 2.0 * ka[1] * m2 * (m3 * m3 * (m1 * m1));
            t[2] = 2.0 * ka[0] * m3 * (m1 * m1 + m2 * m2) + 2.0 * ka[1] * m3 * (m1 * m1 * (m2 * m2));
            if (ta == 2) {
                bs[0] = bs[0] + t[0]; bs[1] = bs[1] + t[1]; bs[2] = bs[2] + t[2];
            } else {
                double sbv = h->sb[i];
                bq[0] = bq[0] + t[0] * sbv; bq[1] = bq[1] + t[1] * sbv; bq[2] = bq[2] + t[2] * sbv;
            }
        }
    }
}

/* tensor_field (:499-542): field(a) = field(a) + J(a,1) m1 + J(a,2) m2 + J(a,3) m3 over
 * the exchange list.  The reference indexes j_tens by the atom i there although the
 * array is allocated per Hamiltonian index (hamiltoniandata.f90:138) and the Monte
 * Carlo energy (montecarlo_common.f90:502-510) indexes it by aham(i); the two agree
 * whenever the Hamiltonian is not reduced, and aham(i) is used here. */
static void tensor_exchange(const orc_ham *h, const double *emomM, int i, int ih, int k, double b[3]) {
    const int N = h->natom;
    int nn = h->nlistsize[ih];
    for (int j = 0; j < nn; ++j) {
        int jn = h->nlist[j + (int64_t)h->max_no_neigh * i] - 1;
        const double *J = &h->j_tens[9 * (j + (int64_t)h->max_no_neigh * ih)];  /* J(a,b) = J[a + 3b] */
        double m1 = V3(emomM, 0, jn, k, N), m2 = V3(emomM, 1, jn, k, N), m3 = V3(emomM, 2, jn, k, N);
        for (int a = 0; a < 3; ++a) b[a] = b[a] + J[a] * m1 + J[a + 3] * m2 + J[a + 6] * m3;
    }
}

/* heisenberg_field (:431-466) or tensor_field (:499-542), dzyaloshinskii_moriya_field
 * (:546-580), uniaxial_anisotropy_field (:842-879), cubic_anisotropy_field (:883-919);
 * accumulation order of effective_field_full (:187-246). */
static void site_field(const orc_ham *h, const double *emomM, int i, int k, double bs[3], double bq[3]) {
    const int N = h->natom;
    bs[0] = bs[1] = bs[2] = 0.0;
    bq[0] = bq[1] = bq[2] = 0.0;
    int ih = h->aham[i] - 1;
    int nn = h->do_jtensor == 1 ? 0 : h->nlistsize[ih];
    if (h->do_jtensor == 1) tensor_exchange(h, emomM, i, ih, k, bs);
    for (int j = 0; j < nn; ++j) {
        int jn = h->nlist[j + (int64_t)h->max_no_neigh * i] - 1;
        double c = h->ncoup[j + (int64_t)h->max_no_neigh * ih];
        bs[0] = bs[0] + c * V3(emomM, 0, jn, k, N);
        bs[1] = bs[1] + c * V3(emomM, 1, jn, k, N);
        bs[2] = bs[2] + c * V3(emomM, 2, jn, k, N);
    }
    if (h->do_dm == 1) {
        int nd = h->dmlistsize[ih];
        for (int j = 0; j < nd; ++j) {
            int jn = h->dmlist[j + (int64_t)h->max_no_dmneigh * i] - 1;
            const double *d = &h->dm_vect[3 * (j + (int64_t)h->max_no_dmneigh * ih)];
            double m1 = V3(emomM, 0, jn, k, N), m2 = V3(emomM, 1, jn, k, N), m3 = V3(emomM, 2, jn, k, N);
            bs[0] = bs[0] + d[2] * m2 - d[1] * m3;
            bs[1] = bs[1] + d[0] * m3 - d[2] * m1;
            bs[2] = bs[2] + d[1] * m1 - d[0] * m2;
        }
    }
    site_field_aniso(h, emomM, i, k, bs, bq);
}

/* dipoleMatrix (Hamiltonian/dipolecommon.f90:51-84): Q(nu, mu) for the separation Rij
 * in units of alat; zero below R^2 = 1e-9 */
static void dipole_matrix(double alat, const double Rij[3], double Q[3][3]) {
    const double tol = 1e-9;
    const double fac = (1.0e-7 / (alat * alat * alat)) * ORC_MUB;
    const double R2 = Rij[0] * Rij[0] + Rij[1] * Rij[1] + Rij[2] * Rij[2];
    const double Rm5 = pow(R2, -2.5) * fac;
    for (int mu = 0; mu < 3; ++mu)
        for (int nu = 0; nu < 3; ++nu) Q[nu][mu] = 0.0;
    if (R2 > tol) {
        for (int mu = 0; mu < 3; ++mu) {
            for (int nu = 0; nu < 3; ++nu) Q[nu][mu] = 3.0 * Rm5 * Rij[nu] * Rij[mu];
            Q[mu][mu] = Q[mu][mu] - Rm5 * R2;
        }
    }
}

static void dipole_coord(const orc_ham *h, int i, double r[3]) {
    const int NA = h->dip_na, N1 = h->dip_n1, N2 = h->dip_n2;
    const int I0 = i % NA, c = i / NA;
    const int I1 = c % N1, I2 = (c / N1) % N2, I3 = c / (N1 * N2);
    for (int q = 0; q < 3; ++q)
        r[q] = I1 * h->dip_cell[q] + I2 * h->dip_cell[3 + q] + I3 * h->dip_cell[6 + q] + h->dip_bas[3 * I0 + q];
}

/* dipolar_field (dipolemanager.f90:223-243) for every (atom, ensemble), Qdip set up as
 * setup_qdip does (dipolecommon.f90:114-159): Qdip(:,:,j,i) = dipoleMatrix(r_i - r_j),
 * zero on the diagonal */
/* dipolar_field of one site (dipolemanager.f90:223-243) */
static void dipole_field_site(const orc_ham *h, const double *emomM, int i, int k, double f[3]) {
    const int N = h->natom;
    double ri[3];
    dipole_coord(h, i, ri);
    f[0] = f[1] = f[2] = 0.0;
    for (int j = 0; j < N; ++j) {
        double rj[3], R[3], Q[3][3];
        dipole_coord(h, j, rj);
        for (int q = 0; q < 3; ++q) R[q] = ri[q] - rj[q];
        dipole_matrix(h->dip_alat, R, Q);
        if (j == i)
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) Q[a][b] = 0.0;
        const double m1 = V3(emomM, 0, j, k, N), m2 = V3(emomM, 1, j, k, N), m3 = V3(emomM, 2, j, k, N);
        for (int nu = 0; nu < 3; ++nu) f[nu] = f[nu] + Q[0][nu] * m1 + Q[1][nu] * m2 + Q[2][nu] * m3;
    }
}

void orc_dipole_field(const orc_ham *h, const double *emomM, double *out) {
    const int N = h->natom, M = h->mensemble;
#pragma omp parallel for collapse(2) schedule(static) num_threads(orc_get_threads())
    for (int k = 0; k < M; ++k)
        for (int i = 0; i < N; ++i) {
            double f[3];
            dipole_field_site(h, emomM, i, k, f);
            for (int nu = 0; nu < 3; ++nu) V3(out, nu, i, k, N) = f[nu];
        }
}

double orc_effective_field(const orc_ham *h, const double *emomM, double *beff) {
    const int N = h->natom, M = h->mensemble;
    double energy = 0.0;
    if (h->do_dip) {
        /* the dipolar field first, with its energy (dipolemanager.f90:147-158) */
        orc_dipole_field(h, emomM, h->dip_work);
        for (int k = 0; k < M; ++k)
            for (int i = 0; i < N; ++i)
                energy = energy - 0.5 * (V3(h->dip_work, 0, i, k, N) * V3(emomM, 0, i, k, N) +
                                         V3(h->dip_work, 1, i, k, N) * V3(emomM, 1, i, k, N) +
                                         V3(h->dip_work, 2, i, k, N) * V3(emomM, 2, i, k, N));
    }
#pragma omp parallel for collapse(2) schedule(static) reduction(+ : energy) num_threads(orc_get_threads())
    for (int k = 0; k < M; ++k) {
        for (int i = 0; i < N; ++i) {
            double bs[3], bq[3];
            site_field(h, emomM, i, k, bs, bq);
            double tf[3];
            for (int c = 0; c < 3; ++c) {
                double ext = V3(h->extfield, c, i, k, N);
                double b2 = bq[c] + ext + 0.0;   /* beff2 = beff_q + external + time_external */
                const double bd = h->do_dip ? V3(h->dip_work, c, i, k, N) : 0.0;
                V3(beff, c, i, k, N) = bd + bs[c] + b2;
                tf[c] = 0.5 * (bs[c] + 2.0 * bq[c] + 2.0 * ext + 0.0);
            }
            energy = energy - V3(emomM, 0, i, k, N) * tf[0] - V3(emomM, 1, i, k, N) * tf[1] -
                     V3(emomM, 2, i, k, N) * tf[2];
        }
    }
    return energy * ORC_MUB / ORC_MRY;
}

/* effective_field_single (hamiltonianactions.f90:253-371): with dipoles on, the dipolar
 * field in dip_work (the caller evaluates it for the moments the field is wanted for)
 * comes first */
void orc_effective_field_single(const orc_ham *h, const double *emomM, int i, int k, double out[3]) {
    const int N = h->natom;
    double bs[3], bq[3];
    site_field(h, emomM, i, k, bs, bq);
    for (int c = 0; c < 3; ++c) {
        double b2 = bq[c] + V3(h->extfield, c, i, k, N) + 0.0;
        const double bd = h->do_dip ? V3(h->dip_work, c, i, k, N) : 0.0;
        out[c] = bd + bs[c] + b2;
    }
}

/* ===================================================================== */
/* Noise                                                                  */
/* ===================================================================== */
void orc_llg_draw_normals(const orc_llg *p, int natom, int mensemble, double *out) {
    int64_t n3 = 3 * (int64_t)natom * mensemble;
    switch (p->noise_mode) {
    case ORC_NOISE_ZIGGURAT: orc_zig_fill(p->zig, out, n3); break;
    case ORC_NOISE_ARRAY: memcpy(out, p->noise, sizeof(double) * n3); break;
    case ORC_NOISE_PHILOX:
#pragma omp parallel for collapse(2) schedule(static) num_threads(orc_get_threads())
        for (int k = 0; k < mensemble; ++k)
            for (int i = 0; i < natom; ++i) {
                double z[3];
                orc_philox_normal3(p->seed, i, k, p->step, 0u, z);
                V3(out, 0, i, k, natom) = z[0];
                V3(out, 1, i, k, natom) = z[1];
                V3(out, 2, i, k, natom) = z[2];
            }
        break;
    default:
        memset(out, 0, sizeof(double) * n3);
    }
}

/* rannum (randomnumbers.f90:625-771), llg==1 branch, compensate_drift==0 */
static void rannum(const orc_llg *p, int N, int M, const double *mmom, double *ranv) {
    orc_llg_draw_normals(p, N, M, ranv);
#pragma omp parallel for collapse(2) schedule(static) num_threads(orc_get_threads())
    for (int j = 0; j < M; ++j)
        for (int i = 0; i < N; ++i) {
            double lam = p->lambda1[i];
            double Dk = (((lam / (1.0 + lam * lam)) * ORC_KBOLT) / ORC_GAMA / ORC_MUB) * (ORC_GAMA / p->bn);
            double mmomi = 1.0 / M2(mmom, i, j, N);
            double D = Dk * mmomi * p->temp[i] * p->temprescale;
            double sigma = sqrt(2.00 * D);
            V3(ranv, 0, i, j, N) = V3(ranv, 0, i, j, N) * sigma;
            V3(ranv, 1, i, j, N) = V3(ranv, 1, i, j, N) * sigma;
            V3(ranv, 2, i, j, N) = V3(ranv, 2, i, j, N) * sigma;
        }
}

/* ===================================================================== */
/* Solvers                                                                */
/* ===================================================================== */
/* depondt_evolve_first (Evolution/depondt.f90:50-193) */
static void depondt_first(const orc_llg *p, int N, int M, orc_state *s) {
    orc_llg_draw_normals(p, N, M, s->ranv); /* btherm */
#pragma omp parallel for collapse(2) schedule(static) num_threads(orc_get_threads())
    for (int k = 0; k < M; ++k)
        for (int i = 0; i < N; ++i) {
            double lam = p->lambda1[i];
            double Dp = (2.0 * lam * ORC_KBOLT) / (p->delta_t * ORC_GAMA * ORC_MUB);
            double sigma = sqrt(Dp * p->temprescale * p->temp[i] / M2(s->mmom, i, k, N));
            double bth[3], bloc[3], bdup[3], e[3];
            for (int c = 0; c < 3; ++c) {
                bth[c] = V3(s->ranv, c, i, k, N) * sigma;
                V3(s->ranv, c, i, k, N) = bth[c];
                bloc[c] = V3(s->beff, c, i, k, N) + bth[c];
                e[c] = V3(s->emom, c, i, k, N);
            }
            bdup[0] = 0.0 + bloc[0] + lam * e[1] * bloc[2] - lam * e[2] * bloc[1];
            bdup[1] = 0.0 + bloc[1] + lam * e[2] * bloc[0] - lam * e[0] * bloc[2];
            bdup[2] = 0.0 + bloc[2] + lam * e[0] * bloc[1] - lam * e[1] * bloc[0];
            double lldamp = 1.0 / (1.0 + lam * lam);
            double Bnorm = bdup[0] * bdup[0] + bdup[1] * bdup[1] + bdup[2] * bdup[2];
            Bnorm = sqrt(Bnorm) + 1.0e-15;
            double hx = bdup[0] / Bnorm, hy = bdup[1] / Bnorm, hz = bdup[2] / Bnorm;
            double v = Bnorm * p->delta_t * ORC_GAMA * lldamp;
            double cosv = cos(v), sinv = sin(v), u = 1.0 - cosv;
            double mr[3];
            mr[0] = hx * hx * u * e[0] + cosv * e[0] + hx * hy * u * e[1] - hz * sinv * e[1] + hx * hz * u * e[2] + hy * sinv * e[2];
            mr[1] = hy * hx * u * e[0] + hz * sinv * e[0] + hy * hy * u * e[1] + cosv * e[1] + hy * hz * u * e[2] - hx * sinv * e[2];
            mr[2] = hx * hz * u * e[0] - hy * sinv * e[0] + hz * hy * u * e[1] + hx * sinv * e[1] + hz * hz * u * e[2] + cosv * e[2];
            double mm = M2(s->mmom, i, k, N);
            for (int c = 0; c < 3; ++c) {
                V3(s->emom2, c, i, k, N) = e[c];
                V3(s->emomM, c, i, k, N) = mr[c] * mm;
                V3(s->emom, c, i, k, N) = mr[c];
                V3(s->b2eff, c, i, k, N) = bdup[c];
            }
        }
}

/* depondt_evolve_second (Evolution/depondt.f90:203-333) */
static void depondt_second(const orc_llg *p, int N, int M, orc_state *s) {
#pragma omp parallel for collapse(2) schedule(static) num_threads(orc_get_threads())
    for (int k = 0; k < M; ++k)
        for (int i = 0; i < N; ++i) {
            double lam = p->lambda1[i];
            double bloc[3], bdup[3], e[3];
            for (int c = 0; c < 3; ++c) {
                bloc[c] = V3(s->beff, c, i, k, N) + V3(s->ranv, c, i, k, N);
                e[c] = V3(s->emom, c, i, k, N);
            }
            bdup[0] = 0.0 + bloc[0] + lam * e[1] * bloc[2] - lam * e[2] * bloc[1];
            bdup[1] = 0.0 + bloc[1] + lam * e[2] * bloc[0] - lam * e[0] * bloc[2];
            bdup[2] = 0.0 + bloc[2] + lam * e[0] * bloc[1] - lam * e[1] * bloc[0];
            for (int c = 0; c < 3; ++c) {
                bdup[c] = 0.50 * bdup[c] + 0.50 * V3(s->b2eff, c, i, k, N);
                e[c] = V3(s->emom2, c, i, k, N);
                V3(s->emom, c, i, k, N) = e[c];
            }
            double lldamp = 1.0 / (1.0 + lam * lam);
            double Bnorm = bdup[0] * bdup[0] + bdup[1] * bdup[1] + bdup[2] * bdup[2];
            Bnorm = sqrt(Bnorm) + 1.0e-15;
            double hx = bdup[0] / Bnorm, hy = bdup[1] / Bnorm, hz = bdup[2] / Bnorm;
            double v = Bnorm * p->delta_t * ORC_GAMA * lldamp;
            double cosv = cos(v), sinv = sin(v), u = 1.0 - cosv;
            double mr[3];
            mr[0] = hx * hx * u * e[0] + cosv * e[0] + hx * hy * u * e[1] - hz * sinv * e[1] + hx * hz * u * e[2] + hy * sinv * e[2];
            mr[1] = hy * hx * u * e[0] + hz * sinv * e[0] + hy * hy * u * e[1] + cosv * e[1] + hy * hz * u * e[2] - hx * sinv * e[2];
            mr[2] = hx * hz * u * e[0] - hy * sinv * e[0] + hz * hy * u * e[1] + hx * sinv * e[1] + hz * hz * u * e[2] + cosv * e[2];
            for (int c = 0; c < 3; ++c) V3(s->emom2, c, i, k, N) = mr[c];
        }
}

/* Cayley step shared by smodeulermpt / modeulermpf (Evolution/midpoint.f90:153-167, 303-315) */
static inline void cayley(const double A[3], const double e[3], double et[3], double *detAi) {
    *detAi = 1.0 / (1.0 + (A[0] * A[0] + A[1] * A[1] + A[2] * A[2]));
    double a2[3];
    a2[0] = e[0] + e[1] * A[2] - e[2] * A[1];
    a2[1] = e[1] + e[2] * A[0] - e[0] * A[2];
    a2[2] = e[2] + e[0] * A[1] - e[1] * A[0];
    et[0] = a2[0] * (1.0 + A[0] * A[0]) + a2[1] * (A[0] * A[1] + A[2]) + a2[2] * (A[0] * A[2] - A[1]);
    et[1] = a2[0] * (A[1] * A[0] - A[2]) + a2[1] * (1.0 + A[1] * A[1]) + a2[2] * (A[1] * A[2] + A[0]);
    et[2] = a2[0] * (A[2] * A[0] + A[1]) + a2[1] * (A[2] * A[1] - A[0]) + a2[2] * (1.0 + A[2] * A[2]);
}

static inline void midpoint_A(double lam, double dtg, double sqrtdtg, const double e[3], const double b[3],
                              const double r[3], double A[3]) {
    double a1[3], s1[3];
    a1[0] = -0.0 - b[0] - lam * (e[1] * b[2] - e[2] * b[1]);
    a1[1] = -0.0 - b[1] - lam * (e[2] * b[0] - e[0] * b[2]);
    a1[2] = -0.0 - b[2] - lam * (e[0] * b[1] - e[1] * b[0]);
    s1[0] = -r[0] - lam * (e[1] * r[2] - e[2] * r[1]);
    s1[1] = -r[1] - lam * (e[2] * r[0] - e[0] * r[2]);
    s1[2] = -r[2] - lam * (e[0] * r[1] - e[1] * r[0]);
    for (int c = 0; c < 3; ++c) A[c] = 0.5 * dtg * a1[c] + 0.5 * sqrtdtg * s1[c];
}

/* smodeulermpt (Evolution/midpoint.f90:34-181) */
static void midpoint_first(const orc_llg *p, int N, int M, orc_state *s) {
#pragma omp parallel for collapse(2) schedule(static) num_threads(orc_get_threads())
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < M; ++j) {
            double lam = p->lambda1[i];
            double lldamp = 1.0 / (1.0 + lam * lam);
            double dt = p->delta_t * p->bn * ORC_GAMA * lldamp;
            double sqrtdt = sqrt(dt);
            double dtg = dt * p->landeg[i], sqrtdtg = sqrtdt * p->landeg[i];
            double e[3], b[3], r[3], A[3], et[3], detAi;
            for (int c = 0; c < 3; ++c) {
                e[c] = V3(s->emom, c, i, j, N);
                b[c] = V3(s->beff, c, i, j, N);
                r[c] = V3(s->ranv, c, i, j, N);
            }
            midpoint_A(lam, dtg, sqrtdtg, e, b, r, A);
            cayley(A, e, et, &detAi);
            double mm = M2(s->mmom, i, j, N);
            for (int c = 0; c < 3; ++c) {
                double v = 0.5 * (e[c] + et[c] * detAi);
                V3(s->emom2, c, i, j, N) = v;
                V3(s->emomM, c, i, j, N) = v * mm;
            }
        }
}

/* modeulermpf (Evolution/midpoint.f90:188-323) */
static void midpoint_second(const orc_llg *p, int N, int M, orc_state *s) {
#pragma omp parallel for collapse(2) schedule(static) num_threads(orc_get_threads())
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < M; ++j) {
            double lam = p->lambda1[i];
            double lldamp = 1.0 / (1.0 + lam * lam);
            double dt = p->delta_t * p->bn * ORC_GAMA * lldamp;
            double sqrtdt = sqrt(dt);
            double dtg = dt * p->landeg[i], sqrtdtg = sqrtdt * p->landeg[i];
            double etp[3], e[3], b[3], r[3], A[3], et[3], detAi;
            for (int c = 0; c < 3; ++c) {
                etp[c] = V3(s->emom2, c, i, j, N);
                e[c] = V3(s->emom, c, i, j, N);
                b[c] = V3(s->beff, c, i, j, N);
                r[c] = V3(s->ranv, c, i, j, N);
            }
            midpoint_A(lam, dtg, sqrtdtg, etp, b, r, A);
            cayley(A, e, et, &detAi);
            for (int c = 0; c < 3; ++c) V3(s->emom2, c, i, j, N) = et[c] * detAi;
        }
}

/* evolve4p / heun4p (Evolution/heun_proper.f90:28-161, 261-369) */
static void heun_first(const orc_llg *p, int N, int M, orc_state *s) {
    orc_llg_draw_normals(p, N, M, s->ranv);
    double dt = p->delta_t * ORC_GAMA;
    for (int k = 0; k < M; ++k)
        for (int i = 0; i < N; ++i) {
            double lam = p->lambda1[i];
            double Dk = lam / (1.0 + lam * lam) * ORC_KBOLT / ORC_MUB;
            double D = Dk * (1.0 / M2(s->mmom, i, k, N)) * p->temp[i] * p->temprescale;
            double sigma = sqrt(dt * 2.0 * D);
            for (int c = 0; c < 3; ++c) V3(s->ranv, c, i, k, N) = V3(s->ranv, c, i, k, N) * sigma;
        }
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < M; ++k) {
            double lam = p->lambda1[i], g = p->landeg[i];
            double e1x = V3(s->emom2, 0, i, k, N), e1y = V3(s->emom2, 1, i, k, N), e1z = V3(s->emom2, 2, i, k, N);
            double hesx = V3(s->beff, 0, i, k, N), hesy = V3(s->beff, 1, i, k, N), hesz = V3(s->beff, 2, i, k, N);
            for (int c = 0; c < 3; ++c) V3(s->b2eff, c, i, k, N) = V3(s->beff, c, i, k, N);
            double lldamp = 1.0 / (1.0 + lam * lam);
            double dtg = dt * g * lldamp;
            double dwx = V3(s->ranv, 0, i, k, N) * g, dwy = V3(s->ranv, 1, i, k, N) * g, dwz = V3(s->ranv, 2, i, k, N) * g;
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
            double mm = M2(s->mmom, i, k, N);
            V3(s->emom, 0, i, k, N) = etx; V3(s->emom, 1, i, k, N) = ety; V3(s->emom, 2, i, k, N) = etz;
            V3(s->emomM, 0, i, k, N) = etx * mm; V3(s->emomM, 1, i, k, N) = ety * mm; V3(s->emomM, 2, i, k, N) = etz * mm;
        }
}

/* evolve4f / heun4f (Evolution/heun_proper.f90:168-254, 376-530), including the
 * reference's b1zz expression (lambda - e1z*e1z - lambda) as written. */
static void heun_second(const orc_llg *p, int N, int M, orc_state *s) {
    double dt = p->delta_t * ORC_GAMA;
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < M; ++k) {
            double lam = p->lambda1[i], g = p->landeg[i];
            double lldamp = 1.0 / (1.0 + lam * lam);
            double dtg = dt * g * lldamp;
            double dwx = V3(s->ranv, 0, i, k, N) * g, dwy = V3(s->ranv, 1, i, k, N) * g, dwz = V3(s->ranv, 2, i, k, N) * g;
            double e1x = V3(s->emom, 0, i, k, N), e1y = V3(s->emom, 1, i, k, N), e1z = V3(s->emom, 2, i, k, N);
            double e2x = V3(s->emom2, 0, i, k, N), e2y = V3(s->emom2, 1, i, k, N), e2z = V3(s->emom2, 2, i, k, N);
            double h1esx = V3(s->beff, 0, i, k, N), h1esy = V3(s->beff, 1, i, k, N), h1esz = V3(s->beff, 2, i, k, N);
            double h1px = lam * h1esx, h1py = lam * h1esy, h1pz = lam * h1esz;
            double h2esx = V3(s->b2eff, 0, i, k, N), h2esy = V3(s->b2eff, 1, i, k, N), h2esz = V3(s->b2eff, 2, i, k, N);
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
            V3(s->emom2, 0, i, k, N) = nx * etot;
            V3(s->emom2, 1, i, k, N) = ny * etot;
            V3(s->emom2, 2, i, k, N) = nz * etot;
        }
}

/* Fixed-point iteration shared by sibt / sibf (Evolution/sphmidpoint.f90:176-231, 396-431) */
static inline void sib_fixed_point(const double e1[3], const double a1[3], const double s1[3], double dtg,
                                   double sqrtdtg, double efp[3]) {
    const double epsilona = F32(1e-12);
    double efp0[3] = {e1[0], e1[1], e1[2]};
    for (int k = 1; k <= 100; ++k) {
        double f1[3], fd[3], fs[3];
        for (int c = 0; c < 3; ++c) {
            f1[c] = 0.5 * (e1[c] + efp0[c]);
            fd[c] = dtg * f1[c];
            fs[c] = sqrtdtg * f1[c];
        }
        efp[0] = e1[0] + fd[1] * a1[2] - fd[2] * a1[1] + fs[1] * s1[2] - fs[2] * s1[1];
        efp[1] = e1[1] + fd[2] * a1[0] - fd[0] * a1[2] + fs[2] * s1[0] - fs[0] * s1[2];
        efp[2] = e1[2] + fd[0] * a1[1] - fd[1] * a1[0] + fs[0] * s1[1] - fs[1] * s1[0];
        double dx = sqrt((efp0[0] - efp[0]) * (efp0[0] - efp[0]));
        double dy = sqrt((efp0[1] - efp[1]) * (efp0[1] - efp[1]));
        double dz = sqrt((efp0[2] - efp[2]) * (efp0[2] - efp[2]));
        if (dx < epsilona && dy < epsilona && dz < epsilona) break;
        efp0[0] = efp[0]; efp0[1] = efp[1]; efp0[2] = efp[2];
    }
}

static inline void sib_a1s1(double lam, const double e[3], const double b[3], const double f[3],
                            double a1[3], double s1[3]) {
    a1[0] = -b[0] - lam * (e[1] * b[2] - e[2] * b[1]);
    a1[1] = -b[1] - lam * (e[2] * b[0] - e[0] * b[2]);
    a1[2] = -b[2] - lam * (e[0] * b[1] - e[1] * b[0]);
    s1[0] = -f[0] - lam * (e[1] * f[2] - e[2] * f[1]);
    s1[1] = -f[1] - lam * (e[2] * f[0] - e[0] * f[2]);
    s1[2] = -f[2] - lam * (e[0] * f[1] - e[1] * f[0]);
}

/* sibt (Evolution/sphmidpoint.f90:36-243) */
static void sib_first(const orc_llg *p, int N, int M, orc_state *s) {
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int64_t ij = 0; ij < (int64_t)N * M; ++ij) {
        int i = (int)(ij % N), j = (int)(ij / N);
        double lam = p->lambda1[i];
        double lldamp = 1.0 / (1.0 + lam * lam);
        double dt = p->delta_t * p->bn * ORC_GAMA * lldamp;
        double dtg = dt * p->landeg[i], sqrtdtg = sqrt(dt) * p->landeg[i];
        double e1[3], b[3], f[3], a1[3], s1[3], efp[3];
        for (int c = 0; c < 3; ++c) {
            e1[c] = V3(s->emom, c, i, j, N);
            b[c] = V3(s->beff, c, i, j, N);
            f[c] = V3(s->ranv, c, i, j, N);
        }
        sib_a1s1(lam, e1, b, f, a1, s1);
        sib_fixed_point(e1, a1, s1, dtg, sqrtdtg, efp);
        double mm = M2(s->mmom, i, j, N);
        for (int c = 0; c < 3; ++c) {
            double v = 0.5 * (e1[c] + efp[c]);
            V3(s->emom2, c, i, j, N) = v;
            V3(s->emomM, c, i, j, N) = v * mm;
        }
    }
}

/* sibf (Evolution/sphmidpoint.f90:250-477) */
static void sib_second(const orc_llg *p, int N, int M, orc_state *s) {
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int64_t ij = 0; ij < (int64_t)N * M; ++ij) {
        int i = (int)(ij % N), j = (int)(ij / N);
        double lam = p->lambda1[i];
        double lldamp = 1.0 / (1.0 + lam * lam);
        double dt = p->delta_t * p->bn * ORC_GAMA * lldamp;
        double dtg = dt * p->landeg[i], sqrtdtg = sqrt(dt) * p->landeg[i];
        double e1[3], etp[3], b[3], f[3], a1[3], s1[3], efp[3];
        for (int c = 0; c < 3; ++c) {
            e1[c] = V3(s->emom, c, i, j, N);
            etp[c] = V3(s->emom2, c, i, j, N);
            b[c] = V3(s->beff, c, i, j, N);
            f[c] = V3(s->ranv, c, i, j, N);
        }
        sib_a1s1(lam, etp, b, f, a1, s1);
        sib_fixed_point(e1, a1, s1, dtg, sqrtdtg, efp);
        for (int c = 0; c < 3; ++c) V3(s->emom2, c, i, j, N) = efp[c];
    }
}

/* Fixed-point iteration of sispht / sisphf (Evolution/sphmidpoint.f90:485-923, SDEalgh 7):
 * SIB's with the midpoint direction normalised, u = (e1 + efp0) / |e1 + efp0|.  efp is the
 * last iterate, efp0 the one before it when the tolerance ended the loop (else the last). */
static inline void sisph_fixed_point(const double e1[3], const double a1[3], const double s1[3], double dtg,
                                     double sqrtdtg, double efp[3], double efp0[3]) {
    const double epsilona = F32(1e-12);
    efp0[0] = e1[0]; efp0[1] = e1[1]; efp0[2] = e1[2];
    for (int k = 1; k <= 100; ++k) {
        double unorm = sqrt((e1[0] + efp0[0]) * (e1[0] + efp0[0]) + (e1[1] + efp0[1]) * (e1[1] + efp0[1]) +
                            (e1[2] + efp0[2]) * (e1[2] + efp0[2]));
        double fd[3], fs[3];
        for (int c = 0; c < 3; ++c) {
            double u = (e1[c] + efp0[c]) / unorm;
            fd[c] = dtg * u;
            fs[c] = sqrtdtg * u;
        }
        efp[0] = e1[0] + fd[1] * a1[2] - fd[2] * a1[1] + fs[1] * s1[2] - fs[2] * s1[1];
        efp[1] = e1[1] + fd[2] * a1[0] - fd[0] * a1[2] + fs[2] * s1[0] - fs[0] * s1[2];
        efp[2] = e1[2] + fd[0] * a1[1] - fd[1] * a1[0] + fs[0] * s1[1] - fs[1] * s1[0];
        double dx = sqrt((efp0[0] - efp[0]) * (efp0[0] - efp[0]));
        double dy = sqrt((efp0[1] - efp[1]) * (efp0[1] - efp[1]));
        double dz = sqrt((efp0[2] - efp[2]) * (efp0[2] - efp[2]));
        if (dx < epsilona && dy < epsilona && dz < epsilona) break;
        efp0[0] = efp[0]; efp0[1] = efp[1]; efp0[2] = efp[2];
    }
}

/* sispht (Evolution/sphmidpoint.f90:485-713): emom2 = the normalised midpoint of e1 and the
 * iterate the loop continues from */
static void sisph_first(const orc_llg *p, int N, int M, orc_state *s) {
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int64_t ij = 0; ij < (int64_t)N * M; ++ij) {
        int i = (int)(ij % N), j = (int)(ij / N);
        double lam = p->lambda1[i];
        double lldamp = 1.0 / (1.0 + lam * lam);
        double dt = p->delta_t * p->bn * ORC_GAMA * lldamp;
        double dtg = dt * p->landeg[i], sqrtdtg = sqrt(dt) * p->landeg[i];
        double e1[3], b[3], f[3], a1[3], s1[3], efp[3], efp0[3];
        for (int c = 0; c < 3; ++c) {
            e1[c] = V3(s->emom, c, i, j, N);
            b[c] = V3(s->beff, c, i, j, N);
            f[c] = V3(s->ranv, c, i, j, N);
        }
        sib_a1s1(lam, e1, b, f, a1, s1);
        sisph_fixed_point(e1, a1, s1, dtg, sqrtdtg, efp, efp0);
        double unorm = sqrt((e1[0] + efp0[0]) * (e1[0] + efp0[0]) + (e1[1] + efp0[1]) * (e1[1] + efp0[1]) +
                            (e1[2] + efp0[2]) * (e1[2] + efp0[2]));
        double mm = M2(s->mmom, i, j, N);
        for (int c = 0; c < 3; ++c) {
            double v = (e1[c] + efp0[c]) / unorm;
            V3(s->emom2, c, i, j, N) = v;
            V3(s->emomM, c, i, j, N) = v * mm;
        }
    }
}

/* sisphf (Evolution/sphmidpoint.f90:721-923): a1, s1 at the midpoint, emom2 = last iterate */
static void sisph_second(const orc_llg *p, int N, int M, orc_state *s) {
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int64_t ij = 0; ij < (int64_t)N * M; ++ij) {
        int i = (int)(ij % N), j = (int)(ij / N);
        double lam = p->lambda1[i];
        double lldamp = 1.0 / (1.0 + lam * lam);
        double dt = p->delta_t * p->bn * ORC_GAMA * lldamp;
        double dtg = dt * p->landeg[i], sqrtdtg = sqrt(dt) * p->landeg[i];
        double e1[3], etp[3], b[3], f[3], a1[3], s1[3], efp[3], efp0[3];
        for (int c = 0; c < 3; ++c) {
            e1[c] = V3(s->emom, c, i, j, N);
            etp[c] = V3(s->emom2, c, i, j, N);
            b[c] = V3(s->beff, c, i, j, N);
            f[c] = V3(s->ranv, c, i, j, N);
        }
        sib_a1s1(lam, etp, b, f, a1, s1);
        sisph_fixed_point(e1, a1, s1, dtg, sqrtdtg, efp, efp0);
        for (int c = 0; c < 3; ++c) V3(s->emom2, c, i, j, N) = efp[c];
    }
}

/* llgiheun (Evolution/llgi.f90:178-278): one implicit step of the inertial LLG,
 * m_new = A^-1 B with A = I + beta [e1]x, from m(t) = e1, m(t - dt) = et and the
 * field h; no Lande factor and no 1/(1 + lambda^2), as there. */
static void llgiheun(double lam, double delta_t, double relaxtime, const double et[3], const double e1[3],
                     const double h[3], double out[3]) {
    double alfa = lam;
    double beta = -alfa * (1.0 + relaxtime / delta_t);
    double zeta = -alfa * (relaxtime / delta_t);
    double dtg = -delta_t * ORC_GAMA;
    double A12 = -beta * e1[2], A13 = beta * e1[1];
    double A21 = beta * e1[2], A23 = -beta * e1[0];
    double A31 = -beta * e1[1], A32 = beta * e1[0];
    double det = 1.0 - A23 * A32 - A12 * A21 - A13 * A31;
    det = 1.0 / det;
    double I11 = (1.0 - A32 * A23) * det, I12 = (A13 * A32 - A12) * det, I13 = (A12 * A23 - A13) * det;
    double I21 = (A23 * A31 - A21) * det, I22 = (1.0 - A31 * A13) * det, I23 = (A13 * A21 - A23) * det;
    double I31 = (A21 * A32 - A31) * det, I32 = (A12 * A31 - A32) * det, I33 = (1.0 - A21 * A12) * det;
    double B1 = e1[0] + dtg * (e1[1] * h[2] - e1[2] * h[1]) + zeta * (e1[2] * et[1] - e1[1] * et[2]);
    double B2 = e1[1] + dtg * (e1[2] * h[0] - e1[0] * h[2]) + zeta * (e1[0] * et[2] - e1[2] * et[0]);
    double B3 = e1[2] + dtg * (e1[0] * h[1] - e1[1] * h[0]) + zeta * (e1[1] * et[0] - e1[0] * et[1]);
    out[0] = I11 * B1 + I12 * B2 + I13 * B3;
    out[1] = I21 * B1 + I22 * B2 + I23 * B3;
    out[2] = I31 * B1 + I32 * B2 + I33 * B3;
}

/* llgi_evolve_first (Evolution/llgi.f90:18-66): thermfield (:120-159, the Depondt
 * noise amplitude), bdup = beff + btherm, predictor from (m(t - dt), m(t)). */
static void llgi_first(const orc_llg *p, int N, int M, orc_state *s) {
    orc_llg_draw_normals(p, N, M, s->ranv); /* btherm */
#pragma omp parallel for collapse(2) schedule(static) num_threads(orc_get_threads())
    for (int k = 0; k < M; ++k)
        for (int i = 0; i < N; ++i) {
            double lam = p->lambda1[i];
            double Dp = (2.0 * lam * ORC_KBOLT) / (p->delta_t * ORC_GAMA * ORC_MUB);
            double sigma = sqrt(Dp * p->temprescale * p->temp[i] / M2(s->mmom, i, k, N));
            double bdup[3], et[3], e1[3], mt[3];
            for (int c = 0; c < 3; ++c) {
                double bth = V3(s->ranv, c, i, k, N) * sigma;
                V3(s->ranv, c, i, k, N) = bth;
                bdup[c] = V3(s->beff, c, i, k, N) + bth;
                et[c] = V3(s->mpast, c, i, k, N);
                e1[c] = V3(s->emom2, c, i, k, N);
            }
            llgiheun(lam, p->delta_t, p->relaxtime, et, e1, bdup, mt);
            double mm = M2(s->mmom, i, k, N);
            for (int c = 0; c < 3; ++c) {
                V3(s->emom, c, i, k, N) = mt[c];
                V3(s->emomM, c, i, k, N) = mt[c] * mm;
                V3(s->b2eff, c, i, k, N) = bdup[c];
            }
        }
}

/* llgi_evolve_second (Evolution/llgi.f90:68-118): bdup = (beff + btherm)/2 + b2eff/2,
 * corrector from (m(t - dt), m(t)), then m(t) becomes the new m(t - dt) and the
 * normalised corrector the new m(t).  norm2 is evaluated as sqrt(x^2 + y^2 + z^2);
 * compilers differ in how they evaluate it, by the last bit. */
static void llgi_second(const orc_llg *p, int N, int M, orc_state *s) {
#pragma omp parallel for collapse(2) schedule(static) num_threads(orc_get_threads())
    for (int k = 0; k < M; ++k)
        for (int i = 0; i < N; ++i) {
            double bdup[3], et[3], e1[3], mt[3];
            for (int c = 0; c < 3; ++c) {
                bdup[c] = 0.5 * (V3(s->beff, c, i, k, N) + V3(s->ranv, c, i, k, N)) +
                          0.5 * V3(s->b2eff, c, i, k, N);
                et[c] = V3(s->mpast, c, i, k, N);
                e1[c] = V3(s->emom2, c, i, k, N);
                V3(s->mpast, c, i, k, N) = e1[c];
            }
            llgiheun(p->lambda1[i], p->delta_t, p->relaxtime, et, e1, bdup, mt);
            double etot = 1.0 / sqrt(mt[0] * mt[0] + mt[1] * mt[1] + mt[2] * mt[2]);
            for (int c = 0; c < 3; ++c) {
                V3(s->emom, c, i, k, N) = e1[c];
                V3(s->emom2, c, i, k, N) = mt[c] * etot;
            }
        }
}

/* copym (Evolution/updatemoments.f90:48-99), initexc /= 'I', mompar = 0 */
static void copym(int N, int M, orc_state *s) {
#pragma omp parallel for collapse(2) schedule(static) num_threads(orc_get_threads())
    for (int j = 0; j < M; ++j)
        for (int i = 0; i < N; ++i) {
            double mm = M2(s->mmom, i, j, N);
            for (int c = 0; c < 3; ++c) {
                double v = V3(s->emom2, c, i, j, N);
                V3(s->emom, c, i, j, N) = v;
                V3(s->emomM, c, i, j, N) = v * mm;
            }
        }
}

static int min_lambda_gt(const orc_llg *p, int N, double tol) {
    for (int i = 0; i < N; ++i)
        if (!(p->lambda1[i] > tol)) return 0;
    return 1;
}

/* perp = 'Y' (Evolution/evolution.f90:104-112 and :327-335): the field loses its
 * component along emom, whatever emom holds at that point of the step. */
static void perp_project(int N, int M, orc_state *s) {
#pragma omp parallel for collapse(2) schedule(static) num_threads(orc_get_threads())
    for (int k = 0; k < M; ++k)
        for (int i = 0; i < N; ++i) {
            double b[3], e[3];
            for (int c = 0; c < 3; ++c) {
                b[c] = V3(s->beff, c, i, k, N);
                e[c] = V3(s->emom, c, i, k, N);
            }
            double d = b[0] * e[0] + b[1] * e[1] + b[2] * e[2];
            for (int c = 0; c < 3; ++c) V3(s->beff, c, i, k, N) = b[c] - e[c] * d;
        }
}

/* sd_mphase step body (sd_driver.f90:657-767) with evolve_first / evolve_second
 * dispatch (Evolution/evolution.f90:38-406). */
int orc_sd_step(const orc_ham *h, const orc_llg *p, orc_state *s) {
    const int N = h->natom, M = h->mensemble;
    orc_effective_field(h, s->emomM, s->beff);
    if (p->perp) perp_project(N, M, s);
    switch (p->sdealgh) {
    case 1:
    case 6:
    case 7:
        if (min_lambda_gt(p, N, 1e-12)) rannum(p, N, M, s->mmom, s->ranv);
        else memset(s->ranv, 0, sizeof(double) * 3 * (size_t)N * M);
        if (p->sdealgh == 1) midpoint_first(p, N, M, s);
        else if (p->sdealgh == 6) sib_first(p, N, M, s);
        else sisph_first(p, N, M, s);
        break;
    case 4: heun_first(p, N, M, s); break;
    case 5: depondt_first(p, N, M, s); break;
    case 11:
        if (!s->mpast) return -1;
        llgi_first(p, N, M, s);
        break;
    default: return -1;
    }
    orc_effective_field(h, s->emomM, s->beff);
    if (p->perp) perp_project(N, M, s);
    switch (p->sdealgh) {
    case 1: midpoint_second(p, N, M, s); break;
    case 6: sib_second(p, N, M, s); break;
    case 7: sisph_second(p, N, M, s); break;
    case 4: heun_second(p, N, M, s); break;
    case 5: depondt_second(p, N, M, s); break;
    case 11: llgi_second(p, N, M, s); break;
    }
    copym(N, M, s);
    return 0;
}

/* magninit initmag==1 (System/magnetizationinit.f90:141-170) */
void orc_initmag_random(orc_mt_state *c, int natom, int mensemble, const double *mmom, double *emom,
                        double *emomM) {
    for (int i = 0; i < natom; ++i) {
        double rn[3];
        for (int t = 0; t < 3; ++t) rn[t] = orc_mt_real2(c);
        double x = 2.0 * (rn[0] - 0.50), y = 2.0 * (rn[1] - 0.50), z = 2.0 * (rn[2] - 0.50);
        while (x * x + y * y + z * z > 1.0) {
            for (int t = 0; t < 3; ++t) rn[t] = orc_mt_real2(c);
            x = 1.0 * (rn[0] - 0.50);
            y = 1.0 * (rn[1] - 0.50);
            z = 1.0 * (rn[2] - 0.50);
        }
        double u[3];
        u[0] = x / sqrt(x * x + y * y + z * z);
        u[1] = y / sqrt(x * x + y * y + z * z);
        u[2] = z / sqrt(x * x + y * y + z * z);
        for (int j = 0; j < mensemble; ++j)
            for (int t = 0; t < 3; ++t) {
                V3(emom, t, i, j, natom) = u[t];
                V3(emomM, t, i, j, natom) = u[t] * M2(mmom, i, j, natom);
            }
    }
}

/* ===================================================================== */
/* Monte Carlo (MonteCarlo/montecarlo.f90, montecarlo_common.f90)       */
/* ===================================================================== */
void orc_choose_random_atom_x(orc_mt_state *c, int natom, int32_t *iflip_a) {
    for (int i = 0; i < natom; ++i) iflip_a[i] = i + 1;
    double *dshift = (double *)malloc(sizeof(double) * natom);
    for (int i = 0; i < natom; ++i) dshift[i] = orc_mt_real2(c);
    for (int i = 0; i < natom; ++i) {
        int ishift = (int)(dshift[i] * natom);
        int t = iflip_a[i];
        int dst = ishift % natom;
        iflip_a[i] = iflip_a[dst];
        iflip_a[dst] = t;
    }
    free(dshift);
}

/* choose_random_flip (montecarlo_common.f90:25-79) */
static void choose_random_flip(const double e[3], double delta, const double rn[3], const double gn[3],
                               double newmom[3]) {
    int ftype = (int)floor(3.0 * rn[0]);
    if (ftype == 0) {
        double phi = rn[1] * 2.0 * ORC_PI;
        double theta = acos(1.0 - 2.0 * rn[2]);
        newmom[0] = sin(theta) * cos(phi);
        newmom[1] = sin(theta) * sin(phi);
        newmom[2] = cos(theta);
    } else if (ftype == 1) {
        double g[3] = {gn[0] * delta, gn[1] * delta, gn[2] * delta};
        double l = sqrt((e[0] + g[0]) * (e[0] + g[0]) + (e[1] + g[1]) * (e[1] + g[1]) + (e[2] + g[2]) * (e[2] + g[2]));
        for (int c = 0; c < 3; ++c) newmom[c] = (e[c] + g[c]) / l;
    } else {
        for (int c = 0; c < 3; ++c) newmom[c] = -e[c];
    }
}

/* calculate_energy (montecarlo_common.f90:431-865): exchange, uniaxial/cubic
 * anisotropy, DMI (with the reference's emom/emomM mix in the current-energy
 * term) and Zeeman.  Returns de = mub*(e_t - e_c). */
static double calculate_energy(const orc_ham *h, const double *emomM, const double *emom, const double *mmom,
                               int iflip, const double newmom[3], const double ext[3], int k) {
    const int N = h->natom;
    double e_c = 0.0, e_t = 0.0, tm[3];
    double mm = M2(mmom, iflip, k, N);
    for (int c = 0; c < 3; ++c) tm[c] = newmom[c] * mm;
    int ih = h->aham[iflip] - 1;
    const double *mi = &V3(emomM, 0, iflip, k, N);
    const double *ei = &V3(emom, 0, iflip, k, N);
    if (h->do_jtensor == 1) {  /* montecarlo_common.f90:502-510 */
        double bt[3] = {0.0, 0.0, 0.0};
        tensor_exchange(h, emomM, iflip, ih, k, bt);
        e_c = e_c - (mi[0] * bt[0] + mi[1] * bt[1] + mi[2] * bt[2]);
        e_t = e_t - (tm[0] * bt[0] + tm[1] * bt[1] + tm[2] * bt[2]);
    }
    int nn = h->do_jtensor == 1 ? 0 : h->nlistsize[ih];
    for (int j = 0; j < nn; ++j) {
        int jn = h->nlist[j + (int64_t)h->max_no_neigh * iflip] - 1;
        double c = h->ncoup[j + (int64_t)h->max_no_neigh * ih];
        const double *mj = &V3(emomM, 0, jn, k, N);
        e_c = e_c - c * (mi[0] * mj[0] + mi[1] * mj[1] + mi[2] * mj[2]);
        e_t = e_t - c * (tm[0] * mj[0] + tm[1] * mj[1] + tm[2] * mj[2]);
    }
    if (h->do_aniso == 1) {
        int ta = h->taniso[iflip];
        const double *ea = &h->eaniso[3 * (int64_t)iflip];
        const double *ka = &h->kaniso[2 * (int64_t)iflip];
        if (ta == 1) {
            double tta = mi[0] * ea[0] + mi[1] * ea[1] + mi[2] * ea[2];
            double ttb = tm[0] * ea[0] + tm[1] * ea[1] + tm[2] * ea[2];
            e_c = e_c + ka[0] * (tta * tta) + ka[1] * (tta * tta * (tta * tta));
            e_t = e_t + ka[0] * (ttb * ttb) + ka[1] * (ttb * ttb * (ttb * ttb));
        } else if (ta == 2) {
            double x2 = mi[0] * mi[0], y2 = mi[1] * mi[1], z2 = mi[2] * mi[2];
            e_c = e_c - ka[0] * (x2 * y2 + y2 * z2 + z2 * x2) - ka[1] * (x2 * y2 * z2);
            x2 = tm[0] * tm[0]; y2 = tm[1] * tm[1]; z2 = tm[2] * tm[2];
            e_t = e_t - ka[0] * (x2 * y2 + y2 * z2 + z2 * x2) - ka[1] * (x2 * y2 * z2);
        }
        if (ta == 7) {
            double tta = mi[0] * ea[0] + mi[1] * ea[1] + mi[2] * ea[2];
            double ttb = tm[0] * ea[0] + tm[1] * ea[1] + tm[2] * ea[2];
            e_c = e_c + ka[0] * (tta * tta) + ka[1] * (tta * tta * (tta * tta));
            e_t = e_t + ka[0] * (ttb * ttb) + ka[1] * (ttb * ttb * (ttb * ttb));
            double aw1 = ka[0] * h->sb[iflip], aw2 = ka[1] * h->sb[iflip];
            double x2 = mi[0] * mi[0], y2 = mi[1] * mi[1], z2 = mi[2] * mi[2];
            e_c = e_c + aw1 * (x2 * y2 + y2 * z2 + z2 * x2) + aw2 * (x2 * y2 * z2);
            x2 = tm[0] * tm[0]; y2 = tm[1] * tm[1]; z2 = tm[2] * tm[2];
            e_t = e_t + aw1 * (x2 * y2 + y2 * z2 + z2 * x2) + aw2 * (x2 * y2 * z2);
        }
    }
    if (h->do_dm == 1) {
        int nd = h->dmlistsize[ih];
        for (int j = 0; j < nd; ++j) {
            int jn = h->dmlist[j + (int64_t)h->max_no_dmneigh * iflip] - 1;
            const double *d = &h->dm_vect[3 * (j + (int64_t)h->max_no_dmneigh * ih)];
            const double *mj = &V3(emomM, 0, jn, k, N);
            e_c = e_c - d[0] * (mi[1] * mj[2] - ei[2] * mj[1]) - d[1] * (mi[2] * mj[0] - mi[0] * mj[2]) -
                  d[2] * (ei[0] * mj[1] - mi[1] * mj[0]);
            e_t = e_t - d[0] * (tm[1] * mj[2] - tm[2] * mj[1]) - d[1] * (tm[2] * mj[0] - tm[0] * mj[2]) -
                  d[2] * (tm[0] * mj[1] - tm[1] * mj[0]);
        }
    }
    e_c = e_c - ext[0] * mi[0] - ext[1] * mi[1] - ext[2] * mi[2];
    e_t = e_t - ext[0] * tm[0] - ext[1] * tm[1] - ext[2] * tm[2];
    return ORC_MUB * (e_t - e_c);
}

/* flip_a (montecarlo_common.f90:139-267), do_lsf=='N', no induced moments */
static int flip_a(double de, double temperature, double temprescale, double flipprob) {
    double beta = 1.0 / ORC_KBOLT / (temprescale * temperature + 1.0e-15);
    return (de <= 0.0 || flipprob < exp(-beta * de));
}

/* flip_h (montecarlo_common.f90:371-422) */
static void flip_h(double mmom, double temperature, double temprescale, double flipprob,
                   const double totfield[3], double q, double out[3]) {
    double beta = 1.0 / ORC_KBOLT / (temprescale * temperature);
    double zfc[3];
    for (int c = 0; c < 3; ++c) zfc[c] = beta * totfield[c] * ORC_MUB * mmom;
    double zarg = sqrt(zfc[0] * zfc[0] + zfc[1] * zfc[1] + zfc[2] * zfc[2]);
    double zctheta = zfc[2] / zarg;
    double zstheta = sqrt(1.0 - zctheta * zctheta) + DBL_TOLERANCE;
    double zcphi = zfc[0] / (zarg * zstheta);
    double zsphi = zfc[1] / (zarg * zstheta);
    double ctheta = 1.0 + (1.0 / zarg) * log((1.0 - exp(-2.0 * zarg)) * q + exp(-2.0 * zarg) + DBL_TOLERANCE);
    double stheta = sqrt(1.0 - ctheta * ctheta);
    double phi = ORC_PI * (2.0 * flipprob - 1.0);
    double st[3] = {stheta * cos(phi), stheta * sin(phi), ctheta};
    out[0] = zcphi * zctheta * st[0] - zsphi * st[1] + zcphi * zstheta * st[2];
    out[1] = zsphi * zctheta * st[0] + zcphi * st[1] + zsphi * zstheta * st[2];
    out[2] = -zstheta * st[0] + zctheta * st[2];
}

/* mc_evolve (montecarlo.f90:44-273), modes 'M' and 'H', single-threaded loop in
 * the reference's (atom, ensemble) order.  beff is (3,natom,mensemble) and is
 * written by the heat-bath branch exactly like effective_field_hb does. */
int orc_mc_evolve_ref(const orc_ham *h, char mode, double temperature, double temprescale,
                      const int32_t *iflip_a, orc_mt_state *c, orc_zig *zig, double *emom, double *emomM,
                      double *mmom, double *beff) {
    const int N = h->natom, M = h->mensemble;
    const int64_t n3 = 3 * (int64_t)N * M, n1 = (int64_t)N * M;
    double delta = F32(2.0 / 25.0) * pow(ORC_KBOLT * temperature / ORC_MUB, 0.20);
    double *fm = (double *)malloc(sizeof(double) * n3);
    double *fg = (double *)malloc(sizeof(double) * n3);
    double *newmom = (double *)malloc(sizeof(double) * n3);
    double *mflip = (double *)malloc(sizeof(double) * n1);
    double *fa = (double *)malloc(sizeof(double) * n1);
    for (int64_t t = 0; t < n3; ++t) fm[t] = orc_mt_real2(c);     /* rng_uniformP(flipprob_m) */
    orc_zig_fill(zig, fg, n3);                                   /* rng_gaussianP(flipprob_g) */
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < M; ++k)
            choose_random_flip(&V3(emom, 0, i, k, N), delta, &V3(fm, 0, i, k, N), &V3(fg, 0, i, k, N),
                               &V3(newmom, 0, i, k, N));
    if (mode == 'H')
        for (int64_t t = 0; t < n1; ++t) mflip[t] = orc_mt_real2(c);
    for (int64_t t = 0; t < n1; ++t) fa[t] = orc_mt_real2(c);    /* rng_uniformP(flipprob_a) */
    /* dipoles: the field of the moments at the start of the step, an extra external field
     * for Metropolis (montecarlo.f90:216-231); the heat bath's effective_field_hb evaluates
     * the site's own dipolar field from the current moments */
    if (h->do_dip && mode != 'H') orc_dipole_field(h, emomM, h->dip_work);
    for (int i = 0; i < N; ++i) {
        for (int k = 0; k < M; ++k) {
            int ia = iflip_a[i] - 1;
            double ext[3];
            for (int cc = 0; cc < 3; ++cc) {
                const double bd = h->do_dip ? V3(h->dip_work, cc, ia, k, N) : 0.0;
                ext[cc] = (V3(h->extfield, cc, ia, k, N) + bd) + 0.0;
            }
            if (mode == 'H') {
                double tf[3], nm[3];
                if (h->do_dip) {
                    double f[3];
                    dipole_field_site(h, emomM, ia, k, f);
                    for (int cc = 0; cc < 3; ++cc) V3(h->dip_work, cc, ia, k, N) = f[cc];
                }
                orc_effective_field_single(h, emomM, ia, k, tf);
                for (int cc = 0; cc < 3; ++cc) V3(beff, cc, ia, k, N) = tf[cc];
                double mm = M2(mmom, ia, k, N);
                flip_h(mm, temperature, temprescale, M2(fa, i, k, N), tf, M2(mflip, i, k, N), nm);
                for (int cc = 0; cc < 3; ++cc) {
                    V3(emom, cc, ia, k, N) = nm[cc];
                    V3(emomM, cc, ia, k, N) = mm * nm[cc];
                }
            } else {
                double de = calculate_energy(h, emomM, emom, mmom, ia, &V3(newmom, 0, ia, k, N), ext, k);
                if (flip_a(de, temperature, temprescale, M2(fa, i, k, N))) {
                    double mm = M2(mmom, ia, k, N);
                    for (int cc = 0; cc < 3; ++cc) {
                        V3(emom, cc, ia, k, N) = V3(newmom, cc, ia, k, N);
                        V3(emomM, cc, ia, k, N) = mm * V3(newmom, cc, ia, k, N);
                    }
                }
            }
        }
    }
    free(fm); free(fg); free(newmom); free(mflip); free(fa);
    return 0;
}

/* The GPU's checkerboard chain: same single-spin kernels as mc_evolve, sites of
 * one colour updated independently, draws from Philox keyed by (site, ensemble,
 * sweep).  Stream 1 gives (ftype/phi, sphere, sphere, accept) or heat-bath
 * (q, phi); stream 2 gives the Gaussian trial vector. */
int orc_mc_sweep_checkerboard(const orc_ham *h, char mode, double temperature,
                              const int32_t *colour_sites, const int32_t *colour_start, int ncolour,
                              uint64_t seed, int64_t sweep, double *emom, double *emomM, const double *mmom) {
    return orc_mc_sweep_checkerboard_temps(h, mode, temperature, NULL, colour_sites, colour_start, ncolour, seed,
                                           sweep, emom, emomM, mmom);
}

/* The same sweep with one temperature per ensemble (temps[k]; NULL: `temperature`
 * for all), as the replicas of pt_iphase (pt_driver.f90:58-367) run it. */
int orc_mc_sweep_checkerboard_temps(const orc_ham *h, char mode, double temperature, const double *temps,
                                    const int32_t *colour_sites, const int32_t *colour_start, int ncolour,
                                    uint64_t seed, int64_t sweep, double *emom, double *emomM, const double *mmom) {
    const int N = h->natom, M = h->mensemble;
    /* dipoles: Metropolis takes the field of the moments at the start of the sweep as an
     * extra external field (montecarlo.f90:216-231); the heat bath takes the field in the
     * site's effective field (effective_field_hb), evaluated here before each colour, the
     * moments of the colour's sites changing only within it */
    if (h->do_dip && mode != 'H') orc_dipole_field(h, emomM, h->dip_work);
    for (int col = 0; col < ncolour; ++col) {
        int beg = colour_start[col], end = colour_start[col + 1];
        if (h->do_dip && mode == 'H') orc_dipole_field(h, emomM, h->dip_work);
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
        for (int t = beg; t < end; ++t) {
            int i = colour_sites[t];
            for (int k = 0; k < M; ++k) {
                const double Tk = temps ? temps[k] : temperature;
                double u[4];
                orc_philox_uniform4(seed, i, k, sweep, 1u, u);
                double mm = M2(mmom, i, k, N);
                if (mode == 'H') {
                    double tf[3], nm[3];
                    orc_effective_field_single(h, emomM, i, k, tf);
                    flip_h(mm, Tk, 1.0, u[1], tf, u[0], nm);
                    for (int cc = 0; cc < 3; ++cc) {
                        V3(emom, cc, i, k, N) = nm[cc];
                        V3(emomM, cc, i, k, N) = mm * nm[cc];
                    }
                } else {
                    double gn[3] = {0.0, 0.0, 0.0}, nm[3], ext[3];
                    double rn[3] = {u[0], u[1], u[2]};
                    if ((int)floor(3.0 * rn[0]) == 1) orc_philox_normal3(seed, i, k, sweep, 2u, gn);
                    const double delta = F32(2.0 / 25.0) * pow(ORC_KBOLT * Tk / ORC_MUB, 0.20);
                    choose_random_flip(&V3(emom, 0, i, k, N), delta, rn, gn, nm);
                    /* loc_mag_fld = extfield + beff + loc_demag_fld (montecarlo.f90:231) */
                    for (int cc = 0; cc < 3; ++cc) {
                        const double bd = h->do_dip ? V3(h->dip_work, cc, i, k, N) : 0.0;
                        ext[cc] = (V3(h->extfield, cc, i, k, N) + bd) + 0.0;
                    }
                    double de = calculate_energy(h, emomM, emom, mmom, i, nm, ext, k);
                    if (flip_a(de, Tk, 1.0, u[3])) {
                        for (int cc = 0; cc < 3; ++cc) {
                            V3(emom, cc, i, k, N) = nm[cc];
                            V3(emomM, cc, i, k, N) = mm * nm[cc];
                        }
                    }
                }
            }
        }
    }
    return 0;
}

/* ===================================================================== */
/* Observables                                                            */
/* ===================================================================== */
void orc_mavg(int natom, int mensemble, const double *emomM, double *mvec, double *mabs) {
    for (int k = 0; k < mensemble; ++k) {
        double m[3] = {0.0, 0.0, 0.0};
        for (int i = 0; i < natom; ++i)
            for (int c = 0; c < 3; ++c) m[c] = m[c] + V3(emomM, c, i, k, natom);
        for (int c = 0; c < 3; ++c) mvec[c + 3 * k] = m[c];
        mabs[k] = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]) / natom;
    }
}

/* calc_energy (energy.f90:60-405): exchange, DMI, anisotropy, external field;
 * per-atom energies converted to mRy with fcinv = mub/mry. */
void orc_energy(const orc_ham *h, const double *emomM, double *e_tot, double *e_xc, double *e_dm,
                double *e_ani, double *e_ext) {
    const int N = h->natom, M = h->mensemble;
    const double fcinv = ORC_MUB / ORC_MRY;
    /* the dipolar field of the same moments (energy.f90:154-167) */
    if (h->do_dip) orc_dipole_field(h, emomM, h->dip_work);
    for (int k = 0; k < M; ++k) {
        double exc = 0.0, edm = 0.0, eani = 0.0, eext = 0.0, edip = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : exc, edm, eani, eext, edip) num_threads(orc_get_threads())
        for (int i = 0; i < N; ++i) {
            const double *mi = &V3(emomM, 0, i, k, N);
            int ih = h->aham[i] - 1;
            double bx[3] = {0.0, 0.0, 0.0};
            if (h->do_jtensor == 1) {
                tensor_exchange(h, emomM, i, ih, k, bx);  /* energy.f90:244-247: the pair energy */
            } else {
                for (int j = 0; j < h->nlistsize[ih]; ++j) {
                    int jn = h->nlist[j + (int64_t)h->max_no_neigh * i] - 1;
                    double c = h->ncoup[j + (int64_t)h->max_no_neigh * ih];
                    for (int cc = 0; cc < 3; ++cc) bx[cc] = bx[cc] + c * V3(emomM, cc, jn, k, N);
                }
            }
            exc = exc + (-0.5 * (mi[0] * bx[0] + mi[1] * bx[1] + mi[2] * bx[2]));
            /* with the tensor the DM energy is not evaluated (energy.f90:219-247, :371-379) */
            if (h->do_dm == 1 && h->do_jtensor != 1) {
                double bd[3] = {0.0, 0.0, 0.0};
                for (int j = 0; j < h->dmlistsize[ih]; ++j) {
                    int jn = h->dmlist[j + (int64_t)h->max_no_dmneigh * i] - 1;
                    const double *d = &h->dm_vect[3 * (j + (int64_t)h->max_no_dmneigh * ih)];
                    const double *mj = &V3(emomM, 0, jn, k, N);
                    bd[0] = bd[0] + d[2] * mj[1] - d[1] * mj[2];
                    bd[1] = bd[1] + d[0] * mj[2] - d[2] * mj[0];
                    bd[2] = bd[2] + d[1] * mj[0] - d[0] * mj[1];
                }
                edm = edm + (-0.5 * (mi[0] * bd[0] + mi[1] * bd[1] + mi[2] * bd[2]));
            }
            if (h->do_aniso == 1) {
                double ta[3], tq[3] = {0.0, 0.0, 0.0};
                ta[0] = ta[1] = ta[2] = 0.0;
                site_field_aniso(h, emomM, i, k, ta, tq);
                for (int cc = 0; cc < 3; ++cc) ta[cc] = ta[cc] + tq[cc];
                eani = eani + (-0.5 * (mi[0] * ta[0] + mi[1] * ta[1] + mi[2] * ta[2]));
            }
            double be[3];
            for (int cc = 0; cc < 3; ++cc) be[cc] = 0.0 + V3(h->extfield, cc, i, k, N);
            eext = eext + (-1.0 * (mi[0] * be[0] + mi[1] * be[1] + mi[2] * be[2]));
            /* update_ene(emomM, bfield_dip, 0.5) (energy.f90:286-291) */
            if (h->do_dip) {
                const double *bd = &V3(h->dip_work, 0, i, k, N);
                edip = edip + (-0.5 * (mi[0] * bd[0] + mi[1] * bd[1] + mi[2] * bd[2]));
            }
        }
        double xc = exc / N, dm = edm / N, an = eani / N, ex = eext / N, dp = edip / N;
        /* ene_xc + ene_dm + ene_ext + ene_ani + ene_dip (energy.f90:372-374) */
        double tot = xc + dm + ex + an + dp;
        if (e_xc) e_xc[k] = xc * fcinv;
        if (e_dm) e_dm[k] = dm * fcinv;
        if (e_ani) e_ani[k] = an * fcinv;
        if (e_ext) e_ext[k] = ex * fcinv;
        if (e_tot) e_tot[k] = tot * fcinv;
    }
}

/* calc_and_print_cumulant (prn_averages.f90:919-1095); weights grow by one per
 * sample, as in the reference. */
void orc_cumulant_update(orc_cumulant *c, int natom, int mensemble, const double *emomM, double temp,
                         const double *energy, double out[6]) {
    double avrgmt = 0, avrgmt2 = 0, avrgmt4 = 0, cumulant = 0, pmsusc = 0, cv = 0;
    for (int k = 0; k < mensemble; ++k) {
        double m[3] = {0.0, 0.0, 0.0};
        for (int i = 0; i < natom; ++i)
            for (int cc = 0; cc < 3; ++cc) m[cc] = m[cc] + V3(emomM, cc, i, k, natom);
        double avrgme = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]) / natom;
        double avrgm2 = avrgme * avrgme;
        double avrgm4 = avrgm2 * avrgm2;
        c->cumuw = c->cumuw + 1.0;
        avrgmt = (c->avrgmcum * c->cumutotw + avrgme * c->cumuw) / (c->cumutotw + c->cumuw);
        avrgmt2 = (c->avrgm2cum * c->cumutotw + avrgm2 * c->cumuw) / (c->cumutotw + c->cumuw);
        avrgmt4 = (c->avrgm4cum * c->cumutotw + avrgm4 * c->cumuw) / (c->cumutotw + c->cumuw);
        cumulant = 1 - (avrgmt4 / 3 / (avrgmt2 * avrgmt2));
        c->avrgmcum = avrgmt;
        c->avrgm2cum = avrgmt2;
        c->avrgm4cum = avrgmt4;
        if (temp > 0.0)
            pmsusc = (avrgmt2 - avrgmt * avrgmt) * ORC_MUB * ORC_MUB * natom / (ORC_KBOLT * ORC_KBOLT) / temp;
        else
            pmsusc = (avrgmt2 - avrgmt * avrgmt) * natom * ORC_MUB * ORC_MUB / ORC_KBOLT;
        if (energy && temp > 0.0) {
            double en = energy[k];
            double avrgen = (c->avrgecum * c->cumutotw + en * c->cumuw) / (c->cumutotw + c->cumuw);
            double avrgen2 = (c->avrge2cum * c->cumutotw + en * en * c->cumuw) / (c->cumutotw + c->cumuw);
            cv = (avrgen2 - avrgen * avrgen) * ORC_MRY * ORC_MRY * natom / (ORC_KBOLT * ORC_KBOLT) / (temp * temp);
            c->avrgecum = avrgen;
            c->avrge2cum = avrgen2;
        }
        c->navrgcum = c->navrgcum + 1;
        c->cumutotw = c->cumutotw + c->cumuw;
    }
    out[0] = avrgmt; out[1] = avrgmt2; out[2] = avrgmt4; out[3] = cumulant; out[4] = pmsusc; out[5] = cv;
}
