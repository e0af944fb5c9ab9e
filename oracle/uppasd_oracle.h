/*
 * uppasd_oracle.h -- CPU restatement of UppASD's spin-update hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle and the
 * CPU baseline; the product path (uppasd_gb300/libuppasd_gb300.so) never links
 * or calls it.  Every routine follows the Fortran routine named beside it, in
 * the reference's own array layout: Fortran column-major (3,Natom,Mensemble)
 * AoS spins, 1-based neighbour indices, couplings already scaled by
 * 2*mRy/muB/(m_i*m_j) exactly as Hamiltonian/hamiltonianinit.f90:1041-1068
 * leaves them.  Arithmetic is written in the Fortran evaluation order and the
 * library is compiled with -ffp-contract=off so results do not depend on FMA
 * contraction.
 *
 * Parity is pinned against the reference's own golden vectors (the
 * tests/Solvers T=0 chain, regulartests.yaml:349-386) by tests/test_oracle_golden.py.
 */
#ifndef UPPASD_ORACLE_H
#define UPPASD_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- constants (Parameters/constants.f90:14-19) ---- */
#define ORC_GAMA_SI   1.760859644e11
#define ORC_KBOLT_SI  1.38064852e-23
#define ORC_MUB_SI    9.274009994e-24
#define ORC_MRY_SI    2.179872325e-21
/* The values in use: SI unless orc_set_units changed them (aunits = 'Y' sets gama,
 * k_bolt, mub and mry to 1, Input/inputhandler.f90:1685-1704). */
extern double orc_gama, orc_kbolt, orc_mub, orc_mry;
void orc_set_units(double gama, double kbolt, double mub, double mry);
#define ORC_GAMA   orc_gama
#define ORC_KBOLT  orc_kbolt
#define ORC_MUB    orc_mub
#define ORC_MRY    orc_mry
#define ORC_PI     3.141592653589793238462643383279502884197

/* ---- Mersenne twister variant (RNG/mtprng.f90:118-325) ---- */
typedef struct {
    int32_t mti;
    uint64_t mt[624]; /* INT64 words of the Fortran state, kept as raw bits */
} orc_mt_state;

void     orc_mt_init(orc_mt_state *s, int32_t seed);
uint64_t orc_mt_rand64(orc_mt_state *s);       /* mtprng_rand64: value in [0,2^32) */
int32_t  orc_mt_rand(orc_mt_state *s);         /* mtprng_rand */
double   orc_mt_real1(orc_mt_state *s);        /* [0,1] */
double   orc_mt_real2(orc_mt_state *s);        /* [0,1) */

/* ---- ziggurat normals (RNG/randomnumbers.f90:330-509) ---- */
typedef struct {
    orc_mt_state z;
    int32_t kn[128];
    double  fn[128];
    double  wn[128];
} orc_zig;

void   orc_zig_setup(orc_zig *g, int32_t seed);   /* r4_nor_setup */
double orc_zig_nor(orc_zig *g);                   /* r4_nor */
void   orc_zig_fill(orc_zig *g, double *out, int64_t n);  /* fill_rngarray */

/* ---- Philox4x32-10 normals: the counter-based stream the GPU uses ---- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* Three N(0,1) draws for (site, ensemble, step, stream); FP64 Box-Muller. */
void orc_philox_normal3(uint64_t seed, int64_t site, int32_t ens, int64_t step,
                        uint32_t stream, double z[3]);
/* Four uniforms in (0,1) for (site, ensemble, step, stream) (MC draws). */
void orc_philox_uniform4(uint64_t seed, int64_t site, int32_t ens, int64_t step,
                         uint32_t stream, double u[4]);

/* ---- Hamiltonian (Hamiltonian/hamiltoniandatatype.f90:14-100) ---- */
typedef struct {
    int natom, mensemble;
    int max_no_neigh, nham;
    const int32_t *nlist;      /* (max_no_neigh, natom), 1-based */
    const int32_t *nlistsize;  /* (nham) */
    const double  *ncoup;      /* (max_no_neigh, nham) */
    const int32_t *aham;       /* (natom), 1-based */
    int do_dm, max_no_dmneigh;
    const int32_t *dmlist;     /* (max_no_dmneigh, natom) */
    const int32_t *dmlistsize; /* (nham) */
    const double  *dm_vect;    /* (3, max_no_dmneigh, nham) */
    int do_aniso;
    const int32_t *taniso;     /* (natom) */
    const double  *eaniso;     /* (3, natom) */
    const double  *kaniso;     /* (2, natom) */
    const double  *sb;         /* (natom) */
    const double  *extfield;   /* (3, natom, mensemble) */
    /* SKKR-style exchange tensor (hamiltoniandata.f90:138, j_tens(3,3,max_no_neigh,nHam));
     * with do_jtensor == 1 it replaces ncoup in the field and energies. */
    int do_jtensor;
    const double  *j_tens;     /* (3, 3, max_no_neigh, nham) */
    /* dipole-dipole field (do_dip = 1, brute force: Hamiltonian/dipolemanager.f90:147-158
     * with the tensor of dipolecommon.f90:51-84); the supercell's geometry: atom
     * i = I0 + NA (I1 + N1 (I2 + N2 I3)) (0-based) at I1 C1 + I2 C2 + I3 C3 + Bas(I0), in
     * units of alat (m); dip_work (3, natom, mensemble) receives the dipolar field. */
    int do_dip;
    int dip_na, dip_n1, dip_n2, dip_n3;
    const double *dip_cell;    /* (3, 3): column a is C_{a+1} */
    const double *dip_bas;     /* (3, NA) */
    double dip_alat;
    double *dip_work;
} orc_ham;

/* The dipolar field of every atom from the full moments emomM (3, natom, mensemble), into
 * out (same layout): B_i = sum_j Q(r_i - r_j) m_j over all atoms j != i, no periodic
 * images, Q(R) = 1e-7 mub / alat^3 (3 R R^T - R^2 I) / R^5 (dipoleMatrix). */
void orc_dipole_field(const orc_ham *h, const double *emomM, double *out);

/* effective_field_full (hamiltonianactions.f90:108-252).  Returns energy in mRy
 * (the routine's own energy*mub/mry).  beff is (3,natom,mensemble). */
double orc_effective_field(const orc_ham *h, const double *emomM, double *beff);
/* effective_field_single (hamiltonianactions.f90:254-392): field of one site. */
void orc_effective_field_single(const orc_ham *h, const double *emomM, int i, int k,
                                double out[3]);

/* ---- LLG integration (sd_driver.f90:554-767 measurement-phase step) ---- */
enum { ORC_NOISE_NONE = 0, ORC_NOISE_ZIGGURAT = 1, ORC_NOISE_ARRAY = 2, ORC_NOISE_PHILOX = 3 };

typedef struct {
    int sdealgh;            /* 1 midpoint, 4 Heun, 5 Depondt, 6 SIB fixed point, 11 LLGI */
    double delta_t, bn, temprescale;
    const double *lambda1;  /* (natom) */
    const double *temp;     /* (natom) */
    const double *landeg;   /* (natom) */
    int noise_mode;
    orc_zig *zig;           /* ORC_NOISE_ZIGGURAT */
    const double *noise;    /* ORC_NOISE_ARRAY: N(0,1) values (3,natom,mensemble) for this step */
    uint64_t seed;          /* ORC_NOISE_PHILOX */
    int64_t step;           /* ORC_NOISE_PHILOX counter */
    double relaxtime;       /* SDEalgh 11: relaxation time of the inertial regime (s) */
    int perp;               /* input perp = 'Y': field projected perpendicular to emom */
} orc_llg;

typedef struct {
    double *emom, *emom2, *emomM;  /* (3,natom,mensemble) */
    double *mmom;                  /* (natom,mensemble) */
    double *b2eff, *beff;          /* (3,natom,mensemble) work */
    double *ranv;                  /* (3,natom,mensemble) work */
    double *mpast;                 /* SDEalgh 11: m(t - dt), zero before the first step */
} orc_state;

/* One full step: field -> evolve_first -> field -> evolve_second -> moment_update. */
int orc_sd_step(const orc_ham *h, const orc_llg *p, orc_state *s);
/* The raw N(0,1) numbers one step draws, in draw order (3,natom,mensemble). */
void orc_llg_draw_normals(const orc_llg *p, int natom, int mensemble, double *out);

/* initmag==1 random start (System/magnetizationinit.f90:141-170) */
void orc_initmag_random(orc_mt_state *c, int natom, int mensemble, const double *mmom,
                        double *emom, double *emomM);

/* ---- Monte Carlo ---- */
/* choose_random_atom_x (MonteCarlo/montecarlo.f90:277-301), 1-based output. */
void orc_choose_random_atom_x(orc_mt_state *c, int natom, int32_t *iflip_a);
/* mc_evolve (montecarlo.f90:44-273) for mode 'M' (Metropolis, Hinzke-Nowak trials)
 * or 'H' (heat bath), in the reference's visiting order and RNG draw order. */
int orc_mc_evolve_ref(const orc_ham *h, char mode, double temperature, double temprescale,
                      const int32_t *iflip_a, orc_mt_state *c, orc_zig *zig,
                      double *emom, double *emomM, double *mmom, double *beff);
/* Checkerboard sweep with Philox draws: the Markov chain the GPU runs.
 * colour_sites lists sites (0-based) colour by colour; colour_start has ncolour+1 entries. */
int orc_mc_sweep_checkerboard(const orc_ham *h, char mode, double temperature,
                              const int32_t *colour_sites, const int32_t *colour_start,
                              int ncolour, uint64_t seed, int64_t sweep,
                              double *emom, double *emomM, const double *mmom);
/* The same with one temperature per ensemble (temps[k]; NULL: `temperature`). */
int orc_mc_sweep_checkerboard_temps(const orc_ham *h, char mode, double temperature, const double *temps,
                                    const int32_t *colour_sites, const int32_t *colour_start, int ncolour,
                                    uint64_t seed, int64_t sweep, double *emom, double *emomM, const double *mmom);

/* ---- observables ---- */
/* |M| per ensemble / natom (measurements.f90:211-235, prn_averages.f90:118) */
void orc_mavg(int natom, int mensemble, const double *emomM, double *mvec /*(3,M)*/, double *mabs /*(M)*/);
/* calc_energy (Hamiltonian/energy.f90:60-405): total energy per atom in mRy per ensemble. */
void orc_energy(const orc_ham *h, const double *emomM, double *e_tot /*(M)*/, double *e_xc,
                double *e_dm, double *e_ani, double *e_ext);

typedef struct {
    double cumuw, cumutotw, avrgmcum, avrgm2cum, avrgm4cum, avrgecum, avrge2cum;
    int navrgcum;
} orc_cumulant;
/* calc_and_print_cumulant (prn_averages.f90:919-1095): running weighted averages. */
void orc_cumulant_update(orc_cumulant *c, int natom, int mensemble, const double *emomM,
                         double temp, const double *energy /*(M) mRy per atom or NULL*/,
                         double out[6] /* <M>, <M^2>, <M^4>, U_L, chi, Cv */);

/* omp threads used by the oracle (0 = library default) */
void orc_set_threads(int n);
int  orc_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
