/*
 * A plain C99 caller of include/uppasd_gpu.h in the role the Fortran driver takes
 * (sd_mphaseCUDA, sd_driver.f90:1118-1153; mc_mphase, mc_driver.f90:234): module arrays in
 * Fortran layout (nlist(mnn, natom) 1-based, ncoup(mnn, nham), emom(3, natom, mensemble)),
 * couplings scaled as setup_neighbour_hamiltonian / setup_anisotropies scale them, every
 * status checked.  No Fortran compiler exists here, so this stands in for the Fortran
 * driver's bind(c) interface module.
 *
 *   c_harness reject           init with an out-of-range neighbour index: expects -1 and
 *                              a message (runs without a GPU: arguments are checked first)
 *   c_harness run <n> <out>    simple cubic 8^3, two ensembles, J = 1 mRy, uniaxial
 *                              K = 0.1 mRy along z, B = 0.5 T along z, moments 2 muB;
 *                              n Depondt steps at 100 K (Philox seed 7), then 3 heat-bath
 *                              sweeps at 50 K; writes to <out> (native doubles): emom after
 *                              the steps, M, |M|, E per ensemble, emom after the sweeps
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/uppasd_gpu.h"

#define L 8
#define NATOM (L * L * L)
#define MENS 2
#define MNN 6
#define MRY 2.179872325e-21
#define MUB 9.274009994e-24

static int site(int x, int y, int z) {
    x = (x + L) % L;
    y = (y + L) % L;
    z = (z + L) % L;
    return x + L * (y + L * z);
}

static int check(const char *what, int rc) {
    if (rc != UPPASD_GPU_OK) {
        fprintf(stderr, "%s failed with status %d: %s\n", what, rc, uppasd_gpu_last_error());
        exit(1);
    }
    return rc;
}

int main(int argc, char **argv) {
    static int32_t nlist[MNN * NATOM], nlistsize[NATOM], aham[NATOM], taniso[NATOM];
    static double ncoup[MNN * NATOM], eaniso[3 * NATOM], kaniso[2 * NATOM], sb[NATOM];
    static double ext[3 * NATOM * MENS], mmom[NATOM * MENS], lam[NATOM], temp[NATOM];
    static double emom[3 * NATOM * MENS], emomM[3 * NATOM * MENS];
    /* the cubic images of the bond (0, 0, 1) in the order the reference generates them */
    static const int off[MNN][3] = {{0, 0, 1}, {0, 0, -1}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}};
    const double mom = 2.0, j_mry = 1.0, k_mry = 0.1;
    int i, k, q;

    if (argc < 2) {
        fprintf(stderr, "usage: %s reject | run <nsteps> <out>\n", argv[0]);
        return 2;
    }
    for (i = 0; i < NATOM; ++i) {
        int x = i % L, y = (i / L) % L, z = i / (L * L);
        for (q = 0; q < MNN; ++q) {
            nlist[q + MNN * i] = site(x + off[q][0], y + off[q][1], z + off[q][2]) + 1;
            ncoup[q + MNN * i] = j_mry * 2.0 * MRY / MUB / (mom * mom);
        }
        nlistsize[i] = MNN;
        aham[i] = i + 1;
        taniso[i] = 1;
        eaniso[3 * i] = 0.0;
        eaniso[3 * i + 1] = 0.0;
        eaniso[3 * i + 2] = 1.0;
        kaniso[2 * i] = MRY / MUB * k_mry / (mom * mom);
        kaniso[2 * i + 1] = 0.0;
        sb[i] = 0.0;
        lam[i] = 0.1;
        temp[i] = 100.0;
        for (k = 0; k < MENS; ++k) {
            size_t o = (size_t)3 * (i + (size_t)NATOM * k);
            double v[3] = {sin(0.37 * i + 1.1 * k), cos(0.23 * i), 0.4 + 0.1 * k};
            double n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            emom[o] = v[0] / n;
            emom[o + 1] = v[1] / n;
            emom[o + 2] = v[2] / n;
            ext[o] = 0.0;
            ext[o + 1] = 0.0;
            ext[o + 2] = 0.5;
            mmom[i + NATOM * k] = mom;
        }
    }

    uppasd_gpu_consts c;
    memset(&c, 0, sizeof c);
    c.natom = NATOM;
    c.mensemble = MENS;
    c.max_no_neigh = MNN;
    c.nham = NATOM;
    c.do_aniso = 1;
    c.sdealgh = 5;
    c.delta_t = 1e-16;
    c.bn = 1.0;
    c.temprescale = 1.0;
    c.gpu_rng_seed = 7;
    c.gpu_rng = 0;
    c.precision = 0;
    c.n1 = c.n2 = c.n3 = L;
    c.na = 1;

    uppasd_gpu_arrays a;
    memset(&a, 0, sizeof a);
    a.nlist = nlist;
    a.nlistsize = nlistsize;
    a.ncoup = ncoup;
    a.aham = aham;
    a.taniso = taniso;
    a.eaniso = eaniso;
    a.kaniso = kaniso;
    a.sb = sb;
    a.external_field = ext;
    a.mmom = mmom;
    a.lambda1_array = lam;
    a.temp_array = temp;
    a.emom = emom;

    uppasd_gpu_sim *sim = NULL;
    if (strcmp(argv[1], "reject") == 0) {
        nlist[3] = NATOM + 1; /* out of range */
        int rc = uppasd_gpu_init(&c, &a, &sim);
        printf("%d %s\n", rc, uppasd_gpu_last_error());
        return rc == UPPASD_GPU_EINVAL && sim == NULL ? 0 : 1;
    }
    if (strcmp(argv[1], "run") != 0 || argc < 4) return 2;
    const long nsteps = strtol(argv[2], NULL, 10);
    FILE *f = fopen(argv[3], "wb");
    if (!f) return 1;

    check("uppasd_gpu_init", uppasd_gpu_init(&c, &a, &sim));
    check("uppasd_gpu_sd_run", uppasd_gpu_sd_run(sim, nsteps));
    check("uppasd_gpu_get_moments", uppasd_gpu_get_moments(sim, emom, emomM));
    double mvec[3 * MENS], mabs[MENS], energy[MENS];
    check("uppasd_gpu_observables", uppasd_gpu_observables(sim, mvec, mabs, energy));
    fwrite(emom, sizeof(double), 3 * NATOM * MENS, f);
    fwrite(mvec, sizeof(double), 3 * MENS, f);
    fwrite(mabs, sizeof(double), MENS, f);
    fwrite(energy, sizeof(double), MENS, f);
    check("uppasd_gpu_mc_run", uppasd_gpu_mc_run(sim, 'H', 50.0, 3));
    check("uppasd_gpu_get_moments", uppasd_gpu_get_moments(sim, emom, emomM));
    fwrite(emom, sizeof(double), 3 * NATOM * MENS, f);
    fclose(f);
    check("uppasd_gpu_finalize", uppasd_gpu_finalize(sim));
    printf("ok\n");
    return 0;
}
