/*
 * uppasd_gpu.h -- C ABI of the GB300 spin-update hot path for UppASD.
 *
 * The Fortran drivers call these through iso_c_binding (bind(c)); every
 * argument is a plain pointer or scalar, arrays are passed in the reference's
 * own layout: Fortran column-major (3, Natom, Mensemble) spins, 1-based
 * neighbour indices, couplings already scaled by the reference's setup.
 * Every entry point returns an int status (0 = success, < 0 = error) and
 * never exits the process; uppasd_gpu_last_error() gives the message.
 *
 * Reference interfaces replaced (paths relative to the UppASD source tree):
 *   uppasd_gpu_init            <- FortranData_Initiate + fortrandata_setconstants_/
 *                                 setmatrices_/setinputdata_ (chelper.f90:166-188,
 *                                 gpu_files/fortranData.cpp:141-185) and
 *                                 cudamdsim_initiateconstants_/initiatematrices_
 *                                 (gpu_files/fort_helper.cpp:52-60)
 *   uppasd_gpu_sd_run          <- cudamdsim_measurementphase_ step loop
 *                                 (gpu_files/fort_helper.cpp:62-64,
 *                                 cudaMdSimulation.cu:461-499), i.e. the
 *                                 effective_field / evolve_first / evolve_second /
 *                                 moment_update sequence of sd_mphase
 *                                 (sd_driver.f90:657-767)
 *   uppasd_gpu_get_moments     <- the measurement copy-back (cudaMeasurement.cu:108-179)
 *   uppasd_gpu_mc_run          <- mc_evolve sweeps of mc_mphase (mc_driver.f90:309-366,
 *                                 MonteCarlo/montecarlo.f90:44-273)
 *   uppasd_gpu_observables     <- calc_mavrg (Measurement/measurements.f90:211-235) and
 *                                 calc_energy (Hamiltonian/energy.f90:60-405)
 *   uppasd_gpu_finalize        <- CudaMdSimulation teardown (cudaMdSimulation.cu:210-243)
 */
#ifndef UPPASD_GPU_H
#define UPPASD_GPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UPPASD_GPU_OK 0
#define UPPASD_GPU_EINVAL -1   /* bad argument or size */
#define UPPASD_GPU_ENOMEM -2   /* device allocation failed */
#define UPPASD_GPU_ECUDA -3    /* CUDA runtime error */
#define UPPASD_GPU_ESTATE -4   /* call not valid in the current state */
#define UPPASD_GPU_ENODEV -6   /* no usable sm_103 device */
#define UPPASD_GPU_EUNSUPPORTED -7

typedef struct uppasd_gpu_sim uppasd_gpu_sim;

/* Scalars of fortrandata_setconstants_ (gpu_files/fortranData.cpp:67-98) that the
 * hot path uses, plus explicit sizes and the solver / RNG selection. */
typedef struct {
    int32_t natom, mensemble;
    int32_t max_no_neigh, nham;        /* ncoup is (max_no_neigh, nham) */
    int32_t do_dm, max_no_dmneigh;
    int32_t do_aniso;
    int32_t sdealgh;                   /* 1 midpoint, 4 Heun, 5 Depondt, 6 SIB fixed point,
                                          7 spherical SIB fixed point, 11 LLGI */
    double delta_t, bn, temprescale;
    uint64_t gpu_rng_seed;             /* Philox key (gpu_rng_seed keyword) */
    int32_t gpu_rng;                   /* 0 Philox in-kernel, 1 caller-injected normals */
    int32_t precision;                 /* 0 FP64 everywhere (any neighbour list);
                                          1 FP32 field gather + FP64 spin master and
                                            renormalisation (structured lattices, Depondt);
                                          2 FP32 field gather + double-single (float-float)
                                            spin master and renormalisation (same scope);
                                          3 FP32 field gather over any neighbour list (scalar
                                            or tensor exchange, DMI, anisotropy, Zeeman) + FP64
                                            spin master and renormalisation (every SDEalgh of
                                            precision 0, perp included); mc_run 'H' and 'M'
                                            run in FP32 on the same mirror (mc_run_temps 'M'
                                            on the FP64 path);
                                          4 as 3 with a double-single (float-float) spin
                                            master renormalised in error-free FP32
                                            arithmetic (every SDEalgh of precision 3):
                                            GB300's FP64 pipe sets precision 3's step time;
                                            the FP64 state is made from the master when a
                                            call reads it */
    /* geometry of the reference's atom numbering i = I0 + NA*(I1 + N1*(I2 + N2*I3));
       0 when unknown (the structured path then stays off) */
    int32_t n1, n2, n3, na;
} uppasd_gpu_consts;

/* Arrays of fortrandata_setmatrices_ (gpu_files/fortranData.cpp:101-130) on the hot path. */
typedef struct {
    const int32_t *nlist;        /* (max_no_neigh, natom), 1-based */
    const int32_t *nlistsize;    /* (nham) */
    const double *ncoup;         /* (max_no_neigh, nham) */
    const int32_t *aham;         /* (natom), 1-based */
    const int32_t *dmlist;       /* (max_no_dmneigh, natom) or NULL */
    const int32_t *dmlistsize;   /* (nham) */
    const double *dm_vect;       /* (3, max_no_dmneigh, nham) */
    const int32_t *taniso;       /* (natom) or NULL */
    const double *eaniso;        /* (3, natom) */
    const double *kaniso;        /* (2, natom) */
    const double *sb;            /* (natom) */
    const double *external_field;/* (3, natom, mensemble) */
    const double *mmom;          /* (natom, mensemble) */
    const double *lambda1_array; /* (natom) */
    const double *temp_array;    /* (natom) */
    const double *landeg;        /* (natom); NULL means 1.0 (g = 2) */
    const double *emom;          /* (3, natom, mensemble) initial unit moments */
    const int32_t *species;      /* (natom) chemical type, 0-based (achtype - 1,
                                    System/chemicaldata.f90:9), or NULL: the structured
                                    path's species and the FP32-gather path's chemical
                                    site classes */
} uppasd_gpu_arrays;

const char *uppasd_gpu_last_error(void);
int uppasd_gpu_device_info(int32_t *sm_count, int32_t *cc_major, int32_t *cc_minor, int64_t *hbm_bytes);

int uppasd_gpu_init(const uppasd_gpu_consts *c, const uppasd_gpu_arrays *a, uppasd_gpu_sim **out);
int uppasd_gpu_finalize(uppasd_gpu_sim *s);

/* Spin state transfer in the reference layout (3, natom, mensemble). */
int uppasd_gpu_put_moments(uppasd_gpu_sim *s, const double *emom);
int uppasd_gpu_get_moments(uppasd_gpu_sim *s, double *emom, double *emomM);
/* Per-atom temperatures (natom).  The structured path (precision 1, 2) takes a uniform
 * temperature only (-7 otherwise). */
int uppasd_gpu_set_temperature(uppasd_gpu_sim *s, const double *temp_array);
int uppasd_gpu_set_step(uppasd_gpu_sim *s, int64_t step);

/* Input keyword perp = 'Y' (Input/inputhandler.f90:784): before each half-step the
 * effective field loses its component along emom (Evolution/evolution.f90:104-112,
 * :327-335).  0 or 1; -7 on the structured path (precision 1, 2). */
int uppasd_gpu_set_perp(uppasd_gpu_sim *s, int32_t perp);

/* The physical constants fortrandata_setconstants_ passes (gama, k_bolt, mub; gpu_files/
 * fortranData.cpp:67-98) and mry, for every LLG and Monte Carlo path of the simulation
 * (noise amplitudes, time scale, Boltzmann factors, energies in mRy).  SI
 * (Parameters/constants.f90:14-19) until called; aunits = 'Y' passes 1, 1, 1, 1
 * (Input/inputhandler.f90:1685-1704).  Each must be finite and > 0.  The batched
 * replica table (uppasd_gpu_mcbatch_*) stays in SI units. */
int uppasd_gpu_set_units(uppasd_gpu_sim *s, double gama, double k_bolt, double mub, double mry);

/* Relaxation time of the inertial regime for SDEalgh 11 (LLGI, Evolution/llgi.f90;
 * input keyword relaxtime, Input/inputhandler.f90:768, default 0).  Seconds, >= 0. */
int uppasd_gpu_set_relaxtime(uppasd_gpu_sim *s, double relaxtime);

/* SKKR-style exchange tensor (do_jtensor = 1): j_tens(3,3,max_no_neigh,nHam) in the
 * reference layout and scaling (Hamiltonian/hamiltoniandata.f90:138), on the exchange
 * list given at init.  It replaces ncoup in the effective field (tensor_field,
 * Hamiltonian/hamiltonianactions.f90:499-542, selected at :191-200), in the Monte
 * Carlo energy change (MonteCarlo/montecarlo_common.f90:502-510) and in the exchange
 * slot of the energy (the pair energy, Hamiltonian/energy.f90:244-247; as there, no
 * separate DM energy is evaluated while the tensor is on, the DM field stays).
 * NULL switches back to ncoup.  -7 on the structured path (precision 1, 2). */
int uppasd_gpu_set_jtensor(uppasd_gpu_sim *s, const double *j_tens);

/* Dipole-dipole field (input keyword do_dip, Hamiltonian/dipolemanager.f90:54-113).
 * Added first to every effective field of the FP64 LLG step and of get_field, its
 * energy -1/2 m.B_dip per atom to the total energy (Hamiltonian/energy.f90:286-291,
 * :372-374).  Open boundaries: every pair of the supercell, no periodic images.
 *   do_dip = 0  off;
 *   do_dip = 1  brute force, the tensor of dipoleMatrix (dipolecommon.f90:51-84) for every
 *               pair, as setup_qdip (dipolecommon.f90:114-143) builds it from coord
 *               (3, natom), in units of alat; with coord NULL the coordinates are those of
 *               the cell grid below;
 *   do_dip = 3  FFT (geometrical_DFFT_wrapper, fftdipole_fftw.f90:51-78): the same sum as a
 *               convolution over the cell grid zero-padded to 2 N - 1 cells per axis;
 *               needs na, n1, n2, n3 with na*n1*n2*n3 == natom, site I0 + NA (I1 + N1 (I2 +
 *               N2 I3)) at I1 C1 + I2 C2 + I3 C3 + Bas(I0); cell holds the rows C1, C2, C3
 *               and bas (3, na) the basis, both Cartesian in units of alat.  cuFFT is
 *               loaded at run time: -6 when it cannot be.
 * alat in metres (the field is 1e-7 mub / alat^3 (3 R R^T - R^2 I) / R^5 . m).  Only on
 * the FP64 path (precision 0; -7 otherwise).  Monte Carlo (mc_run, mc_run_temps, pt_run)
 * takes it as the reference does: Metropolis adds the field of the sweep's start to the
 * external field of the energy change (montecarlo.f90:216-231); the heat bath has it in
 * the site field, evaluated again before each colour of the checkerboard.  The structured
 * square heat bath and the learned moves return -7 while it is on. */
int uppasd_gpu_set_dipole(uppasd_gpu_sim *s, int32_t do_dip, double alat, const double *coord, int32_t na,
                          int32_t n1, int32_t n2, int32_t n3, const double *cell, const double *bas);

/* Caller-provided N(0,1) numbers for the next `nsteps` steps, laid out as
 * nsteps consecutive (3, natom, mensemble) blocks (the order the reference's
 * fill_rngarray draws them).  Selects gpu_rng = 1 until exhausted. */
int uppasd_gpu_set_noise(uppasd_gpu_sim *s, const double *normals, int64_t nsteps);

/* nsteps full LLG steps (field, predictor, field, corrector, moment update). */
int uppasd_gpu_sd_run(uppasd_gpu_sim *s, int64_t nsteps);

/* One block of the reference's step loop from and to host arrays: the same result as
 * put_moments(emom_in) + sd_run(nsteps) + get_moments(emom_out, emomM_out), any of the
 * three arrays NULL to skip it.  On the structured path (precision 1, 2) with
 * mensemble > 1 and page-locked arrays, the ensembles are split into up to eight groups,
 * each copied in, stepped and copied out on its own stream, so that one group's host
 * copies run while the others step; otherwise the three calls run in turn.  The call
 * returns (on success or on an error) after every copy it issued has finished, so the
 * caller's arrays are free again. */
int uppasd_gpu_sd_run_io(uppasd_gpu_sim *s, const double *emom_in, int64_t nsteps, double *emom_out,
                         double *emomM_out);

/* Measurement callback: the state after `step` steps, emom and emomM in the reference
 * layout (3, natom, mensemble), library-owned host memory valid during the call.  A
 * nonzero return stops the run. */
typedef int (*uppasd_gpu_measure_cb)(int64_t step, const double *emom, const double *emomM, void *user);

/* nsteps LLG steps with a measurement every `every` steps (the measure() cadence of
 * sd_mphase, sd_driver.f90:554-579; the reference's GPU path hands its measurements to a
 * host thread, gpu_files/measurementQueue.cpp:10-80).  The copy of each snapshot to the
 * host overlaps the next block of steps; the callbacks come in order on the calling
 * thread, each once the following block has been issued.  A nonzero callback value ends
 * the run after the block in flight and is returned: that block has run, so the state
 * then stands `every` steps past the snapshot of the callback that stopped it (and the
 * call returns once that block's snapshot copy has finished).  Steps beyond the last whole
 * block run without a measurement. */
int uppasd_gpu_sd_run_measured(uppasd_gpu_sim *s, int64_t nsteps, int64_t every, uppasd_gpu_measure_cb cb,
                               void *user);
/* Effective field of the current state, (3, natom, mensemble). */
int uppasd_gpu_get_field(uppasd_gpu_sim *s, double *beff);

/* Monte Carlo sweeps on a colouring of the coupling graph ('M' Metropolis with
 * Hinzke-Nowak trials, temperature >= 0 (at 0 only moves that do not raise the energy,
 * the relax entry of the reference's Python layer, pyasd.f90:255-298); 'H' heat bath,
 * temperature > 0). */
int uppasd_gpu_mc_run(uppasd_gpu_sim *s, char mode, double temperature, int64_t nsweeps);

/* Structured heat bath for a uniform square lattice of edge L (site i = x + L y;
 * exchange and DMI on x +- 1, y +- 1, uniform moment and Zeeman field, no
 * anisotropy; recognised from the arrays given at init, -7 otherwise): the
 * checkerboard chain of uppasd_gpu_mc_run 'H' with FP32 draws on the FP64 state,
 * all ensembles per launch. */
int uppasd_gpu_mc_run_square(uppasd_gpu_sim *s, int32_t L, double temperature, int64_t nsweeps);
/* The same with one temperature per ensemble (temps[mensemble], K): a temperature grid
 * swept in one launch per colour, as uppasd_gpu_mc_run_temps does on the general path. */
int uppasd_gpu_mc_run_square_temps(uppasd_gpu_sim *s, int32_t L, const double *temps, int64_t nsweeps);

/* Monte Carlo sweeps with one temperature per ensemble (temps[mensemble], K): the
 * chain of uppasd_gpu_mc_run with T taken per ensemble (on precision 3 and 4 the heat
 * bath draws in FP32 as there). */
int uppasd_gpu_mc_run_temps(uppasd_gpu_sim *s, char mode, const double *temps, int64_t nsweeps);

/* Parallel tempering of pt_iphase (pt_driver.f90:58-367) with the ensembles as its
 * replicas: heat-bath sweeps at temps[replica]; every pt_step sweeps during the
 * first 90 % of nsweeps, swap attempts between replica positions (r, r + 1),
 * r = 0, 2, ... then 1, 3, ..., accepted with min(1, exp((e_{r+1} - e_r)(b_{r+1} - b_r)))
 * on energies per atom (J) and b = 1 / kB / (T + 1e-15), one uniform per position
 * from the Philox stream (position, 0, sweep).  temps comes back permuted (the
 * temperature each replica ended with); selected = the replica of lowest energy,
 * the one pt_iphase continues from.  The replica energy is calc_energy's total,
 * which pt_iphase's effective_field energy equals except for the weight of the
 * cubic-anisotropy term. */
int uppasd_gpu_pt_run(uppasd_gpu_sim *s, double *temps, int64_t nsweeps, int32_t pt_step, int64_t *n_trial,
                      int64_t *n_hit, int32_t *selected);

/* Per-ensemble total moment (3, mensemble), |M|/natom (mensemble) and energy per
 * atom in mRy (mensemble); any output may be NULL. */
int uppasd_gpu_observables(uppasd_gpu_sim *s, double *mvec, double *mabs, double *energy);

/* Per-ensemble energy terms of calc_energy (Hamiltonian/energy.f90:60-405) in mRy per
 * atom, terms(5, mensemble) = {total, exchange (the pair energy with the tensor),
 * anisotropy, DM, Zeeman}: the ene%energy / ene_xc / ene_ani / ene_dm / ene_ext values
 * that totenergy.<simid>.out averages over the ensembles (:407-500).  With the dipolar
 * field on (uppasd_gpu_set_dipole), total includes ene_dip, which has no column here. */
int uppasd_gpu_energy_terms(uppasd_gpu_sim *s, double *terms);

/* Run the library's work on the caller's CUDA stream (a cudaStream_t passed as
 * void*); NULL returns to the library's own stream.  Replaces the reference's
 * two internal streams (cudaParallelizationHelper.hpp:88-175). */
int uppasd_gpu_set_stream(uppasd_gpu_sim *s, void *cuda_stream);
/* Profiling hook (the reference's StopwatchDeviceSync, gpu_files/stopwatchDeviceSync.hpp):
 * advances `nrep` steps launching kernel by kernel and returns the mean device
 * time per launch in ms, measured with CUDA events on the launching stream:
 * ms[0] predictor kernel, ms[1] corrector kernel, ms[2] whole step. */
int uppasd_gpu_time_kernels(uppasd_gpu_sim *s, int32_t nrep, double *ms);
/* Which path and data forms init chose (diagnostics; no counterpart in the reference):
 * info[0] precision, info[1] 1 on the structured stencil path, and on the FP32-gather
 * path (precision 3 / 4): info[2] site classes (0: the per-site lists are read),
 * info[3] distinct coupling rows, info[4] chemical types the exchange couplings are
 * looked up by (0: none; a random alloy whose couplings are a function of the
 * neighbours' types, with the types given in uppasd_gpu_arrays.species), info[5] 1
 * when one external-field entry serves every spin; info[6] device bytes the
 * simulation allocated; info[7] 0. */
int uppasd_gpu_path_info(uppasd_gpu_sim *s, int64_t *info);

/* Allocation-free magnetisation sums.  This entry point has no counterpart in
 * the reference; it is for callers that cannot call cudaMalloc: a host code
 * that manages device memory through its own pool or arena and forbids
 * allocations behind it, code that runs while a CUDA graph is being captured
 * elsewhere in the process, or an embedding runtime that reserves the whole
 * device up front.
 *   d_emomM : device array of full moments in the reference layout
 *             (3, natom, mensemble), FP64, owned by the caller;
 *   d_out   : device array (4, mensemble), owned by the caller: total moment
 *             x, y, z and |M| / natom per ensemble;
 *   cuda_stream : cudaStream_t as void* (NULL = legacy default stream).
 * It allocates nothing: its scratch is a fixed 192 KiB device array inside this
 * library, which every GPU that loads the library keeps until the process
 * exits.  Limit: mensemble <= 64 (larger values return UPPASD_GPU_EINVAL);
 * natom is not limited.  The first call on each device looks up that array's
 * device address (cudaGetSymbolAddress) with the device current, so make the
 * first call on a device before any stream capture.  The address is kept per
 * device context: after a cudaDeviceReset the next call on that device looks it
 * up again (that call, too, should come before any stream capture).  All calls share the
 * array: calls that overlap on the GPU (different streams) race and must be
 * serialised by the caller.  The result is asynchronous on `cuda_stream`. */
int uppasd_gpu_moment_sums_noalloc(const double *d_emomM, int32_t natom, int32_t mensemble, double *d_out,
                                   void *cuda_stream);

/* ---- Batched replica Monte Carlo ------------------------------------------
 * Many bcc J1/J2 Heisenberg replicas (temperatures x sizes, uneven atom counts)
 * swept together by one persistent cooperative launch, replayed from a captured
 * CUDA graph.  This is the replica table the reference's temperature loops feed
 * one system at a time: mc_mphase (MonteCarlo/mc_driver.f90:234-420) per
 * temperature, and the replica list of parallel tempering
 * (MonteCarlo/pt_driver.f90:58-367).  The single-spin updates are flip_h and
 * flip_a (MonteCarlo/montecarlo_common.f90:139-200, 371-422) over checkerboard
 * colours (sublattice x cell parity); observables are E (mRy/atom, as
 * calc_energy, Hamiltonian/energy.f90:60-405) and M (muB/atom, as calc_mavrg,
 * Measurement/measurements.f90:211-235) after every sweep, accumulated in FP64. */
typedef struct uppasd_gpu_mcbatch uppasd_gpu_mcbatch;

/* nrep replicas; replica r: L[r]^3 bcc cells (2 L^3 atoms, L even, 4..1024),
 * temperature[r] (K), heatbath[r] (1 heat bath, 0 Metropolis; NULL = all heat
 * bath).  j_shells_mry[2] = J1, J2 (mRy), mom = moment (muB), bfield[3] (T or
 * NULL).  Initial spins are uniform on the sphere from `seed`.  series_len > 0
 * keeps a ring buffer of (E, |M|) per replica and measured sweep;
 * max_sweeps_per_launch bounds the sweeps of one persistent launch. */
int uppasd_gpu_mcbatch_create(int32_t nrep, const int32_t *L, const double *temperature, const int32_t *heatbath,
                              const double *j_shells_mry, double mom, const double *bfield, uint64_t seed,
                              int32_t series_len, int32_t max_sweeps_per_launch, uppasd_gpu_mcbatch **out);
int uppasd_gpu_mcbatch_destroy(uppasd_gpu_mcbatch *b);
int uppasd_gpu_mcbatch_set_stream(uppasd_gpu_mcbatch *b, void *cuda_stream);
/* Schedule: register build of the sweep kernel (0: unconstrained, 1: sized for 3
 * CTAs per SM, 2: for 4), threads per CTA (multiple of 32, <= 256) and CTAs per
 * replica (>= 1 each, total within the co-resident limit). */
int uppasd_gpu_mcbatch_set_schedule(uppasd_gpu_mcbatch *b, int32_t reg_build, int32_t threads,
                                    const int32_t *ctas_per_rep);
int uppasd_gpu_mcbatch_get_schedule(uppasd_gpu_mcbatch *b, int32_t *reg_build, int32_t *threads,
                                    int32_t *ctas_per_rep);
/* Autotuner: times register builds, block sizes and CTAs per SM, rebalances the CTAs per replica
 * from per-group times, installs the fastest; cached per device and replica
 * table in cache_path (NULL = no cache).  Its sweeps are real sweeps (the chain
 * advances; use it during thermalisation). */
int uppasd_gpu_mcbatch_autotune(uppasd_gpu_mcbatch *b, int32_t sweeps_per_trial, const char *cache_path,
                                float *best_ms_per_sweep);
/* nsweeps sweeps in graph replays of sweeps_per_launch; measure != 0 adds every
 * sweep to the moments and the series.  Synchronises and checks the barrier
 * error flag. */
int uppasd_gpu_mcbatch_run(uppasd_gpu_mcbatch *b, int64_t nsweeps, int32_t sweeps_per_launch, int32_t measure);
/* Same, asynchronous on the batch's stream; uppasd_gpu_mcbatch_check synchronises. */
int uppasd_gpu_mcbatch_enqueue(uppasd_gpu_mcbatch *b, int64_t nsweeps, int32_t sweeps_per_launch, int32_t measure);
int uppasd_gpu_mcbatch_check(uppasd_gpu_mcbatch *b);
/* acc (nrep, 10): n, sum E, E^2, |M|, M^2, M^4, Mx, My, Mz, |M|^3 over measured sweeps;
 * nsample (nrep); last (nrep, 4): E, Mx, My, Mz after the latest sweep.  Any may be NULL. */
int uppasd_gpu_mcbatch_stats(uppasd_gpu_mcbatch *b, double *acc, int64_t *nsample, double *last);
/* (nrep, series_len, 2) ring buffer of (E, |M|); sample k of replica r at k % series_len. */
int uppasd_gpu_mcbatch_series(uppasd_gpu_mcbatch *b, double *series);
int uppasd_gpu_mcbatch_reset_stats(uppasd_gpu_mcbatch *b);
/* Unit spins, replica-major, each in the reference layout (3, 2 L^3), site b + 2 (x + L (y + L z)). */
int uppasd_gpu_mcbatch_get_spins(uppasd_gpu_mcbatch *b, double *emom);
int uppasd_gpu_mcbatch_put_spins(uppasd_gpu_mcbatch *b, const double *emom);
/* Sweep counter (the Philox step of the next sweep). */
int uppasd_gpu_mcbatch_set_sweep(uppasd_gpu_mcbatch *b, int64_t sweep);
/* This batch as a contiguous share of a larger replica table (one share per GPU;
 * the reference's replica loop, pt_driver.f90:58-367, has no such split): its
 * replica r draws its Philox numbers, and its initial state, as replica
 * first_id + r of the whole table, so every replica's chain is the same whichever
 * GPU runs it.  Redraws the initial state; call right after create. */
int uppasd_gpu_mcbatch_set_replica_ids(uppasd_gpu_mcbatch *b, int32_t first_id);
/* Poll limit of the replica-group barrier's wait (0 = the default, beyond any real
 * wait).  A wait that runs past it records an error and its group leaves the
 * launch; run/check then return UPPASD_GPU_ESTATE and reset the barrier state, so the
 * batch stays usable (its spins are those the groups had reached).  Whatever the
 * poll limit, a wait also gives up after about two seconds.  For testing the error path:
 * a limit of 1 makes every CTA of a group of two or more give up at the group's first
 * barrier, on arrival (so no CTA waits for another and the outcome does not depend on
 * timing). */
int uppasd_gpu_mcbatch_set_spin_limit(uppasd_gpu_mcbatch *b, int64_t limit);
/* Replica exchange (the swap step of MonteCarlo/pt_driver.f90:58-367 on the batch):
 * after every launch, replicas holding adjacent temperatures of one size swap
 * their temperatures with probability min(1, exp((beta_a - beta_b)(E_a - E_b))),
 * even and odd ladder pairs alternately.  Statistics and series then belong to
 * the temperature slots (the original replica order of temperature[]); spins
 * stay with their replica. */
int uppasd_gpu_mcbatch_set_exchange(uppasd_gpu_mcbatch *b, int32_t enable);
/* slot_of_rep (nrep), ladder pairs of slots (npairs x 2), attempts and accepts per
 * pair; any output may be NULL, *npairs is always written. */
int uppasd_gpu_mcbatch_exchange_state(uppasd_gpu_mcbatch *b, int32_t *slot_of_rep, int32_t *npairs,
                                      int32_t *pairs, int64_t *attempts, int64_t *accepts);

/* ---- BF16 tensor-core GEMM (tcgen05, TMEM accumulator, TMA operands) -------
 * No counterpart in the reference: the dense contraction of the learned patch
 * proposal.  C (M x N) = A (M x K) B (N x K)^T on host buffers (bf16 as raw
 * uint16 bit patterns, row-major), FP32 accumulation; M % 128 == 0, K % 64 == 0,
 * N % bn == 0, bn in {64, 128, 256}.  epilogue: 0 Cf = AB^T; 1 Cf = AB^T + bias;
 * 2 Cb = tanh(AB^T + bias) in bf16; 3 Cb = AB^T * (1 - Y^2) in bf16 (Y: M x N bf16). */
int uppasd_gpu_tc_gemm(int32_t M, int32_t N, int32_t K, const uint16_t *A, const uint16_t *B, const float *bias,
                       const uint16_t *Y, int32_t epilogue, int32_t bn, float *Cf, uint16_t *Cb);
/* Self-test of the tensor-core pipeline's bounded waits: one CTA waits, with the
 * wait the GEMM uses, on an mbarrier that nothing arrives at.  Expected result:
 * UPPASD_GPU_ESTATE with the message "a pipeline wait ran past its limit (code 4)"
 * after about a second (the limit of every wait of the pipeline), the context still usable.  No copy or MMA is in
 * flight during the wait.  No counterpart in the reference. */
int uppasd_gpu_tc_wait_selftest(void);

/* ---- Learned 4x4-patch proposal with exact Metropolis-Hastings -------------
 * No counterpart in the reference; it acts beside the heat bath of mc_mphase
 * (uppasd_gpu_mc_run) on the same simulation's spins.  The simulation must be
 * an L x L square lattice, one atom per cell, site i = x + L y, L % 8 == 0 and
 * Mensemble * (L/8)^2 a multiple of 128.  Network: MADE over the patch's four
 * sub-lattice groups; input the 8 x 8 window (192 features), 3 tanh layers of
 * 256, output eta = kappa mu per patch spin (48 of 64 used), eta = eta_scale *
 * output; BF16 tensor-core GEMMs with FP32 accumulation.  data_capacity = rows
 * of the training-window buffer (0 = none).  Parameter vector layout: W1
 * (256 x 192), W2, W3 (256 x 256), W4 (64 x 256), b1, b2, b3 (256), b4 (64). */
typedef struct uppasd_gpu_proposal uppasd_gpu_proposal;
int uppasd_gpu_proposal_create(uppasd_gpu_sim *s, int32_t L, float eta_scale, int32_t data_capacity, uint64_t seed,
                               uppasd_gpu_proposal **out);
int uppasd_gpu_proposal_destroy(uppasd_gpu_proposal *p);
int uppasd_gpu_proposal_nparams(uppasd_gpu_proposal *p, int64_t *n);
int uppasd_gpu_proposal_get_params(uppasd_gpu_proposal *p, float *params);
/* Rejects parameter vectors whose masked (non-autoregressive) weights are non-zero. */
int uppasd_gpu_proposal_set_params(uppasd_gpu_proposal *p, const float *params);
/* The 0/1 autoregressive masks of W1..W4 (weights part of the parameter layout). */
int uppasd_gpu_proposal_get_masks(uppasd_gpu_proposal *p, float *masks);
/* Network outputs (rows x 64) for explicit windows (rows x 192, fp32, rounded to bf16). */
int uppasd_gpu_proposal_forward(uppasd_gpu_proposal *p, const float *x, int32_t rows, float *out);
/* Mean negative log-likelihood of the windows' patches and its gradient (parameter layout). */
int uppasd_gpu_proposal_loss_grad(uppasd_gpu_proposal *p, const float *x, int32_t rows, double *loss,
                                  float *grad);
/* Append the windows of every patch of every chain of the simulation's current spins. */
int uppasd_gpu_proposal_collect(uppasd_gpu_proposal *p);
/* nsteps Adam steps on random minibatches of `rows` collected windows; losses[nsteps] or NULL. */
int uppasd_gpu_proposal_train(uppasd_gpu_proposal *p, int32_t nsteps, int32_t rows, float lr, double *losses);
/* nsweeps learned sweeps (each: the four patch colours) at `temperature` (K) on the
 * simulation's spins; counts of accepted and proposed patch moves and the summed
 * energy change of accepted moves (J). */
int uppasd_gpu_proposal_sweep(uppasd_gpu_proposal *p, double temperature, int64_t nsweeps, int64_t *accepted,
                              int64_t *proposed, double *dE_accepted);
/* ncycles of (hb_per_cycle sweeps of uppasd_gpu_mc_run_square, then one learned
 * sweep), enqueued back to back (the learned sweep replayed from a captured CUDA
 * graph) with one synchronisation at the end; counts as for proposal_sweep. */
int uppasd_gpu_proposal_mix(uppasd_gpu_proposal *p, double temperature, int64_t ncycles, int32_t hb_per_cycle,
                            int64_t *accepted, int64_t *proposed, double *dE_accepted);
/* The same with one temperature per ensemble (temps[mensemble], K), for the heat-bath
 * sweeps and for every learned move's acceptance: a temperature grid in one learned
 * sweep.  The network is shared by all temperatures; the acceptance stays exact. */
int uppasd_gpu_proposal_mix_temps(uppasd_gpu_proposal *p, const double *temps, int64_t ncycles,
                                  int32_t hb_per_cycle, int64_t *accepted, int64_t *proposed, double *dE_accepted);

#ifdef __cplusplus
}
#endif
#endif
