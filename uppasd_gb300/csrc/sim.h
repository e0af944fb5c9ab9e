// sim.h -- internal state of one simulation (one Hamiltonian, Mensemble spin
// replicas) on one GB300.  Not part of the public C ABI (include/uppasd_gpu.h).
//
// HBM layout (all device arrays, ensemble-major structure of arrays):
//   spin component c of site i in ensemble k lives at  c_array[k * natom + i];
//   x, y, z are separate arrays so a warp's loads of one component coalesce.
//   The reference's Fortran (3, natom, mensemble) AoS arrays are converted at
//   the boundary by the transpose kernels in abi.cu.
//   Neighbour lists are stored slot-major ("transposed ELL"): slot s of site i
//   at nlist[s * natom + i], 0-based, so consecutive sites read consecutive words.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <string>

#include "../../include/uppasd_gpu.h"
#include "common.cuh"

namespace uppasd {

struct Vec3D {
    double *x = nullptr, *y = nullptr, *z = nullptr;
};

struct HamDev {
    int natom = 0, mensemble = 0, mnn = 0, nham = 0;
    int32_t *nlist = nullptr;   // [mnn][natom] 0-based
    int32_t *nsize = nullptr;   // [natom] = nlistsize(aham(i))
    int32_t *aham = nullptr;    // [natom] 0-based
    double *ncoup = nullptr;    // [mnn][nham]
    int do_dm = 0, mnn_dm = 0;
    int32_t *dmlist = nullptr;  // [mnn_dm][natom]
    int32_t *dmsize = nullptr;  // [natom]
    double *dmx = nullptr, *dmy = nullptr, *dmz = nullptr;  // [mnn_dm][nham]
    int do_aniso = 0;
    int32_t *taniso = nullptr;  // [natom]
    double *eax = nullptr, *eay = nullptr, *eaz = nullptr;  // [natom]
    double *k1 = nullptr, *k2 = nullptr, *sb = nullptr;     // [natom]
    Vec3D ext;                  // [mensemble][natom]
    // exchange tensor (do_jtensor = 1): J_ab of slot s, Hamiltonian index ih at
    // jt[(s * nham + ih) * 9 + 3 a + b]; replaces ncoup in fields and energies
    int do_jtensor = 0;
    double *jt = nullptr;
    // the caller's physical constants (fortrandata_setconstants_ passes gama, k_bolt and
    // mub): SI by default, all 1 under aunits = 'Y' (Input/inputhandler.f90:1685-1704)
    double gama = kGama, kbolt = kKbolt, mub = kMub, mry = kMry;
    // dipole-dipole field (do_dip 1 brute force, 3 FFT): dip holds the field of the
    // moments the caller last evaluated it for, added first in site_field
    int do_dip = 0;
    Vec3D dip;                  // [mensemble][natom]
};

struct LlgDev {
    int sdealgh = 5;
    double delta_t = 1e-16, bn = 1.0, temprescale = 1.0;
    double relaxtime = 0.0;  // SDEalgh 11: relaxation time of the inertial regime (s)
    int perp = 0;            // input perp = 'Y': field projected perpendicular to emom
    double *lambda = nullptr, *temp = nullptr, *landeg = nullptr;  // [natom]
    double *mmom = nullptr;  // [mensemble][natom]
    uint64_t seed = 0;
    int noise_mode = 0;            // 0 Philox, 1 injected normals, 2 none
    int noise_on = 1;              // midpoint/SIB draw noise only when min(lambda) > 1e-12
    double *inj = nullptr;         // injected N(0,1): [nsteps][3][mensemble][natom]
    int64_t inj_steps = 0, inj_first = 0;
    int64_t *d_step = nullptr;     // device step counter (read by kernels, advanced in-stream)
};

struct DipoleDev;       // dipolar field state (dipole.cu)
struct StructuredFast;  // mixed-precision structured-lattice path (llg_stencil.cu)

// precision 3 (llg_mixed.cu): FP32 gather over the caller's neighbour lists with
// the FP64 state e / eM as master.  mt mirrors e (unit vector, w = moment), mp is
// the predictor, b2 the Depondt predictor's damped field.
struct MixedDev {
    float4 *mt = nullptr, *mp = nullptr;
    float *b2x = nullptr, *b2y = nullptr, *b2z = nullptr;
    int valid = 0;  // mt equals e / mmom
    // FP32 copies of the Hamiltonian, one row per distinct coupling row: equal rows of a
    // non-reduced Hamiltonian (a translation-invariant lattice) share one, so the per-site
    // reads hit the caches instead of streaming per-site copies from DRAM
    int nrow = 0;            // distinct (exchange, DM, tensor) rows
    int32_t *row = nullptr;  // [natom] row of atom i
    float *nc = nullptr;     // [mnn][nrow]
    float4 *dm = nullptr;    // [mnn_dm][nrow] (Dx, Dy, Dz, 0)
    float *jt = nullptr;     // [mnn][nrow][9]
    int32_t *arow = nullptr; // [natom] anisotropy row of atom i
    float4 *an = nullptr;    // [distinct anisotropy rows] (ex, ey, ez, k1)
    float2 *an2 = nullptr;   // [distinct anisotropy rows] (k2, sb)
    float4 *ext = nullptr;   // [mensemble][natom] (Bx, By, Bz, 0), or one entry when uniform
    int ext_uniform = 0;     // every spin sees ext[0]
    // Site classes: sites with the same coupling row, anisotropy row and type, list sizes
    // and neighbour offsets j - i share one class, so a site reads one 4-byte class id
    // instead of its neighbour and DM lists, sizes and rows (a translation-invariant
    // lattice has a handful of classes: the interior and its periodic edges).  ncls = 0:
    // too many distinct sites, the per-site lists are read.
    int ncls = 0;
    int32_t *cls = nullptr;    // [natom] class of site i
    int4 *cinfo = nullptr;     // [ncls] (nn | nd << 16, coupling row, anisotropy row, anisotropy type)
    int32_t *cnb = nullptr;    // [ncls][mnn] exchange neighbour offsets j - i
    int32_t *cdm = nullptr;    // [ncls][mnn_dm] DM neighbour offsets j - i
    // Chemical resolution (a random alloy, where each site's exchange row depends on its
    // neighbours' chemical types): nsp > 0 when every scalar exchange coupling is a
    // function of (class, slot, chemical type of the neighbour); the classes then key on
    // the site's own type and geometry only, nc is [mnn][nrow][nsp] (nrow = ncls) and a
    // neighbour's coupling is indexed by spc[j].
    int nsp = 0;
    int8_t *spc = nullptr;     // [natom] chemical type, 0-based, when the caller gave one
    // per-site parameters that are the same everywhere are passed as scalars
    int uni_lam = 0, uni_g = 0, uni_T = 0, uni_m = 0;
    float lam_u = 0.f, g_u = 0.f, T_u = 0.f;
    double mmom_u = 0.0;       // moment of every (ensemble, site) when uni_m
    uint8_t *moved = nullptr;  // [mensemble][natom] Metropolis: mirror moved, FP64 state not yet
    // precision 4: the master is double-single, hi = the mirror, lo here; e / eM are made
    // from it when a caller reads them (e_stale: the steps have moved it since)
    int ds = 0, e_stale = 0;
    float *lox = nullptr, *loy = nullptr, *loz = nullptr;  // [mensemble][natom]
};

// Uniform square-lattice Hamiltonian recognised for the structured heat bath
// (mc_square.cu): per neighbour direction (+x, -x, +y, -y) the exchange field per
// unit neighbour and the DMI vector, uniform moment and Zeeman field.
struct SquareMC {
    int L = 0;          // 0: not recognised yet; -1: recognised as not square-uniform
    float c[4];         // ncoup * m (T per unit neighbour vector)
    float d[4][3];      // D * m (field e_j x d)
    float ext[3];       // Zeeman field (T)
    float mom;          // moment (muB)
};

struct Sim {
    HamDev ham;
    LlgDev llg;
    Vec3D e, eM;        // state at t: unit vectors and full moments
    Vec3D p, pM;        // predictor / midpoint estimate
    Vec3D b2;           // Depondt b2eff / Heun field at t
    Vec3D mpast;        // SDEalgh 11: m(t - dt), zero before the first step
    int64_t step = 0;   // host mirror of the step counter
    cudaStream_t stream = nullptr;      // stream all work is issued on
    cudaStream_t own_stream = nullptr;  // the library's stream while a caller's stream is set
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    int device = 0;
    int precision = 0;  // 0 FP64 generic, 1 / 2 structured, 3 / 4 FP32 gather with FP64 / double-single master
    StructuredFast *fast = nullptr;
    // MC
    int ncolour = 0;
    int32_t *colour_sites = nullptr;   // sites listed colour by colour
    int32_t *colour_start_h = nullptr; // host copy, ncolour+1
    int64_t mc_sweep = 0;
    SquareMC sq;
    // FP32 mirror of the unit spins (x, y, z, 0), [mensemble][natom], for the structured
    // square heat bath and the learned patch moves: the heat bath writes its draws to it
    // and makes e / eM from it at the end of a call, the learned moves write every update
    // to both it and e / eM; any other writer of e marks it stale.
    float4 *sqm = nullptr;
    int sqm_valid = 0;
    MixedDev mix;
    DipoleDev *dip = nullptr;
    // (3, natom, mensemble) staging array of the host transfers, kept between calls
    // measured runs: two device snapshot pairs (emom, emomM in the reference layout), their
    // page-locked host copies, a copy stream and the events that order them
    double *snap_d[2] = {nullptr, nullptr}, *snap_h[2] = {nullptr, nullptr};
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t snap_ev[2] = {nullptr, nullptr}, copy_ev[2] = {nullptr, nullptr};
    // pipelined host runs (sd_run_io): one stream and one completion event per ensemble group
    static constexpr int kIoGroups = 8;
    cudaStream_t io_stream[kIoGroups] = {};
    cudaEvent_t io_ev[kIoGroups] = {}, io_in[kIoGroups] = {}, io_start = nullptr;
    double *stage = nullptr;
    // per-ensemble temperatures of mc_run_temps / pt_run: K and muB / (kB T) (FP32)
    double *tk = nullptr;
    float *betak = nullptr;
    // scratch for observables
    double *red = nullptr;             // [mensemble][8]
    size_t bytes_allocated = 0;
};

}  // namespace uppasd

// the public handle of include/uppasd_gpu.h
struct uppasd_gpu_sim {
    uppasd::Sim s;
};

namespace uppasd {

// llg_generic.cu
// phase: 1 predictor only, 2 corrector only, 3 both
int llg_generic_step(Sim &s, int64_t step_offset, int phase = 3);
// observables.cu
// terms_h (optional): per ensemble {total, exchange (pair energy with the tensor),
// anisotropy, DM, Zeeman} in mRy per atom, the per-ensemble values of calc_energy.
int observables(Sim &s, double *mvec_h, double *mabs_h, double *energy_h, const Vec3D *src,
                double *terms_h = nullptr);
int field_to_host(Sim &s, double *beff_h);
// dipole.cu: set up (mode 0 removes), free, and enqueue the field of the full moments m
// into ham.dip
// coord (3, natom) or nullptr for the cell grid of na, n1..n3, cell (rows C1..C3), bas
int dipole_setup(Sim &s, int mode, double alat, const double *coord, int na, int n1, int n2, int n3,
                 const double *cell, const double *bas);
void dipole_free(Sim &s);
int dipole_field(Sim &s, const Vec3D &m);
// mc.cu
// tk: temperature per ensemble on the device (nullptr: `temperature` for all)
int mc_checkerboard_sweeps(Sim &s, char mode, double temperature, int64_t nsweeps, const double *tk = nullptr);
// mc_square.cu: recognise a uniform square-lattice Hamiltonian (fills s.sq)
int square_recognise(Sim &s, int L);
int square_mirror_ready(Sim &s);  // builds the FP32 mirror from e when it is stale
// structured heat-bath sweeps at one temperature, or per ensemble (betak on the device)
int square_sweeps(Sim &s, int L, double temperature, const float *betak, int64_t nsweeps);
// abi.cu: one temperature per ensemble (K) to s.tk and muB / (kB T) to s.betak
int set_ensemble_temps(Sim &s, const double *temps);
void set_error(const std::string &msg);
// the host-transfer staging array (allocated on first use); nullptr with the error set
inline double *stage_buffer(Sim &s) {
    if (!s.stage) {
        const size_t bytes = 3 * sizeof(double) * (size_t)s.ham.natom * s.ham.mensemble;
        if (cudaMalloc(&s.stage, bytes) != cudaSuccess) {
            s.stage = nullptr;
            set_error("staging array: cudaMalloc failed");
            return nullptr;
        }
        s.bytes_allocated += bytes;
    }
    return s.stage;
}
// every FP32 mirror of e is stale (a writer of e other than the mirror's own users)
inline void square_mirror_stale(Sim &s) {
    s.sqm_valid = 0;
    s.mix.valid = 0;
}
// precision 1 / 2: the structured bcc path owns the state between sync points
inline bool structured(const Sim &s) { return s.precision == 1 || s.precision == 2; }
// precision 3 / 4: FP32 gather over the caller's lists, FP64 (3) or double-single (4) master
inline bool mixed_path(const Sim &s) { return s.precision == 3 || s.precision == 4; }
// e / eM brought up to date from the master of the path that owns the state (abi.cu)
int sync_state(Sim &s);

void set_error(const std::string &msg);

#define UPPASD_CUDA_TRY(expr)                                                              \
    do {                                                                                   \
        cudaError_t _e = (expr);                                                           \
        if (_e != cudaSuccess) {                                                           \
            ::uppasd::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));       \
            return UPPASD_GPU_ECUDA;                                                       \
        }                                                                                  \
    } while (0)

}  // namespace uppasd
