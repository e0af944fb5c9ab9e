// abi.cu -- the C ABI (include/uppasd_gpu.h): set-up, layout conversion at the
// boundary, the step loop under a CUDA graph, and teardown.
//
// Ownership follows the reference's CUDA path (cudaMdSimulation.cu:133-243):
// the caller owns every host array; init copies what the hot path needs into
// device memory in the layout described in sim.h; get_moments copies the
// state back in the caller's Fortran layout.  Unlike the reference, nothing
// here exits the process: every failure returns a status code.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "common.cuh"
#include "sim.h"


namespace uppasd {

static thread_local std::string g_err;
void set_error(const std::string &msg) { g_err = msg; }

int structured_init(Sim &s, const uppasd_gpu_consts *c, const uppasd_gpu_arrays *a);  // llg_stencil.cu
int structured_step(Sim &s, int64_t step_offset, int phase);
int structured_set_temperature(Sim &s, const double *temp_array);
void structured_refresh(Sim &s);
int structured_sync_state(Sim &s);  // master state -> s.e / s.eM
int structured_load_range(Sim &s, const double *aos, int k0, int kn, cudaStream_t st);  // ensemble ranges
int structured_steps_range(Sim &s, int64_t nsteps, int k0, int kn, cudaStream_t st);
int structured_store_range(Sim &s, double *aos, int full, int k0, int kn, cudaStream_t st);
int structured_check_flag(Sim &s);
int structured_load_state(Sim &s);  // s.e -> master state
void structured_free(Sim &s);
int mixed_init(Sim &s, const int32_t *species);  // llg_mixed.cu
void mixed_free(Sim &s);
int mixed_ready(Sim &s);
int mixed_sync(Sim &s);  // precision 4: e / eM from the double-single master
int mixed_step(Sim &s, int64_t step_offset, int phase);
int mixed_heat_bath_sweeps(Sim &s, double temperature, int64_t nsweeps, const float *betak = nullptr);
int mixed_metropolis_sweeps(Sim &s, double temperature, int64_t nsweeps);
int mixed_coefficients(Sim &s);
void mixed_temperature(Sim &s, const double *temp_array);

// e / eM up to date from the master of the path that owns the state between calls
int sync_state(Sim &s) {
    if (structured(s)) return structured_sync_state(s);
    if (s.precision == 4) return mixed_sync(s);
    return UPPASD_GPU_OK;
}

static int io_streams(Sim &s) {
    if (s.io_start) return UPPASD_GPU_OK;
    cudaStream_t st[Sim::kIoGroups] = {};
    cudaEvent_t ev[Sim::kIoGroups] = {}, in[Sim::kIoGroups] = {}, start = nullptr;
    cudaError_t e = cudaEventCreateWithFlags(&start, cudaEventDisableTiming);
    // earlier groups at higher priority: their input arrives first, so they finish first
    // and their output copies run under the later groups' steps (measured 2-3 % faster per
    // block than equal priorities; the reverse order was slower)
    int lowest = 0, highest = 0;
    cudaDeviceGetStreamPriorityRange(&lowest, &highest);
    for (int g = 0; g < Sim::kIoGroups && e == cudaSuccess; ++g) {
        const int prio = highest + (lowest - highest) * g / (Sim::kIoGroups - 1);
        e = cudaStreamCreateWithPriority(&st[g], cudaStreamNonBlocking, prio);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[g], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&in[g], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        for (int g = 0; g < Sim::kIoGroups; ++g) {
            if (st[g]) cudaStreamDestroy(st[g]);
            if (ev[g]) cudaEventDestroy(ev[g]);
            if (in[g]) cudaEventDestroy(in[g]);
        }
        if (start) cudaEventDestroy(start);
        set_error(std::string("sd_run_io: streams: ") + cudaGetErrorString(e));
        return UPPASD_GPU_ECUDA;
    }
    for (int g = 0; g < Sim::kIoGroups; ++g) {
        s.io_stream[g] = st[g];
        s.io_ev[g] = ev[g];
        s.io_in[g] = in[g];
    }
    s.io_start = start;
    return UPPASD_GPU_OK;
}

namespace {

template <typename T>
int dalloc(Sim &s, T **p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        set_error(std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
        *p = nullptr;
        return UPPASD_GPU_ENOMEM;
    }
    s.bytes_allocated += n * sizeof(T);
    return UPPASD_GPU_OK;
}

template <typename T>
int upload(Sim &s, T **p, const std::vector<T> &h) {
    int rc = dalloc(s, p, h.size());
    if (rc) return rc;
    UPPASD_CUDA_TRY(cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return UPPASD_GPU_OK;
}

int alloc_vec3(Sim &s, Vec3D &v, size_t n) {
    int rc;
    if ((rc = dalloc(s, &v.x, n)) || (rc = dalloc(s, &v.y, n)) || (rc = dalloc(s, &v.z, n))) return rc;
    return UPPASD_GPU_OK;
}

void free_vec3(Vec3D &v) {
    cudaFree(v.x);
    cudaFree(v.y);
    cudaFree(v.z);
    v = Vec3D{};
}

__global__ void aos_to_soa(const double *aos, Vec3D e, Vec3D eM, const double *mmom, int64_t n) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    double x = aos[3 * t], y = aos[3 * t + 1], z = aos[3 * t + 2];
    double m = mmom[t];
    e.x[t] = x;
    e.y[t] = y;
    e.z[t] = z;
    eM.x[t] = x * m;
    eM.y[t] = y * m;
    eM.z[t] = z * m;
}

__global__ void soa_to_aos(Vec3D v, double *aos, int64_t n) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    aos[3 * t] = v.x[t];
    aos[3 * t + 1] = v.y[t];
    aos[3 * t + 2] = v.z[t];
}

// The same conversions one 256-site block at a time through shared memory, so that every
// warp access to the AoS side is one contiguous run of doubles: these read or write the
// caller's page-locked host buffer directly (over the CPU-GPU link, no staging copy).
__global__ void __launch_bounds__(256) aos_to_soa_blocked(const double *aos, Vec3D e, Vec3D eM, const double *mmom,
                                                          int64_t n) {
    __shared__ double buf[3 * 256];
    const int64_t base = (int64_t)blockIdx.x * 256;
    const int cnt = (int)(n - base < 256 ? n - base : 256);
    for (int q = threadIdx.x; q < 3 * cnt; q += 256) buf[q] = aos[3 * base + q];
    __syncthreads();
    if ((int)threadIdx.x >= cnt) return;
    const int64_t t = base + threadIdx.x;
    const double x = buf[3 * threadIdx.x], y = buf[3 * threadIdx.x + 1], z = buf[3 * threadIdx.x + 2];
    const double m = mmom[t];
    e.x[t] = x;
    e.y[t] = y;
    e.z[t] = z;
    eM.x[t] = x * m;
    eM.y[t] = y * m;
    eM.z[t] = z * m;
}

__global__ void __launch_bounds__(256) soa_to_aos_blocked(Vec3D v, double *aos, int64_t n) {
    __shared__ double buf[3 * 256];
    const int64_t base = (int64_t)blockIdx.x * 256;
    const int cnt = (int)(n - base < 256 ? n - base : 256);
    if ((int)threadIdx.x < cnt) {
        const int64_t t = base + threadIdx.x;
        buf[3 * threadIdx.x] = v.x[t];
        buf[3 * threadIdx.x + 1] = v.y[t];
        buf[3 * threadIdx.x + 2] = v.z[t];
    }
    __syncthreads();
    for (int q = threadIdx.x; q < 3 * cnt; q += 256) aos[3 * base + q] = buf[q];
}

// A device-usable address of `p` when it is page-locked host memory (cudaHostAlloc or
// cudaHostRegister: mapped under unified addressing); nullptr for pageable memory.
static void *mapped_host(const void *p) {
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return pa.type == cudaMemoryTypeHost ? pa.devicePointer : nullptr;
}

__global__ void advance_step(int64_t *d_step, int64_t n) { *d_step += n; }

int check_device(Sim &s) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_error(std::string("no CUDA device: ") + cudaGetErrorString(e));
        return UPPASD_GPU_ENODEV;
    }
    cudaDeviceProp p;
    e = cudaGetDeviceProperties(&p, dev);
    if (e != cudaSuccess) {
        set_error(std::string("cudaGetDeviceProperties: ") + cudaGetErrorString(e));
        return UPPASD_GPU_ENODEV;
    }
    if (!(p.major == 10 && p.minor == 3)) {
        char buf[160];
        snprintf(buf, sizeof(buf), "device %d is sm_%d%d; this library is built for sm_103a (GB300) only", dev,
                 p.major, p.minor);
        set_error(buf);
        return UPPASD_GPU_ENODEV;
    }
    s.device = dev;
    return UPPASD_GPU_OK;
}

// Colouring of the coupling graph so that same-colour sites share no bond.
// Tries the sublattices alone, then cell parity x sublattice (exact for the
// simple and bcc lattices with nearest and next-nearest shells), verifying each,
// and falls back to greedy colouring.
int build_colouring(Sim &s, const uppasd_gpu_consts *c, const std::vector<int32_t> &nlT,
                    const std::vector<int32_t> &nsize, const std::vector<int32_t> &dmT,
                    const std::vector<int32_t> &dmsize) {
    const int N = c->natom, mnn = c->max_no_neigh, mdm = c->do_dm ? c->max_no_dmneigh : 0;
    std::vector<int32_t> col(N, -1);
    auto ok = [&](const std::vector<int32_t> &cc) {
        for (int i = 0; i < N; ++i) {
            for (int q = 0; q < nsize[i]; ++q)
                if (cc[nlT[(size_t)q * N + i]] == cc[i]) return false;
            for (int q = 0; mdm && q < dmsize[i]; ++q)
                if (cc[dmT[(size_t)q * N + i]] == cc[i]) return false;
        }
        return true;
    };
    bool done = false;
    if (c->n1 > 0 && c->n2 > 0 && c->n3 > 0 && c->na > 0 && (int64_t)c->n1 * c->n2 * c->n3 * c->na == N) {
        // the sublattices alone (kagome, honeycomb, bcc with nearest neighbours only),
        // then sublattice x cell parity
        std::vector<int32_t> cand(N);
        for (int i = 0; i < N; ++i) cand[i] = i % c->na;
        if (c->na > 1 && ok(cand)) {
            col = cand;
            done = true;
        }
        for (int i = 0; i < N && !done; ++i) {
            int b = i % c->na, cell = i / c->na;
            int x = cell % c->n1, y = (cell / c->n1) % c->n2, z = cell / (c->n1 * c->n2);
            cand[i] = b * 2 + ((x + y + z) & 1);
        }
        if (!done && ok(cand)) {
            col = cand;
            done = true;
        }
    }
    if (!done) {
        std::vector<char> used;
        for (int i = 0; i < N; ++i) {
            used.assign(used.size(), 0);
            auto mark = [&](int j) {
                int cj = col[j];
                if (cj < 0) return;
                if ((size_t)cj >= used.size()) used.resize(cj + 1, 0);
                used[cj] = 1;
            };
            for (int q = 0; q < nsize[i]; ++q) mark(nlT[(size_t)q * N + i]);
            for (int q = 0; mdm && q < dmsize[i]; ++q) mark(dmT[(size_t)q * N + i]);
            int cc = 0;
            while ((size_t)cc < used.size() && used[cc]) ++cc;
            col[i] = cc;
        }
        if (!ok(col)) {
            set_error("colouring failed verification");
            return UPPASD_GPU_EINVAL;
        }
        (void)mnn;
    }
    int ncol = *std::max_element(col.begin(), col.end()) + 1;
    std::vector<int32_t> start(ncol + 1, 0), order;
    for (int i = 0; i < N; ++i) start[col[i] + 1]++;
    for (int q = 0; q < ncol; ++q) start[q + 1] += start[q];
    order.resize(N);
    std::vector<int32_t> fill(start.begin(), start.end() - 1);
    for (int i = 0; i < N; ++i) order[fill[col[i]]++] = i;
    // drop empty colours
    std::vector<int32_t> st2{0};
    for (int q = 0; q < ncol; ++q)
        if (start[q + 1] > start[q]) st2.push_back(start[q + 1]);
    s.ncolour = (int)st2.size() - 1;
    s.colour_start_h = new (std::nothrow) int32_t[st2.size()];
    if (!s.colour_start_h) return UPPASD_GPU_ENOMEM;
    std::copy(st2.begin(), st2.end(), s.colour_start_h);
    return upload(s, &s.colour_sites, order);
}

int validate(const uppasd_gpu_consts *c, const uppasd_gpu_arrays *a) {
    auto bad = [](const char *m) {
        set_error(m);
        return UPPASD_GPU_EINVAL;
    };
    if (!c || !a) return bad("null consts or arrays");
    if (c->natom <= 0 || c->mensemble <= 0) return bad("natom and mensemble must be positive");
    if ((int64_t)c->natom * c->mensemble > (int64_t)1 << 31) return bad("natom*mensemble exceeds 2^31");
    if (c->max_no_neigh < 0 || c->nham <= 0 || c->nham > c->natom) return bad("bad max_no_neigh or nham");
    if (!a->nlist || !a->nlistsize || !a->ncoup || !a->aham || !a->mmom || !a->lambda1_array || !a->temp_array ||
        !a->emom || !a->external_field)
        return bad("required array missing");
    if (c->do_dm && (!a->dmlist || !a->dmlistsize || !a->dm_vect || c->max_no_dmneigh <= 0))
        return bad("do_dm set but DM arrays missing");
    if (c->do_aniso && (!a->taniso || !a->eaniso || !a->kaniso)) return bad("do_aniso set but anisotropy arrays missing");
    if (!(c->sdealgh == 1 || c->sdealgh == 4 || c->sdealgh == 5 || c->sdealgh == 6 || c->sdealgh == 7 ||
          c->sdealgh == 11))
        return bad("SDEalgh must be 1, 4, 5, 6, 7 or 11");
    if (!(c->delta_t > 0.0) || !(c->bn > 0.0)) return bad("delta_t and bn must be positive");
    if (c->gpu_rng != 0 && c->gpu_rng != 1) return bad("gpu_rng must be 0 (Philox) or 1 (injected)");
    if (c->precision < 0 || c->precision > 4) return bad("precision must be 0, 1, 2, 3 or 4");
    for (int i = 0; i < c->natom; ++i)
        if (a->aham[i] < 1 || a->aham[i] > c->nham) return bad("aham out of range");
    for (int h = 0; h < c->nham; ++h) {
        if (a->nlistsize[h] < 0 || a->nlistsize[h] > c->max_no_neigh) return bad("nlistsize out of range");
        if (c->do_dm && (a->dmlistsize[h] < 0 || a->dmlistsize[h] > c->max_no_dmneigh))
            return bad("dmlistsize out of range");
    }
    for (int i = 0; i < c->natom; ++i) {
        int ih = a->aham[i] - 1;
        for (int q = 0; q < a->nlistsize[ih]; ++q) {
            int j = a->nlist[q + (size_t)c->max_no_neigh * i];
            if (j < 1 || j > c->natom) return bad("nlist entry out of range");
        }
        if (c->do_dm)
            for (int q = 0; q < a->dmlistsize[ih]; ++q) {
                int j = a->dmlist[q + (size_t)c->max_no_dmneigh * i];
                if (j < 1 || j > c->natom) return bad("dmlist entry out of range");
            }
        if (c->do_aniso) {
            int t = a->taniso[i];
            if (t != 0 && t != 1 && t != 2 && t != 7) return bad("taniso must be 0, 1, 2 or 7");
        }
    }
    for (int64_t t = 0; t < (int64_t)c->natom * c->mensemble; ++t)
        if (!(a->mmom[t] > 0.0)) return bad("mmom must be positive");
    return UPPASD_GPU_OK;
}

int do_init(Sim &s, const uppasd_gpu_consts *c, const uppasd_gpu_arrays *a) {
    int rc = validate(c, a);
    if (rc) return rc;
    if ((rc = check_device(s))) return rc;
    UPPASD_CUDA_TRY(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking));
    const int N = c->natom, M = c->mensemble, mnn = c->max_no_neigh, nham = c->nham;
    const size_t NM = (size_t)N * M;
    HamDev &h = s.ham;
    h.natom = N;
    h.mensemble = M;
    h.mnn = mnn;
    h.nham = nham;
    // neighbour lists, slot-major, 0-based, padded with the site itself
    std::vector<int32_t> nlT((size_t)std::max(mnn, 1) * N), nsize(N), aham0(N);
    std::vector<double> ncT((size_t)std::max(mnn, 1) * nham);
    for (int i = 0; i < N; ++i) {
        aham0[i] = a->aham[i] - 1;
        nsize[i] = a->nlistsize[aham0[i]];
        for (int q = 0; q < mnn; ++q)
            nlT[(size_t)q * N + i] = q < nsize[i] ? a->nlist[q + (size_t)mnn * i] - 1 : i;
    }
    for (int ih = 0; ih < nham; ++ih)
        for (int q = 0; q < mnn; ++q) ncT[(size_t)q * nham + ih] = a->ncoup[q + (size_t)mnn * ih];
    if ((rc = upload(s, &h.nlist, nlT)) || (rc = upload(s, &h.nsize, nsize)) || (rc = upload(s, &h.aham, aham0)) ||
        (rc = upload(s, &h.ncoup, ncT)))
        return rc;
    std::vector<int32_t> dmT, dmsize;
    if (c->do_dm) {
        const int mdm = c->max_no_dmneigh;
        h.do_dm = 1;
        h.mnn_dm = mdm;
        dmT.resize((size_t)mdm * N);
        dmsize.resize(N);
        std::vector<double> dx((size_t)mdm * nham), dy(dx.size()), dz(dx.size());
        for (int i = 0; i < N; ++i) {
            dmsize[i] = a->dmlistsize[aham0[i]];
            for (int q = 0; q < mdm; ++q)
                dmT[(size_t)q * N + i] = q < dmsize[i] ? a->dmlist[q + (size_t)mdm * i] - 1 : i;
        }
        for (int ih = 0; ih < nham; ++ih)
            for (int q = 0; q < mdm; ++q) {
                const double *d = &a->dm_vect[3 * (q + (size_t)mdm * ih)];
                dx[(size_t)q * nham + ih] = d[0];
                dy[(size_t)q * nham + ih] = d[1];
                dz[(size_t)q * nham + ih] = d[2];
            }
        if ((rc = upload(s, &h.dmlist, dmT)) || (rc = upload(s, &h.dmsize, dmsize)) || (rc = upload(s, &h.dmx, dx)) ||
            (rc = upload(s, &h.dmy, dy)) || (rc = upload(s, &h.dmz, dz)))
            return rc;
    }
    if (c->do_aniso) {
        h.do_aniso = 1;
        std::vector<int32_t> ta(a->taniso, a->taniso + N);
        std::vector<double> ex(N), ey(N), ez(N), k1(N), k2(N), sb(N, 0.0);
        for (int i = 0; i < N; ++i) {
            ex[i] = a->eaniso[3 * (size_t)i];
            ey[i] = a->eaniso[3 * (size_t)i + 1];
            ez[i] = a->eaniso[3 * (size_t)i + 2];
            k1[i] = a->kaniso[2 * (size_t)i];
            k2[i] = a->kaniso[2 * (size_t)i + 1];
            if (a->sb) sb[i] = a->sb[i];
        }
        if ((rc = upload(s, &h.taniso, ta)) || (rc = upload(s, &h.eax, ex)) || (rc = upload(s, &h.eay, ey)) ||
            (rc = upload(s, &h.eaz, ez)) || (rc = upload(s, &h.k1, k1)) || (rc = upload(s, &h.k2, k2)) ||
            (rc = upload(s, &h.sb, sb)))
            return rc;
    }
    {
        std::vector<double> ex(NM), ey(NM), ez(NM);
        for (size_t t = 0; t < NM; ++t) {
            ex[t] = a->external_field[3 * t];
            ey[t] = a->external_field[3 * t + 1];
            ez[t] = a->external_field[3 * t + 2];
        }
        if ((rc = upload(s, &h.ext.x, ex)) || (rc = upload(s, &h.ext.y, ey)) || (rc = upload(s, &h.ext.z, ez)))
            return rc;
    }
    // integrator parameters
    LlgDev &p = s.llg;
    p.sdealgh = c->sdealgh;
    p.delta_t = c->delta_t;
    p.bn = c->bn;
    p.temprescale = c->temprescale;
    p.seed = c->gpu_rng_seed;
    p.noise_mode = 0;
    {
        std::vector<double> lam(a->lambda1_array, a->lambda1_array + N), tmp(a->temp_array, a->temp_array + N);
        std::vector<double> g(N, 1.0);
        if (a->landeg) g.assign(a->landeg, a->landeg + N);
        std::vector<double> mm(a->mmom, a->mmom + NM);
        double lmin = *std::min_element(lam.begin(), lam.end());
        p.noise_on = lmin > 1e-12 ? 1 : 0;  // evolution.f90:143 (lambdatol)
        if ((rc = upload(s, &p.lambda, lam)) || (rc = upload(s, &p.temp, tmp)) || (rc = upload(s, &p.landeg, g)) ||
            (rc = upload(s, &p.mmom, mm)))
            return rc;
        std::vector<int64_t> st(1, 0);
        if ((rc = upload(s, &p.d_step, st))) return rc;
    }
    if ((rc = alloc_vec3(s, s.e, NM)) || (rc = alloc_vec3(s, s.eM, NM)) || (rc = alloc_vec3(s, s.p, NM)) ||
        (rc = alloc_vec3(s, s.pM, NM)) || (rc = alloc_vec3(s, s.b2, NM)) || (rc = dalloc(s, &s.red, (size_t)8 * M)))
        return rc;
    if (c->sdealgh == 11 && (rc = alloc_vec3(s, s.mpast, NM))) return rc;  // zeroed by put_moments
    if ((rc = build_colouring(s, c, nlT, nsize, dmT, dmsize))) return rc;
    s.precision = c->precision;
    if (structured(s)) {
        if ((rc = structured_init(s, c, a))) return rc;
    } else if (c->precision == 3 || c->precision == 4) {
        if ((rc = mixed_init(s, a->species))) return rc;
    }
    if ((rc = uppasd_gpu_put_moments(reinterpret_cast<uppasd_gpu_sim *>(&s), a->emom))) return rc;
    UPPASD_CUDA_TRY(cudaStreamSynchronize(s.stream));
    return UPPASD_GPU_OK;
}

void destroy(Sim &s) {
    if (s.stream) cudaStreamSynchronize(s.stream);
    if (s.copy_stream) cudaStreamSynchronize(s.copy_stream);  // a measured run's last copy
    if (s.graph) cudaGraphExecDestroy(s.graph);
    structured_free(s);
    mixed_free(s);
    dipole_free(s);
    HamDev &h = s.ham;
    void *ptrs[] = {h.nlist, h.nsize, h.aham, h.ncoup, h.jt, h.dmlist, h.dmsize, h.dmx, h.dmy, h.dmz, h.taniso,
                    h.eax, h.eay, h.eaz, h.k1, h.k2, h.sb, s.llg.lambda, s.llg.temp, s.llg.landeg, s.llg.mmom,
                    s.llg.inj, s.llg.d_step, s.red, s.colour_sites, s.sqm, s.stage, s.tk, s.betak};
    for (void *q : ptrs) cudaFree(q);
    for (int b = 0; b < 2; ++b) {
        cudaFree(s.snap_d[b]);
        cudaFreeHost(s.snap_h[b]);
        if (s.snap_ev[b]) cudaEventDestroy(s.snap_ev[b]);
        if (s.copy_ev[b]) cudaEventDestroy(s.copy_ev[b]);
    }
    if (s.copy_stream) cudaStreamDestroy(s.copy_stream);
    for (int g = 0; g < Sim::kIoGroups; ++g) {
        if (s.io_stream[g]) cudaStreamDestroy(s.io_stream[g]);
        if (s.io_ev[g]) cudaEventDestroy(s.io_ev[g]);
        if (s.io_in[g]) cudaEventDestroy(s.io_in[g]);
    }
    if (s.io_start) cudaEventDestroy(s.io_start);
    free_vec3(h.ext);
    free_vec3(s.e);
    free_vec3(s.eM);
    free_vec3(s.p);
    free_vec3(s.pM);
    free_vec3(s.b2);
    free_vec3(s.mpast);
    delete[] s.colour_start_h;
    if (s.own_stream) s.stream = s.own_stream;
    if (s.stream) cudaStreamDestroy(s.stream);
}

int one_step(Sim &s, int64_t off, int phase = 3) {
    if (structured(s)) return structured_step(s, off, phase);
    return mixed_path(s) ? mixed_step(s, off, phase) : llg_generic_step(s, off, phase);
}

int run_steps(Sim &s, int64_t n) {
    const int G = 16;
    int rc;
    if (mixed_path(s)) {
        s.sqm_valid = 0;  // the mixed steps keep their own mirror current
        if ((rc = mixed_ready(s))) return rc;
    } else {
        square_mirror_stale(s);
    }
    // structured path with several ensembles: the captured steps run as two independent
    // chains of ensemble halves on two streams, so the last partial wave of one half's
    // kernels fills with the other half's CTAs (the step 4-5 % shorter on the 100^3 alloy
    // x 8 than one chain; four or eight chains gained less)
    const int SG = structured(s) && s.ham.mensemble >= 2 ? 2 : 1;
    if (SG > 1 && (rc = io_streams(s))) return rc;
    // the FFT form of the dipolar field issues cuFFT launches, kept out of the captured graph
    if (!s.graph && n >= G && s.ham.do_dip != 3) {
        cudaGraph_t g;
        UPPASD_CUDA_TRY(cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal));
        if (SG > 1) {
            // fork and join through events, inside the capture
            UPPASD_CUDA_TRY(cudaEventRecord(s.io_start, s.stream));
            const int M = s.ham.mensemble;
            for (int q = 0; q < SG; ++q) {
                const int k0 = (int)((int64_t)M * q / SG), kn = (int)((int64_t)M * (q + 1) / SG) - k0;
                UPPASD_CUDA_TRY(cudaStreamWaitEvent(s.io_stream[q], s.io_start, 0));
                if ((rc = structured_steps_range(s, G, k0, kn, s.io_stream[q]))) {
                    cudaStreamEndCapture(s.stream, &g);
                    return rc;
                }
                UPPASD_CUDA_TRY(cudaEventRecord(s.io_ev[q], s.io_stream[q]));
                UPPASD_CUDA_TRY(cudaStreamWaitEvent(s.stream, s.io_ev[q], 0));
            }
        } else {
            for (int j = 0; j < G; ++j)
                if ((rc = one_step(s, j))) {
                    cudaStreamEndCapture(s.stream, &g);
                    return rc;
                }
        }
        advance_step<<<1, 1, 0, s.stream>>>(s.llg.d_step, G);
        UPPASD_CUDA_TRY(cudaStreamEndCapture(s.stream, &g));
        cudaError_t e = cudaGraphInstantiate(&s.graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            s.graph = nullptr;
            set_error(std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
            return UPPASD_GPU_ECUDA;
        }
        s.graph_steps = G;
    }
    int64_t done = 0;
    if (s.graph)
        for (; done + s.graph_steps <= n; done += s.graph_steps) UPPASD_CUDA_TRY(cudaGraphLaunch(s.graph, s.stream));
    int64_t rem = n - done;
    if (rem > 0 && SG > 1) {
        // the steps a graph does not cover as the same two chains, launched directly
        UPPASD_CUDA_TRY(cudaEventRecord(s.io_start, s.stream));
        const int M = s.ham.mensemble;
        for (int q = 0; q < SG; ++q) {
            const int k0 = (int)((int64_t)M * q / SG), kn = (int)((int64_t)M * (q + 1) / SG) - k0;
            UPPASD_CUDA_TRY(cudaStreamWaitEvent(s.io_stream[q], s.io_start, 0));
            if ((rc = structured_steps_range(s, rem, k0, kn, s.io_stream[q]))) return rc;
            UPPASD_CUDA_TRY(cudaEventRecord(s.io_ev[q], s.io_stream[q]));
            UPPASD_CUDA_TRY(cudaStreamWaitEvent(s.stream, s.io_ev[q], 0));
        }
    } else {
        for (int64_t j = 0; j < rem; ++j)
            if ((rc = one_step(s, j))) return rc;
    }
    if (rem > 0) advance_step<<<1, 1, 0, s.stream>>>(s.llg.d_step, rem);
    UPPASD_CUDA_TRY(cudaGetLastError());
    s.step += n;
    return UPPASD_GPU_OK;
}

void drop_graph(Sim &s) {
    if (s.graph) {
        cudaStreamSynchronize(s.stream);
        cudaGraphExecDestroy(s.graph);
        s.graph = nullptr;
    }
}

}  // namespace
}  // namespace uppasd

using uppasd::Sim;

extern "C" {

const char *uppasd_gpu_last_error(void) { return uppasd::g_err.c_str(); }

int uppasd_gpu_device_info(int32_t *sm_count, int32_t *cc_major, int32_t *cc_minor, int64_t *hbm_bytes) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    cudaDeviceProp p;
    if (e == cudaSuccess) e = cudaGetDeviceProperties(&p, dev);
    if (e != cudaSuccess) {
        uppasd::set_error(std::string("no CUDA device: ") + cudaGetErrorString(e));
        return UPPASD_GPU_ENODEV;
    }
    if (sm_count) *sm_count = p.multiProcessorCount;
    if (cc_major) *cc_major = p.major;
    if (cc_minor) *cc_minor = p.minor;
    if (hbm_bytes) *hbm_bytes = (int64_t)p.totalGlobalMem;
    return UPPASD_GPU_OK;
}

int uppasd_gpu_init(const uppasd_gpu_consts *c, const uppasd_gpu_arrays *a, uppasd_gpu_sim **out) {
    if (!out) {
        uppasd::set_error("out is NULL");
        return UPPASD_GPU_EINVAL;
    }
    *out = nullptr;
    uppasd_gpu_sim *w = new (std::nothrow) uppasd_gpu_sim();
    if (!w) {
        uppasd::set_error("host allocation failed");
        return UPPASD_GPU_ENOMEM;
    }
    int rc = uppasd::do_init(w->s, c, a);
    if (rc) {
        uppasd::destroy(w->s);
        delete w;
        return rc;
    }
    *out = w;
    return UPPASD_GPU_OK;
}

int uppasd_gpu_finalize(uppasd_gpu_sim *w) {
    if (!w) return UPPASD_GPU_EINVAL;
    uppasd::destroy(w->s);
    delete w;
    return UPPASD_GPU_OK;
}

int uppasd_gpu_put_moments(uppasd_gpu_sim *w, const double *emom) {
    if (!w || !emom) {
        uppasd::set_error("null argument");
        return UPPASD_GPU_EINVAL;
    }
    Sim &s = w->s;
    uppasd::square_mirror_stale(s);
    s.mix.e_stale = 0;  // e is written whole here: it is the state from now on
    const int64_t n = (int64_t)s.ham.natom * s.ham.mensemble;
    const unsigned grid = (unsigned)((n + 255) / 256);
    cudaError_t e = cudaSuccess;
    if (const double *h = static_cast<const double *>(uppasd::mapped_host(emom))) {
        // page-locked caller buffer: the conversion kernel reads it in place
        uppasd::aos_to_soa_blocked<<<grid, 256, 0, s.stream>>>(h, s.e, s.eM, s.llg.mmom, n);
        e = cudaGetLastError();
    } else {
        double *d = uppasd::stage_buffer(s);
        if (!d) return UPPASD_GPU_ENOMEM;
        e = cudaMemcpyAsync(d, emom, 3 * n * sizeof(double), cudaMemcpyHostToDevice, s.stream);
        if (e == cudaSuccess) {
            uppasd::aos_to_soa<<<grid, 256, 0, s.stream>>>(d, s.e, s.eM, s.llg.mmom, n);
            e = cudaGetLastError();
        }
    }
    // SDEalgh 11: a new state has no previous step (the reference's mpast starts at zero, llgi.f90:295)
    for (double *q : {s.mpast.x, s.mpast.y, s.mpast.z})
        if (e == cudaSuccess && q) e = cudaMemsetAsync(q, 0, n * sizeof(double), s.stream);
    if (e == cudaSuccess && uppasd::structured(s)) {
        int rc = uppasd::structured_load_state(s);
        if (rc) {
            cudaStreamSynchronize(s.stream);  // the caller's buffer is free on return, error or not
            return rc;
        }
    }
    // the caller may reuse its buffer once this returns
    if (e == cudaSuccess) e = cudaStreamSynchronize(s.stream);
    if (e != cudaSuccess) {
        uppasd::set_error(std::string("put_moments: ") + cudaGetErrorString(e));
        return UPPASD_GPU_ECUDA;
    }
    return UPPASD_GPU_OK;
}

int uppasd_gpu_get_moments(uppasd_gpu_sim *w, double *emom, double *emomM) {
    if (!w) {
        uppasd::set_error("null sim");
        return UPPASD_GPU_EINVAL;
    }
    Sim &s = w->s;
    int rc;
    if ((rc = uppasd::sync_state(s))) return rc;
    const int64_t n = (int64_t)s.ham.natom * s.ham.mensemble;
    cudaError_t e = cudaSuccess;
    const unsigned grid = (unsigned)((n + 255) / 256);
    auto copy_out = [&](const uppasd::Vec3D &v, double *out) {
        if (double *h = static_cast<double *>(uppasd::mapped_host(out))) {
            // page-locked caller buffer: the conversion kernel writes it in place
            uppasd::soa_to_aos_blocked<<<grid, 256, 0, s.stream>>>(v, h, n);
            return cudaGetLastError();
        }
        double *d = uppasd::stage_buffer(s);
        if (!d) return cudaErrorMemoryAllocation;
        uppasd::soa_to_aos<<<grid, 256, 0, s.stream>>>(v, d, n);
        return cudaMemcpyAsync(out, d, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, s.stream);
    };
    if (emom) e = copy_out(s.e, emom);
    if (e == cudaSuccess && emomM) e = copy_out(s.eM, emomM);  // stream order keeps the staging array safe
    if (e == cudaSuccess) e = cudaStreamSynchronize(s.stream);
    if (e != cudaSuccess) {
        uppasd::set_error(std::string("get_moments: ") + cudaGetErrorString(e));
        return UPPASD_GPU_ECUDA;
    }
    return UPPASD_GPU_OK;
}

int uppasd_gpu_set_temperature(uppasd_gpu_sim *w, const double *temp_array) {
    if (!w || !temp_array) return UPPASD_GPU_EINVAL;
    Sim &s = w->s;
    if (uppasd::structured(s)) {
        // the structured kernels take the thermal amplitude by value
        int rc = uppasd::structured_set_temperature(s, temp_array);
        if (rc) return rc;
        uppasd::drop_graph(s);
    }
    if (uppasd::mixed_path(s)) {
        uppasd::mixed_temperature(s, temp_array);
        uppasd::drop_graph(s);  // the uniform temperature is a step argument, captured by value
    }
    UPPASD_CUDA_TRY(cudaMemcpyAsync(s.llg.temp, temp_array, sizeof(double) * s.ham.natom, cudaMemcpyHostToDevice,
                                    s.stream));
    UPPASD_CUDA_TRY(cudaStreamSynchronize(s.stream));
    return UPPASD_GPU_OK;
}

int uppasd_gpu_set_perp(uppasd_gpu_sim *w, int32_t perp) {
    if (!w || (perp != 0 && perp != 1)) {
        uppasd::set_error("set_perp: perp must be 0 or 1");
        return UPPASD_GPU_EINVAL;
    }
    Sim &s = w->s;
    if (perp && uppasd::structured(s)) {
        uppasd::set_error("set_perp: the structured path (precision 1, 2) has no field projection");
        return UPPASD_GPU_EUNSUPPORTED;
    }
    uppasd::drop_graph(s);  // the step arguments are captured by value
    s.llg.perp = perp;
    return UPPASD_GPU_OK;
}

int uppasd_gpu_set_units(uppasd_gpu_sim *w, double gama, double k_bolt, double mub, double mry) {
    if (!w) return UPPASD_GPU_EINVAL;
    for (double v : {gama, k_bolt, mub, mry})
        if (!std::isfinite(v) || !(v > 0.0)) {
            uppasd::set_error("set_units: gama, k_bolt, mub and mry must be finite and > 0");
            return UPPASD_GPU_EINVAL;
        }
    Sim &s = w->s;
    uppasd::drop_graph(s);  // the step arguments are captured by value
    s.ham.gama = gama;
    s.ham.kbolt = k_bolt;
    s.ham.mub = mub;
    s.ham.mry = mry;
    uppasd::structured_refresh(s);
    return UPPASD_GPU_OK;
}

int uppasd_gpu_set_relaxtime(uppasd_gpu_sim *w, double relaxtime) {
    if (!w || !std::isfinite(relaxtime) || relaxtime < 0.0) {
        uppasd::set_error("set_relaxtime: relaxtime must be finite and >= 0");
        return UPPASD_GPU_EINVAL;
    }
    Sim &s = w->s;
    uppasd::drop_graph(s);  // the step arguments are captured by value
    s.llg.relaxtime = relaxtime;
    return UPPASD_GPU_OK;
}

int uppasd_gpu_set_jtensor(uppasd_gpu_sim *w, const double *j_tens) {
    if (!w) return UPPASD_GPU_EINVAL;
    Sim &s = w->s;
    uppasd::HamDev &h = s.ham;
    if (uppasd::structured(s)) {
        uppasd::set_error("set_jtensor: the structured path (precision 1, 2) covers scalar exchange; use precision 0 or 3");
        return UPPASD_GPU_EUNSUPPORTED;
    }
    std::vector<double> jt;
    if (j_tens) {
        // Fortran j_tens(3,3,max_no_neigh,nHam): J_ab of slot q at a + 3 b + 9 (q + mnn ih)
        const int mnn = h.mnn, nham = h.nham;
        jt.resize((size_t)std::max(mnn, 1) * nham * 9, 0.0);
        for (int ih = 0; ih < nham; ++ih)
            for (int q = 0; q < mnn; ++q)
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) {
                        const double v = j_tens[a + 3 * b + 9 * (q + (size_t)mnn * ih)];
                        if (!std::isfinite(v)) {
                            uppasd::set_error("set_jtensor: non-finite tensor element");
                            return UPPASD_GPU_EINVAL;
                        }
                        jt[((size_t)q * nham + ih) * 9 + 3 * a + b] = v;
                    }
    }
    uppasd::drop_graph(s);
    UPPASD_CUDA_TRY(cudaStreamSynchronize(s.stream));
    cudaFree(h.jt);
    h.jt = nullptr;
    h.do_jtensor = 0;
    s.sq.L = 0;  // the structured square recognition no longer holds
    if (!j_tens) return uppasd::mixed_path(s) ? uppasd::mixed_coefficients(s) : UPPASD_GPU_OK;
    int rc = uppasd::upload(s, &h.jt, jt);
    if (rc) return rc;
    UPPASD_CUDA_TRY(cudaStreamSynchronize(s.stream));
    h.do_jtensor = 1;
    if (uppasd::mixed_path(s)) return uppasd::mixed_coefficients(s);
    return UPPASD_GPU_OK;
}

int uppasd_gpu_set_dipole(uppasd_gpu_sim *w, int32_t do_dip, double alat, const double *coord, int32_t na,
                          int32_t n1, int32_t n2, int32_t n3, const double *cell, const double *bas) {
    if (!w || (do_dip != 0 && do_dip != 1 && do_dip != 3)) {
        uppasd::set_error("set_dipole: do_dip 0 (off), 1 (brute force) or 3 (FFT)");
        return UPPASD_GPU_EINVAL;
    }
    Sim &s = w->s;
    if (do_dip) {
        if (s.precision != 0) {
            uppasd::set_error("set_dipole: the dipolar field runs on the FP64 path (precision 0)");
            return UPPASD_GPU_EUNSUPPORTED;
        }
        if (!(alat > 0.0) || !std::isfinite(alat)) {
            uppasd::set_error("set_dipole: alat must be finite and > 0");
            return UPPASD_GPU_EINVAL;
        }
        const bool grid = do_dip == 3 || !coord;
        if (grid && (!cell || !bas || na < 1 || n1 < 1 || n2 < 1 || n3 < 1 ||
                     (int64_t)na * n1 * n2 * n3 != s.ham.natom)) {
            uppasd::set_error("set_dipole: need coord, or cell, bas and NA * N1 * N2 * N3 == natom");
            return UPPASD_GPU_EINVAL;
        }
        auto finite = [](const double *v, size_t n) {
            for (size_t q = 0; q < n; ++q)
                if (!std::isfinite(v[q])) return false;
            return true;
        };
        if (grid ? !(finite(cell, 9) && finite(bas, 3 * (size_t)na)) : !finite(coord, 3 * (size_t)s.ham.natom)) {
            uppasd::set_error("set_dipole: non-finite coordinate");
            return UPPASD_GPU_EINVAL;
        }
        // the padded grids index in 32-bit FFT dimensions
        if (do_dip == 3 && (int64_t)(2 * n1 - 1) * (2 * n2 - 1) * (2 * n3 - 1) > (int64_t)1 << 31) {
            uppasd::set_error("set_dipole: padded grid too large");
            return UPPASD_GPU_EINVAL;
        }
    }
    uppasd::drop_graph(s);
    UPPASD_CUDA_TRY(cudaStreamSynchronize(s.stream));
    return uppasd::dipole_setup(s, do_dip, alat, do_dip == 1 ? coord : nullptr, na, n1, n2, n3, cell, bas);
}

int uppasd_gpu_set_step(uppasd_gpu_sim *w, int64_t step) {
    if (!w) return UPPASD_GPU_EINVAL;
    Sim &s = w->s;
    UPPASD_CUDA_TRY(cudaMemcpyAsync(s.llg.d_step, &step, sizeof(int64_t), cudaMemcpyHostToDevice, s.stream));
    UPPASD_CUDA_TRY(cudaStreamSynchronize(s.stream));
    s.step = step;
    return UPPASD_GPU_OK;
}

int uppasd_gpu_set_noise(uppasd_gpu_sim *w, const double *normals, int64_t nsteps) {
    if (!w) return UPPASD_GPU_EINVAL;
    Sim &s = w->s;
    uppasd::drop_graph(s);
    cudaFree(s.llg.inj);
    s.llg.inj = nullptr;
    s.llg.inj_steps = 0;
    if (!normals || nsteps <= 0) {
        s.llg.noise_mode = 0;
        return UPPASD_GPU_OK;
    }
    const size_t n = (size_t)nsteps * 3 * s.ham.natom * s.ham.mensemble;
    UPPASD_CUDA_TRY(cudaMalloc(&s.llg.inj, n * sizeof(double)));
    UPPASD_CUDA_TRY(cudaMemcpy(s.llg.inj, normals, n * sizeof(double), cudaMemcpyHostToDevice));
    s.llg.inj_steps = nsteps;
    s.llg.inj_first = s.step;
    s.llg.noise_mode = 1;
    return UPPASD_GPU_OK;
}

int uppasd_gpu_sd_run(uppasd_gpu_sim *w, int64_t nsteps) {
    if (!w || nsteps < 0) {
        uppasd::set_error("bad arguments");
        return UPPASD_GPU_EINVAL;
    }
    Sim &s = w->s;
    if (s.llg.noise_mode == 1 && (s.step < s.llg.inj_first || s.step + nsteps > s.llg.inj_first + s.llg.inj_steps)) {
        uppasd::set_error("injected noise does not cover the requested steps");
        return UPPASD_GPU_ESTATE;
    }
    return uppasd::run_steps(s, nsteps);
}

namespace uppasd {

// put + steps + get of the structured path, pipelined: the ensembles split into up to
// kIoGroups contiguous groups, each on its own stream copying its slice of the
// caller's (page-locked) arrays in, converting, stepping, converting and copying out,
// so one group's copies run under the other groups' steps.  Every group reads the
// same device step counter, advanced once at the end: the Philox counters, and so the
// results, are those of put_moments + sd_run + get_moments.
// One group of the pipelined block: its input slice in, its steps, its outputs back.
static int sd_run_io_group(Sim &s, double *stage, int g, int k0, int kn, const double *in, int64_t nsteps,
                           double *out, double *outM) {
    const int N = s.ham.natom;
    cudaStream_t st = s.io_stream[g];
    const size_t off = (size_t)k0 * N, cnt = (size_t)kn * N;
    int rc;
    // the input copies one after another in group order, so the first group has its
    // slice at the full host-link rate and starts stepping while the rest arrive
    UPPASD_CUDA_TRY(cudaStreamWaitEvent(st, g ? s.io_in[g - 1] : s.io_start, 0));
    UPPASD_CUDA_TRY(cudaMemcpyAsync(stage + 3 * off, in + 3 * off, 3 * cnt * sizeof(double), cudaMemcpyHostToDevice,
                                    st));
    UPPASD_CUDA_TRY(cudaEventRecord(s.io_in[g], st));
    // the staging slice straight into the structured state and back (the generic e / eM
    // are brought up to date by the next call that reads them)
    if ((rc = structured_load_range(s, stage, k0, kn, st)) || (rc = structured_steps_range(s, nsteps, k0, kn, st)))
        return rc;
    // the two outputs share the group's slice of the staging array in stream order
    for (auto [full, h] : {std::pair<int, double *>{0, out}, {1, outM}}) {
        if (!h) continue;
        if ((rc = structured_store_range(s, stage, full, k0, kn, st))) return rc;
        UPPASD_CUDA_TRY(cudaMemcpyAsync(h + 3 * off, stage + 3 * off, 3 * cnt * sizeof(double),
                                        cudaMemcpyDeviceToHost, st));
    }
    UPPASD_CUDA_TRY(cudaEventRecord(s.io_ev[g], st));
    UPPASD_CUDA_TRY(cudaStreamWaitEvent(s.stream, s.io_ev[g], 0));
    return UPPASD_GPU_OK;
}

static int sd_run_io_pipelined(Sim &s, const double *in, int64_t nsteps, double *out, double *outM) {
    int rc = io_streams(s);
    if (rc) return rc;
    double *stage = stage_buffer(s);
    if (!stage) return UPPASD_GPU_ENOMEM;
    square_mirror_stale(s);
    const int M = s.ham.mensemble;
    // groups: UPPASD_IO_GROUPS (1 .. kIoGroups) when set, else kIoGroups
    static const int groups = [] {
        const char *v = std::getenv("UPPASD_IO_GROUPS");
        const int n = v ? std::atoi(v) : Sim::kIoGroups;
        return n >= 1 && n <= Sim::kIoGroups ? n : (int)Sim::kIoGroups;
    }();
    const int G = std::min(M, groups);
    UPPASD_CUDA_TRY(cudaEventRecord(s.io_start, s.stream));
    for (int g = 0; g < G; ++g) {
        const int k0 = (int)((int64_t)M * g / G), kn = (int)((int64_t)M * (g + 1) / G) - k0;
        if ((rc = sd_run_io_group(s, stage, g, k0, kn, in, nsteps, out, outM))) {
            // nothing issued so far may still touch the caller's arrays once the call returns
            for (int q = 0; q <= g; ++q) cudaStreamSynchronize(s.io_stream[q]);
            return rc;
        }
    }
    advance_step<<<1, 1, 0, s.stream>>>(s.llg.d_step, nsteps);
    UPPASD_CUDA_TRY(cudaGetLastError());
    s.step += nsteps;
    UPPASD_CUDA_TRY(cudaStreamSynchronize(s.stream));
    return structured_check_flag(s);
}

// The measured-run resources (copy stream, two device and two page-locked snapshot
// buffers, their events), made into locals and installed in s only when every one
// of them exists, so that a failed set-up leaves nothing half-made behind and the
// next call tries again from the start.
int snapshot_setup(Sim &s, size_t bytes) {
    cudaStream_t cs = nullptr;
    double *dd[2] = {nullptr, nullptr}, *hh[2] = {nullptr, nullptr};
    cudaEvent_t se[2] = {nullptr, nullptr}, ce[2] = {nullptr, nullptr};
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
        e = cudaMalloc(&dd[b], bytes);
        if (e == cudaSuccess) e = cudaHostAlloc(&hh[b], bytes, cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&se[b], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ce[b], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(ce[b], cs);
    }
    if (e != cudaSuccess) {
        for (int b = 0; b < 2; ++b) {
            if (dd[b]) cudaFree(dd[b]);
            if (hh[b]) cudaFreeHost(hh[b]);
            if (se[b]) cudaEventDestroy(se[b]);
            if (ce[b]) cudaEventDestroy(ce[b]);
        }
        if (cs) cudaStreamDestroy(cs);
        set_error(std::string("sd_run_measured: snapshot buffers: ") + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? UPPASD_GPU_ENOMEM : UPPASD_GPU_ECUDA;
    }
    for (int b = 0; b < 2; ++b) {
        s.snap_d[b] = dd[b];
        s.snap_h[b] = hh[b];
        s.snap_ev[b] = se[b];
        s.copy_ev[b] = ce[b];
        s.bytes_allocated += bytes;
    }
    s.copy_stream = cs;
    return UPPASD_GPU_OK;
}

}  // namespace uppasd

int uppasd_gpu_sd_run_io(uppasd_gpu_sim *w, const double *emom_in, int64_t nsteps, double *emom_out,
                         double *emomM_out) {
    if (!w || nsteps < 0) {
        uppasd::set_error("bad arguments");
        return UPPASD_GPU_EINVAL;
    }
    Sim &s = w->s;
    // the pipelined form needs the structured path, an input, several ensembles and
    // page-locked caller arrays (copies from pageable memory do not overlap anything)
    bool pipelined = uppasd::structured(s) && emom_in && s.ham.mensemble > 1 && s.llg.noise_mode != 1 &&
                     uppasd::mapped_host(emom_in) &&
                     (!emom_out || uppasd::mapped_host(emom_out)) && (!emomM_out || uppasd::mapped_host(emomM_out));
    if (pipelined) return uppasd::sd_run_io_pipelined(s, emom_in, nsteps, emom_out, emomM_out);
    int rc;
    if (emom_in && (rc = uppasd_gpu_put_moments(w, emom_in))) return rc;
    if ((rc = uppasd_gpu_sd_run(w, nsteps))) return rc;
    if (emom_out || emomM_out) return uppasd_gpu_get_moments(w, emom_out, emomM_out);
    return UPPASD_GPU_OK;
}

int uppasd_gpu_sd_run_measured(uppasd_gpu_sim *w, int64_t nsteps, int64_t every, uppasd_gpu_measure_cb cb,
                               void *user) {
    if (!w || nsteps < 0 || every < 1 || !cb) {
        uppasd::set_error("sd_run_measured: nsteps >= 0, every >= 1 and a callback are required");
        return UPPASD_GPU_EINVAL;
    }
    Sim &s = w->s;
    if (s.llg.noise_mode == 1 && (s.step < s.llg.inj_first || s.step + nsteps > s.llg.inj_first + s.llg.inj_steps)) {
        uppasd::set_error("injected noise does not cover the requested steps");
        return UPPASD_GPU_ESTATE;
    }
    const int64_t n = (int64_t)s.ham.natom * s.ham.mensemble;
    const size_t bytes = 6 * sizeof(double) * (size_t)n;  // emom then emomM
    if (!s.copy_stream) {
        int src = uppasd::snapshot_setup(s, bytes);
        if (src) return src;
    }
    const unsigned grid = (unsigned)((n + 255) / 256);
    const int64_t nblocks = nsteps / every;
    int64_t pending_step = -1;
    int rc = UPPASD_GPU_OK;
    // Block i runs on the library's stream and leaves its snapshot in buffer i % 2; the copy
    // stream brings it to the host while block i + 1 runs; the callback of block i is made
    // once block i + 1 has been issued.
    for (int64_t i = 0; i <= nblocks && rc == UPPASD_GPU_OK; ++i) {
        const int b = (int)(i % 2);
        if (i < nblocks) {
            if ((rc = uppasd::run_steps(s, every))) break;
            if ((rc = uppasd::sync_state(s))) break;
            UPPASD_CUDA_TRY(cudaStreamWaitEvent(s.stream, s.copy_ev[b], 0));  // buffer b copied out
            uppasd::soa_to_aos<<<grid, 256, 0, s.stream>>>(s.e, s.snap_d[b], n);
            uppasd::soa_to_aos<<<grid, 256, 0, s.stream>>>(s.eM, s.snap_d[b] + 3 * n, n);
            UPPASD_CUDA_TRY(cudaGetLastError());
            UPPASD_CUDA_TRY(cudaEventRecord(s.snap_ev[b], s.stream));
            UPPASD_CUDA_TRY(cudaStreamWaitEvent(s.copy_stream, s.snap_ev[b], 0));
            UPPASD_CUDA_TRY(cudaMemcpyAsync(s.snap_h[b], s.snap_d[b], bytes, cudaMemcpyDeviceToHost, s.copy_stream));
            UPPASD_CUDA_TRY(cudaEventRecord(s.copy_ev[b], s.copy_stream));
        }
        if (pending_step >= 0) {
            const int pb = (int)((i - 1) % 2);
            UPPASD_CUDA_TRY(cudaEventSynchronize(s.copy_ev[pb]));
            const int r = cb(pending_step, s.snap_h[pb], s.snap_h[pb] + 3 * n, user);
            if (r != 0) rc = r;
        }
        pending_step = i < nblocks ? s.step : -1;
    }
    // a callback that stopped the run leaves the copy of the block issued after it in
    // flight: wait for it, so that the host buffers are quiet when this call returns
    if (rc != UPPASD_GPU_OK) cudaStreamSynchronize(s.copy_stream);
    if (rc == UPPASD_GPU_OK && nsteps % every) rc = uppasd::run_steps(s, nsteps % every);
    if (rc == UPPASD_GPU_OK) UPPASD_CUDA_TRY(cudaStreamSynchronize(s.stream));
    return rc;
}

int uppasd_gpu_get_field(uppasd_gpu_sim *w, double *beff) {
    if (!w || !beff) return UPPASD_GPU_EINVAL;
    Sim &s = w->s;
    int rc;
    if ((rc = uppasd::sync_state(s))) return rc;
    return uppasd::field_to_host(s, beff);
}

int uppasd_gpu_mc_run(uppasd_gpu_sim *w, char mode, double temperature, int64_t nsweeps) {
    // Metropolis also at T = 0 (only moves that do not raise the energy are taken, as flip_a
    // does with its + 1e-15); the heat bath needs T > 0
    if (!w || nsweeps < 0 || (mode != 'M' && mode != 'H') || !std::isfinite(temperature) ||
        !(mode == 'M' ? temperature >= 0.0 : temperature > 0.0)) {
        uppasd::set_error("mc_run: mode 'M' (temperature >= 0) or 'H' (temperature > 0), nsweeps >= 0");
        return UPPASD_GPU_EINVAL;
    }
    Sim &s = w->s;
    int rc;
    if ((rc = uppasd::sync_state(s))) return rc;
    // precision 3 / 4: heat bath and Metropolis in FP32 on the mirror
    if (uppasd::mixed_path(s))
        rc = mode == 'H' ? uppasd::mixed_heat_bath_sweeps(s, temperature, nsweeps)
                         : uppasd::mixed_metropolis_sweeps(s, temperature, nsweeps);
    else
        rc = uppasd::mc_checkerboard_sweeps(s, mode, temperature, nsweeps);
    if (rc) return rc;
    if (uppasd::structured(s)) return uppasd::structured_load_state(s);
    return UPPASD_GPU_OK;
}

}  // extern "C"

namespace uppasd {
namespace {
// per-ensemble temperatures (K) and muB / (kB T) to the device
int upload_temps(Sim &s, const double *temps) {
    const int M = s.ham.mensemble;
    for (int k = 0; k < M; ++k)
        if (!(temps[k] > 0.0) || !std::isfinite(temps[k])) {
            set_error("temperatures must be finite and > 0");
            return UPPASD_GPU_EINVAL;
        }
    if (!s.tk) {
        UPPASD_CUDA_TRY(cudaMalloc(&s.tk, M * sizeof(double)));
        UPPASD_CUDA_TRY(cudaMalloc(&s.betak, M * sizeof(float)));
    }
    std::vector<float> b(M);
    for (int k = 0; k < M; ++k) b[k] = (float)(s.ham.mub / (s.ham.kbolt * temps[k]));
    UPPASD_CUDA_TRY(cudaStreamSynchronize(s.stream));
    UPPASD_CUDA_TRY(cudaMemcpy(s.tk, temps, M * sizeof(double), cudaMemcpyHostToDevice));
    UPPASD_CUDA_TRY(cudaMemcpy(s.betak, b.data(), M * sizeof(float), cudaMemcpyHostToDevice));
    return UPPASD_GPU_OK;
}

}  // namespace

int set_ensemble_temps(Sim &s, const double *temps) { return upload_temps(s, temps); }

namespace {
int sweeps_with_temps(Sim &s, char mode, int64_t nsweeps) {
    int rc;
    if ((rc = sync_state(s))) return rc;
    rc = mixed_path(s) && mode == 'H' ? mixed_heat_bath_sweeps(s, 0.0, nsweeps, s.betak)
                                         : mc_checkerboard_sweeps(s, mode, 0.0, nsweeps, s.tk);
    if (rc) return rc;
    if (structured(s)) return structured_load_state(s);
    return UPPASD_GPU_OK;
}
}  // namespace
}  // namespace uppasd

extern "C" {

int uppasd_gpu_mc_run_temps(uppasd_gpu_sim *w, char mode, const double *temps, int64_t nsweeps) {
    if (!w || !temps || nsweeps < 0 || (mode != 'M' && mode != 'H')) {
        uppasd::set_error("mc_run_temps: mode 'M' or 'H', one temperature per ensemble, nsweeps >= 0");
        return UPPASD_GPU_EINVAL;
    }
    Sim &s = w->s;
    int rc = uppasd::upload_temps(s, temps);
    return rc ? rc : uppasd::sweeps_with_temps(s, mode, nsweeps);
}

int uppasd_gpu_pt_run(uppasd_gpu_sim *w, double *temps, int64_t nsweeps, int32_t pt_step, int64_t *n_trial,
                      int64_t *n_hit, int32_t *selected) {
    if (!w || !temps || nsweeps < 0 || pt_step < 1) {
        uppasd::set_error("pt_run: one temperature per ensemble, nsweeps >= 0, pt_step >= 1");
        return UPPASD_GPU_EINVAL;
    }
    Sim &s = w->s;
    const int M = s.ham.mensemble;
    std::vector<double> T(temps, temps + M), E(M), u(M);
    int64_t trial = 0, hit = 0;
    int rc = uppasd::upload_temps(s, T.data());
    for (int64_t step = 1; step <= nsweeps && !rc; ++step) {
        if ((rc = uppasd::sweeps_with_temps(s, 'H', 1))) break;
        // swap attempts every pt_step sweeps during the first 90 % (pt_driver.f90:196-233)
        if (step % pt_step || step / (1.0 * nsweeps) >= 0.90) continue;
        if ((rc = uppasd::observables(s, nullptr, nullptr, E.data(), nullptr))) break;
        for (int r = 0; r < M; ++r) u[r] = uppasd::u01_open(uppasd::philox_draw(s.llg.seed, r, 0, step, uppasd::kStreamPT).x);
        bool swapped = false;
        for (int ishift = 0; ishift < 2; ++ishift)
            for (int r = ishift; r + 1 < M; r += 2) {
                ++trial;
                const double b1 = 1.0 / s.ham.kbolt / (T[r] + 1.0e-15), b2 = 1.0 / s.ham.kbolt / (T[r + 1] + 1.0e-15);
                const double e1 = E[r] * s.ham.mry, e2 = E[r + 1] * s.ham.mry;  // J per atom
                const double prob = std::min(1.0, exp((e2 - e1) * (b2 - b1)));
                if (u[r] <= prob) {
                    std::swap(T[r], T[r + 1]);
                    ++hit;
                    swapped = true;
                }
            }
        if (swapped) rc = uppasd::upload_temps(s, T.data());
    }
    if (!rc) rc = uppasd::observables(s, nullptr, nullptr, E.data(), nullptr);
    if (rc) return rc;
    int sel = 0;
    for (int r = 1; r < M; ++r)
        if (E[r] < E[sel]) sel = r;
    std::copy(T.begin(), T.end(), temps);
    if (n_trial) *n_trial = trial;
    if (n_hit) *n_hit = hit;
    if (selected) *selected = sel;
    return UPPASD_GPU_OK;
}

int uppasd_gpu_set_stream(uppasd_gpu_sim *w, void *cuda_stream) {
    if (!w) return UPPASD_GPU_EINVAL;
    Sim &s = w->s;
    uppasd::drop_graph(s);
    UPPASD_CUDA_TRY(cudaStreamSynchronize(s.stream));
    if (!s.own_stream) s.own_stream = s.stream;
    s.stream = cuda_stream ? (cudaStream_t)cuda_stream : s.own_stream;
    return UPPASD_GPU_OK;
}

int uppasd_gpu_path_info(uppasd_gpu_sim *w, int64_t *info) {
    if (!w || !info) return UPPASD_GPU_EINVAL;
    const Sim &s = w->s;
    const uppasd::MixedDev &m = s.mix;
    const bool mixed = uppasd::mixed_path(s);
    info[0] = s.precision;
    info[1] = uppasd::structured(s) ? 1 : 0;
    info[2] = mixed ? m.ncls : 0;
    info[3] = mixed ? m.nrow : 0;
    info[4] = mixed ? m.nsp : 0;
    info[5] = mixed ? m.ext_uniform : 0;
    info[6] = (int64_t)s.bytes_allocated;
    info[7] = 0;
    return UPPASD_GPU_OK;
}

int uppasd_gpu_time_kernels(uppasd_gpu_sim *w, int32_t nrep, double *ms) {
    if (!w || nrep <= 0 || !ms) return UPPASD_GPU_EINVAL;
    Sim &s = w->s;
    if (s.llg.noise_mode == 1 && (s.step < s.llg.inj_first || s.step + nrep > s.llg.inj_first + s.llg.inj_steps)) {
        uppasd::set_error("injected noise does not cover the requested steps");
        return UPPASD_GPU_ESTATE;
    }
    cudaEvent_t ev[3];
    for (auto &e : ev) UPPASD_CUDA_TRY(cudaEventCreate(&e));
    double acc[3] = {0.0, 0.0, 0.0};
    int rc = UPPASD_GPU_OK;
    if (uppasd::mixed_path(s)) {
        s.sqm_valid = 0;
        if ((rc = uppasd::mixed_ready(s))) return rc;
    } else {
        uppasd::square_mirror_stale(s);
    }
    for (int r = 0; r < nrep && rc == UPPASD_GPU_OK; ++r) {
        cudaEventRecord(ev[0], s.stream);
        rc = uppasd::one_step(s, 0, 1);
        cudaEventRecord(ev[1], s.stream);
        if (rc == UPPASD_GPU_OK) rc = uppasd::one_step(s, 0, 2);
        cudaEventRecord(ev[2], s.stream);
        uppasd::advance_step<<<1, 1, 0, s.stream>>>(s.llg.d_step, 1);
        s.step += 1;
        cudaError_t e = cudaEventSynchronize(ev[2]);
        if (e != cudaSuccess) {
            uppasd::set_error(std::string("time_kernels: ") + cudaGetErrorString(e));
            rc = UPPASD_GPU_ECUDA;
            break;
        }
        float a = 0.f, b = 0.f;
        cudaEventElapsedTime(&a, ev[0], ev[1]);
        cudaEventElapsedTime(&b, ev[1], ev[2]);
        acc[0] += a;
        acc[1] += b;
        acc[2] += a + b;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    for (int q = 0; q < 3; ++q) ms[q] = acc[q] / nrep;
    return rc;
}

int uppasd_gpu_observables(uppasd_gpu_sim *w, double *mvec, double *mabs, double *energy) {
    if (!w) return UPPASD_GPU_EINVAL;
    Sim &s = w->s;
    int rc;
    if ((rc = uppasd::sync_state(s))) return rc;
    return uppasd::observables(s, mvec, mabs, energy, nullptr);
}

int uppasd_gpu_energy_terms(uppasd_gpu_sim *w, double *terms) {
    if (!w || !terms) return UPPASD_GPU_EINVAL;
    Sim &s = w->s;
    int rc;
    if ((rc = uppasd::sync_state(s))) return rc;
    return uppasd::observables(s, nullptr, nullptr, nullptr, nullptr, terms);
}

}  // extern "C"
