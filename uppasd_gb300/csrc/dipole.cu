// dipole.cu -- the dipole-dipole field on the FP64 path.
//
// The reference adds, before the short-range terms of every field evaluation, the
// field of all other moments (Hamiltonian/dipolemanager.f90:119-184):
//   do_dip = 1: brute force over every pair with the tensor of dipoleMatrix
//               (dipolecommon.f90:51-84): Q(R) = 1e-7 mub / alat^3 (3 R R^T - R^2 I) / R^5,
//               R in units of the lattice constant, zero below R^2 = 1e-9;
//   do_dip = 3: the same sum as a convolution on the supercell's cell grid, zero-padded
//               to 2 N - 1 cells per axis (fftdipole_fftw.f90): FFT of the moments per
//               basis atom and component, a 3 x 3 tensor product per wave vector with the
//               transformed Q of every basis pair, inverse FFT.
// Both give the open-boundary sum (no periodic images).  Here:
//   * dip_direct: one thread per (site, ensemble, share of the sources); the j-loop reads
//     coordinates and moments in tiles staged in shared memory and adds
//     fac (3 (R.m) R - R^2 m) / R^5, the product Q m written out (about a third of the
//     FP64 operations of forming Q); the shares, which keep every SM busy on small
//     systems, are summed in a fixed order by dip_sum_shares;
//   * the FFT form with cuFFT (real-to-complex transforms of the padded grids, batched
//     over ensembles x basis atoms x components), the tensor product in dip_multiply,
//     the transformed tensors built once at set-up.  Any padded length P >= 2 N - 1 gives
//     the same linear convolution; P is the next length with no prime factor above 7, so
//     the transforms never fall back to a prime-length algorithm (2 N - 1 is 127 for
//     N = 64 and 199 for N = 100, both prime).  cuFFT is loaded at run time (dlopen), so
//     the library loads and runs without it; set_dipole(3) then reports it.
// The field lands in HamDev::dip, which site_field adds first, as the reference's
// effective_field_full does (hamiltonianactions.f90:173-181, 244).
#include <cufft.h>
#include <dlfcn.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "sim.h"

namespace uppasd {

struct DipoleDev {
    int mode = 0;
    int na = 0, n1 = 0, n2 = 0, n3 = 0;
    double fac = 0.0;               // 1e-7 mub / alat^3
    double *coord = nullptr;        // [natom][3], units of alat
    int shares = 1;                 // brute force: source shares per site
    double *part = nullptr;         // [shares][3][M][natom] partial fields when shares > 1
    // FFT form
    int p1 = 0, p2 = 0, p3 = 0;     // padded grid, >= 2 n - 1 per axis
    long long npad = 0, nc = 0;     // real and complex (half) grid sizes
    double *mr = nullptr, *fr = nullptr;            // [M][NA][3][npad]
    cufftDoubleComplex *mk = nullptr, *fk = nullptr; // [M][NA][3][nc]
    cufftDoubleComplex *kt = nullptr;                // [NA][NA][6][nc]
    cufftHandle pf = 0, pi = 0;
    bool pf_made = false, pi_made = false;  // each plan destroyed only if it was made
};

namespace {

// cuFFT entry points, resolved once at run time
struct CufftApi {
    bool tried = false, ok = false;
    cufftResult (*plan_many)(cufftHandle *, int, int *, int *, int, int, int *, int, int, cufftType, int) = nullptr;
    cufftResult (*exec_d2z)(cufftHandle, cufftDoubleReal *, cufftDoubleComplex *) = nullptr;
    cufftResult (*exec_z2d)(cufftHandle, cufftDoubleComplex *, cufftDoubleReal *) = nullptr;
    cufftResult (*set_stream)(cufftHandle, cudaStream_t) = nullptr;
    cufftResult (*destroy)(cufftHandle) = nullptr;
};
CufftApi g_fft;
std::mutex g_fft_mu;

bool cufft_load() {
    std::lock_guard<std::mutex> lk(g_fft_mu);
    if (g_fft.tried) return g_fft.ok;
    g_fft.tried = true;
    void *h = nullptr;
    for (const char *name : {"libcufft.so.12", "libcufft.so"})
        if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) return false;
    g_fft.plan_many = reinterpret_cast<decltype(g_fft.plan_many)>(dlsym(h, "cufftPlanMany"));
    g_fft.exec_d2z = reinterpret_cast<decltype(g_fft.exec_d2z)>(dlsym(h, "cufftExecD2Z"));
    g_fft.exec_z2d = reinterpret_cast<decltype(g_fft.exec_z2d)>(dlsym(h, "cufftExecZ2D"));
    g_fft.set_stream = reinterpret_cast<decltype(g_fft.set_stream)>(dlsym(h, "cufftSetStream"));
    g_fft.destroy = reinterpret_cast<decltype(g_fft.destroy)>(dlsym(h, "cufftDestroy"));
    g_fft.ok = g_fft.plan_many && g_fft.exec_d2z && g_fft.exec_z2d && g_fft.set_stream && g_fft.destroy;
    return g_fft.ok;
}

// dipoleMatrix: Q(nu, mu) of separation R (units of alat), fac = 1e-7 mub / alat^3
__host__ __device__ inline void dip_matrix(double fac, const double R[3], double Q[3][3]) {
    const double R2 = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
    if (!(R2 > 1e-9)) {
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) Q[a][b] = 0.0;
        return;
    }
    const double ir = 1.0 / sqrt(R2);
    const double Rm5 = (ir * ir) * (ir * ir) * ir * fac;
    for (int mu = 0; mu < 3; ++mu) {
        for (int nu = 0; nu < 3; ++nu) Q[nu][mu] = 3.0 * Rm5 * R[nu] * R[mu];
        Q[mu][mu] = Q[mu][mu] - Rm5 * R2;
    }
}

constexpr int kDipTile = 128;

// Brute force: B_i = sum_{j} fac (3 (R.m_j) R - R^2 m_j) / R^5, R = r_i - r_j, over the
// sources of share blockIdx.z; pairs with R^2 <= 1e-9 (the site itself) add nothing, as
// the zero diagonal of Qdip and the cut of dipoleMatrix do.
__global__ void __launch_bounds__(kDipTile) dip_direct(const double *__restrict__ coord, Vec3D m, Vec3D out,
                                                        double *part, int N, int M, int span, double fac) {
    __shared__ double sc[kDipTile][3], sm[kDipTile][3];
    const int k = blockIdx.y;
    const int i = blockIdx.x * kDipTile + threadIdx.x;
    const size_t off = (size_t)k * N;
    const int jbeg = blockIdx.z * span, jend = min(N, jbeg + span);
    double ri[3] = {0.0, 0.0, 0.0}, f[3] = {0.0, 0.0, 0.0};
    if (i < N)
        for (int q = 0; q < 3; ++q) ri[q] = coord[3 * (size_t)i + q];
    for (int j0 = jbeg; j0 < jend; j0 += kDipTile) {
        const int jj = j0 + threadIdx.x;
        __syncthreads();
        if (jj < jend) {
            for (int q = 0; q < 3; ++q) sc[threadIdx.x][q] = coord[3 * (size_t)jj + q];
            sm[threadIdx.x][0] = m.x[off + jj];
            sm[threadIdx.x][1] = m.y[off + jj];
            sm[threadIdx.x][2] = m.z[off + jj];
        } else {
            // padding sources: far away, no moment
            for (int q = 0; q < 3; ++q) sc[threadIdx.x][q] = 1e30;
            sm[threadIdx.x][0] = sm[threadIdx.x][1] = sm[threadIdx.x][2] = 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int t = 0; t < kDipTile; ++t) {
            const double R0 = ri[0] - sc[t][0], R1 = ri[1] - sc[t][1], R2c = ri[2] - sc[t][2];
            const double R2 = R0 * R0 + R1 * R1 + R2c * R2c;
            const double ir = rsqrt(fmax(R2, 1e-9));
            const double ir2 = ir * ir;
            const double rm5 = R2 > 1e-9 ? ir2 * ir2 * ir * fac : 0.0;
            const double rdm = R0 * sm[t][0] + R1 * sm[t][1] + R2c * sm[t][2];
            const double a = 3.0 * rdm * rm5, c = R2 * rm5;
            f[0] += a * R0 - c * sm[t][0];
            f[1] += a * R1 - c * sm[t][1];
            f[2] += a * R2c - c * sm[t][2];
        }
    }
    if (i >= N) return;
    if (gridDim.z == 1) {
        out.x[off + i] = f[0];
        out.y[off + i] = f[1];
        out.z[off + i] = f[2];
    } else {
        const size_t sh = (size_t)blockIdx.z * 3 * M * N;
        part[sh + off + i] = f[0];
        part[sh + (size_t)M * N + off + i] = f[1];
        part[sh + 2 * (size_t)M * N + off + i] = f[2];
    }
}

// the shares' partial fields summed in share order (the same result on every run)
__global__ void dip_sum_shares(const double *__restrict__ part, Vec3D out, long long nm, int shares) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nm) return;
    double f0 = 0.0, f1 = 0.0, f2 = 0.0;
    for (int s = 0; s < shares; ++s) {
        const double *p = part + (size_t)s * 3 * nm;
        f0 += p[t];
        f1 += p[nm + t];
        f2 += p[2 * nm + t];
    }
    out.x[t] = f0;
    out.y[t] = f1;
    out.z[t] = f2;
}

// Site i = I0 + NA (I1 + N1 (I2 + N2 I3)) -> padded cell index I1 + p1 (I2 + p2 I3)
__device__ __forceinline__ long long pad_index(const DipoleDev &d, int i, int &I0) {
    I0 = i % d.na;
    const int c = i / d.na;
    const int I1 = c % d.n1, I2 = (c / d.n1) % d.n2, I3 = c / (d.n1 * d.n2);
    return I1 + (long long)d.p1 * (I2 + (long long)d.p2 * I3);
}

// moments into the (pre-zeroed) padded grids: mr[((k NA + I0) 3 + c) npad + cell]
__global__ void dip_pad(DipoleDev d, Vec3D m, int N, int M) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * M) return;
    const int k = (int)(t / N), i = (int)(t - (long long)k * N);
    int I0;
    const long long cell = pad_index(d, i, I0);
    const size_t base = ((size_t)k * d.na + I0) * 3;
    d.mr[(base + 0) * d.npad + cell] = m.x[t];
    d.mr[(base + 1) * d.npad + cell] = m.y[t];
    d.mr[(base + 2) * d.npad + cell] = m.z[t];
}

// separation of padded index I on an axis of n cells padded to p: I for I < n, I - p for
// I > p - n, none (no pair of sites is that far apart) in between.  With p = 2 n - 1 this
// is the reference's paddingShift (dipolecommon.f90:92-106) up to the sign, which the
// even tensor Q(-R) = Q(R) does not see.
__device__ __forceinline__ bool pad_sep(int I, int n, int p, int &s) {
    s = I < n ? I : I - p;
    return I < n || I > p - n;
}

// the padded, transform-ready tensor of one basis pair (a receiving, b source) and
// symmetric component s (xx, xy, xz, yy, yz, zz) at every grid point:
// Q(s1 C1 + s2 C2 + s3 C3 + Bas(a) - Bas(b)), zero where a separation is none
__global__ void dip_tensor(DipoleDev d, const double *cell, const double *bas, double *out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = (long long)d.na * d.na * d.npad;
    if (t >= total) return;
    const long long g = t % d.npad;
    const int ab = (int)(t / d.npad), a = ab / d.na, b = ab % d.na;
    const int I1 = (int)(g % d.p1), I2 = (int)((g / d.p1) % d.p2), I3 = (int)(g / ((long long)d.p1 * d.p2));
    int s1, s2, s3;
    const bool in = pad_sep(I1, d.n1, d.p1, s1) & pad_sep(I2, d.n2, d.p2, s2) & pad_sep(I3, d.n3, d.p3, s3);
    double R[3];
    for (int q = 0; q < 3; ++q)
        R[q] = s1 * cell[q] + s2 * cell[3 + q] + s3 * cell[6 + q] + bas[3 * a + q] - bas[3 * b + q];
    double Q[3][3];
    dip_matrix(d.fac, R, Q);
    if (!in)
        for (int x = 0; x < 3; ++x)
            for (int y = 0; y < 3; ++y) Q[x][y] = 0.0;
    const double v[6] = {Q[0][0], Q[0][1], Q[0][2], Q[1][1], Q[1][2], Q[2][2]};
    for (int s = 0; s < 6; ++s) out[((size_t)ab * 6 + s) * d.npad + g] = v[s];
}

__device__ __forceinline__ int sym6(int nu, int mu) {
    const int lo = nu < mu ? nu : mu, hi = nu < mu ? mu : nu;
    return lo == 0 ? hi : (lo == 1 ? 2 + hi : 5);
}

// F_{k,a,nu}(q) = sum_b sum_mu K_{a,b,nu mu}(q) M_{k,b,mu}(q): one thread per (a, q), the
// ensembles in turn, so a thread's tensors are read from DRAM once and then from L1
__global__ void dip_multiply(DipoleDev d, int M) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)d.na * d.nc) return;
    const long long q = t % d.nc;
    const int a = (int)(t / d.nc);
    for (int k = 0; k < M; ++k) {
        double fr[3] = {0.0, 0.0, 0.0}, fi[3] = {0.0, 0.0, 0.0};
        for (int b = 0; b < d.na; ++b) {
            cufftDoubleComplex mv[3], kv[6];
            for (int mu = 0; mu < 3; ++mu) mv[mu] = d.mk[(((size_t)k * d.na + b) * 3 + mu) * d.nc + q];
            for (int s = 0; s < 6; ++s) kv[s] = d.kt[(((size_t)a * d.na + b) * 6 + s) * d.nc + q];
#pragma unroll
            for (int nu = 0; nu < 3; ++nu)
#pragma unroll
                for (int mu = 0; mu < 3; ++mu) {
                    const cufftDoubleComplex kc = kv[sym6(nu, mu)];
                    fr[nu] += kc.x * mv[mu].x - kc.y * mv[mu].y;
                    fi[nu] += kc.x * mv[mu].y + kc.y * mv[mu].x;
                }
        }
        for (int nu = 0; nu < 3; ++nu) {
            cufftDoubleComplex o;
            o.x = fr[nu];
            o.y = fi[nu];
            d.fk[(((size_t)k * d.na + a) * 3 + nu) * d.nc + q] = o;
        }
    }
}

// the field of every site back from the padded grids, normalised by the grid size
__global__ void dip_unpad(DipoleDev d, Vec3D out, int N, int M) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * M) return;
    const int k = (int)(t / N), i = (int)(t - (long long)k * N);
    int I0;
    const long long cell = pad_index(d, i, I0);
    const size_t base = ((size_t)k * d.na + I0) * 3;
    const double s = 1.0 / (double)d.npad;
    out.x[t] = d.fr[(base + 0) * d.npad + cell] * s;
    out.y[t] = d.fr[(base + 1) * d.npad + cell] * s;
    out.z[t] = d.fr[(base + 2) * d.npad + cell] * s;
}

void dipole_release(DipoleDev &d) {
    if (d.pf_made) g_fft.destroy(d.pf);
    if (d.pi_made) g_fft.destroy(d.pi);
    for (void *q : {(void *)d.coord, (void *)d.part, (void *)d.mr, (void *)d.fr, (void *)d.mk, (void *)d.fk,
                    (void *)d.kt})
        cudaFree(q);
    d = DipoleDev{};
}

// the smallest length >= n with no prime factor above 7
int smooth_length(int n) {
    for (int p = std::max(n, 1);; ++p) {
        int r = p;
        for (int f : {2, 3, 5, 7})
            while (r % f == 0) r /= f;
        if (r == 1) return p;
    }
}

cudaError_t dip_alloc3(Vec3D &v, size_t n) {
    cudaError_t e = cudaMalloc(&v.x, n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&v.y, n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&v.z, n * sizeof(double));
    return e;
}

void dip_free3(Vec3D &v) {
    cudaFree(v.x);
    cudaFree(v.y);
    cudaFree(v.z);
    v = Vec3D{};
}

int plan3(cufftHandle *h, const DipoleDev &d, cufftType type, int batch) {
    int n[3] = {d.p3, d.p2, d.p1};
    const int idist = type == CUFFT_D2Z ? (int)d.npad : (int)d.nc;
    const int odist = type == CUFFT_D2Z ? (int)d.nc : (int)d.npad;
    if (g_fft.plan_many(h, 3, n, nullptr, 1, idist, nullptr, 1, odist, type, batch) != CUFFT_SUCCESS) {
        set_error("set_dipole: cuFFT plan creation failed");
        return UPPASD_GPU_ECUDA;
    }
    return UPPASD_GPU_OK;
}

}  // namespace

void dipole_free(Sim &s) {
    if (s.dip) {
        dipole_release(*s.dip);
        delete s.dip;
        s.dip = nullptr;
    }
    dip_free3(s.ham.dip);
    s.ham.do_dip = 0;
}

// The field of the full moments m into s.ham.dip (the caller enqueues it before each
// field evaluation).
int dipole_field(Sim &s, const Vec3D &m) {
    DipoleDev &d = *s.dip;
    const int N = s.ham.natom, M = s.ham.mensemble;
    if (d.mode == 1) {
        const int span = (int)(((long long)N + d.shares - 1) / d.shares);
        dip_direct<<<dim3((unsigned)((N + kDipTile - 1) / kDipTile), (unsigned)M, (unsigned)d.shares), kDipTile, 0,
                      s.stream>>>(d.coord, m, s.ham.dip, d.part, N, M, span, d.fac);
        if (d.shares > 1) {
            const long long nm = (long long)N * M;
            dip_sum_shares<<<(unsigned)((nm + 255) / 256), 256, 0, s.stream>>>(d.part, s.ham.dip, nm, d.shares);
        }
    } else {
        const long long nm = (long long)N * M;
        // the padding cells stay zero; cleared every call rather than trusting the transform
        // to leave its input untouched
        UPPASD_CUDA_TRY(cudaMemsetAsync(d.mr, 0, (size_t)M * d.na * 3 * d.npad * sizeof(double), s.stream));
        dip_pad<<<(unsigned)((nm + 255) / 256), 256, 0, s.stream>>>(d, m, N, M);
        if (g_fft.set_stream(d.pf, s.stream) != CUFFT_SUCCESS || g_fft.set_stream(d.pi, s.stream) != CUFFT_SUCCESS ||
            g_fft.exec_d2z(d.pf, d.mr, d.mk) != CUFFT_SUCCESS) {
            set_error("dipolar field: cuFFT forward transform failed");
            return UPPASD_GPU_ECUDA;
        }
        const long long nmul = (long long)d.na * d.nc;
        dip_multiply<<<(unsigned)((nmul + 255) / 256), 256, 0, s.stream>>>(d, M);
        if (g_fft.exec_z2d(d.pi, d.fk, d.fr) != CUFFT_SUCCESS) {
            set_error("dipolar field: cuFFT inverse transform failed");
            return UPPASD_GPU_ECUDA;
        }
        dip_unpad<<<(unsigned)((nm + 255) / 256), 256, 0, s.stream>>>(d, s.ham.dip, N, M);
    }
    UPPASD_CUDA_TRY(cudaGetLastError());
    return UPPASD_GPU_OK;
}

int dipole_setup(Sim &s, int mode, double alat, const double *coord_in, int na, int n1, int n2, int n3,
                 const double *cell, const double *bas) {
    dipole_free(s);
    if (mode == 0) return UPPASD_GPU_OK;
    const int N = s.ham.natom, M = s.ham.mensemble;
    if (mode == 3 && !cufft_load()) {
        set_error("set_dipole: do_dip = 3 needs cuFFT (libcufft.so.12), which could not be loaded");
        return UPPASD_GPU_ENODEV;
    }
    DipoleDev *d = new (std::nothrow) DipoleDev();
    if (!d) return UPPASD_GPU_ENOMEM;
    d->mode = mode;
    d->na = na;
    d->n1 = n1;
    d->n2 = n2;
    d->n3 = n3;
    d->fac = (1.0e-7 / (alat * alat * alat)) * s.ham.mub;
    // the caller's coordinates (setup_qdip), else the reference's numbering of the cell grid:
    // site i = I0 + NA (I1 + N1 (I2 + N2 I3)) at I1 C1 + I2 C2 + I3 C3 + Bas(I0)
    std::vector<double> coord(3 * (size_t)N);
    if (coord_in)
        std::copy(coord_in, coord_in + 3 * (size_t)N, coord.begin());
    else
        for (int i = 0; i < N; ++i) {
            const int I0 = i % na, c = i / na;
            const int I1 = c % n1, I2 = (c / n1) % n2, I3 = c / (n1 * n2);
            for (int q = 0; q < 3; ++q)
                coord[3 * (size_t)i + q] = I1 * cell[q] + I2 * cell[3 + q] + I3 * cell[6 + q] + bas[3 * I0 + q];
        }
    cudaError_t e = cudaMalloc(&d->coord, coord.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(d->coord, coord.data(), coord.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = dip_alloc3(s.ham.dip, (size_t)N * M);
    int rc = UPPASD_GPU_OK;
    if (e == cudaSuccess && mode == 1) {
        // enough (site, share) threads to fill the SMs about eight 128-thread blocks deep,
        // a share holding at least one tile of sources
        int sms = 152;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s.device);
        const long long target = (long long)sms * 8 * kDipTile, nm = (long long)N * M;
        long long sh = (target + nm - 1) / nm;
        sh = std::min<long long>(sh, std::min<long long>(64, (N + kDipTile - 1) / kDipTile));
        d->shares = (int)std::max<long long>(sh, 1);
        if (d->shares > 1) e = cudaMalloc(&d->part, (size_t)d->shares * 3 * nm * sizeof(double));
    }
    if (e == cudaSuccess && mode == 3) {
        d->p1 = smooth_length(2 * n1 - 1);
        d->p2 = smooth_length(2 * n2 - 1);
        d->p3 = smooth_length(2 * n3 - 1);
        d->npad = (long long)d->p1 * d->p2 * d->p3;
        d->nc = (long long)(d->p1 / 2 + 1) * d->p2 * d->p3;
        const size_t nb = (size_t)M * na * 3;
        // cuFFT's batched plans take the distances between transforms as int
        if (d->npad > INT_MAX || nb > (size_t)INT_MAX || (long long)na * na * 6 > INT_MAX) {
            set_error("set_dipole: the padded grid is too large for the FFT form (more than 2^31 points)");
            rc = UPPASD_GPU_EINVAL;
        }
        if (!rc) {
            e = cudaMalloc(&d->mr, nb * d->npad * sizeof(double));
            if (e == cudaSuccess) e = cudaMalloc(&d->fr, nb * d->npad * sizeof(double));
            if (e == cudaSuccess) e = cudaMalloc(&d->mk, nb * d->nc * sizeof(cufftDoubleComplex));
            if (e == cudaSuccess) e = cudaMalloc(&d->fk, nb * d->nc * sizeof(cufftDoubleComplex));
            if (e == cudaSuccess) e = cudaMalloc(&d->kt, (size_t)na * na * 6 * d->nc * sizeof(cufftDoubleComplex));
        }
        if (e == cudaSuccess && !rc) {
            rc = plan3(&d->pf, *d, CUFFT_D2Z, (int)nb);
            d->pf_made = rc == UPPASD_GPU_OK;
            if (!rc) {
                rc = plan3(&d->pi, *d, CUFFT_Z2D, (int)nb);
                d->pi_made = rc == UPPASD_GPU_OK;
            }
        }
        // the transformed tensors, once
        if (e == cudaSuccess && !rc) {
            double *treal = nullptr, *dcell = nullptr, *dbas = nullptr;
            cufftHandle pt = 0;
            bool pt_made = false;
            const size_t nt = (size_t)na * na * 6;
            e = cudaMalloc(&treal, nt * d->npad * sizeof(double));
            if (e == cudaSuccess) e = cudaMalloc(&dcell, 9 * sizeof(double));
            if (e == cudaSuccess) e = cudaMalloc(&dbas, 3 * (size_t)na * sizeof(double));
            if (e == cudaSuccess) e = cudaMemcpy(dcell, cell, 9 * sizeof(double), cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = cudaMemcpy(dbas, bas, 3 * (size_t)na * sizeof(double), cudaMemcpyHostToDevice);
            if (e == cudaSuccess) {
                const long long tot = (long long)na * na * d->npad;
                dip_tensor<<<(unsigned)((tot + 255) / 256), 256>>>(*d, dcell, dbas, treal);
                e = cudaGetLastError();
            }
            if (e == cudaSuccess) {
                rc = plan3(&pt, *d, CUFFT_D2Z, (int)nt);
                pt_made = rc == UPPASD_GPU_OK;
            }
            if (e == cudaSuccess && !rc && g_fft.exec_d2z(pt, treal, d->kt) != CUFFT_SUCCESS) {
                set_error("set_dipole: cuFFT transform of the tensor failed");
                rc = UPPASD_GPU_ECUDA;
            }
            if (e == cudaSuccess) e = cudaDeviceSynchronize();
            if (pt_made) g_fft.destroy(pt);
            cudaFree(treal);
            cudaFree(dcell);
            cudaFree(dbas);
        }
    }
    if (e != cudaSuccess || rc) {
        if (e != cudaSuccess) set_error(std::string("set_dipole: ") + cudaGetErrorString(e));
        dipole_release(*d);
        delete d;
        dip_free3(s.ham.dip);
        return rc ? rc : (e == cudaErrorMemoryAllocation ? UPPASD_GPU_ENOMEM : UPPASD_GPU_ECUDA);
    }
    s.dip = d;
    s.ham.do_dip = mode;
    return UPPASD_GPU_OK;
}

}  // namespace uppasd
