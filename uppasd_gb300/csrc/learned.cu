// learned.cu -- learned autoregressive 4x4-patch proposal with exact
// Metropolis-Hastings acceptance, on a square-lattice simulation's spins.
//
// Geometry: an L x L square lattice (site i = x + L y, one atom per cell,
// L % 8 == 0), Mensemble chains.  The lattice is tiled by 4 x 4 patches; patch
// (I, J) covers x in [4J, 4J+4), y in [4I, 4I+4).  Patches of one colour
// (I % 2, J % 2) are 4 sites apart, so their 8 x 8 windows (the patch plus a
// 2-site boundary) never contain another patch of the colour: all patches of
// a colour move at once, each against a fixed boundary.
//
// Network (MADE, block-autoregressive over 4 groups): input = the 8 x 8
// window's unit vectors (3 x 64 = 192 features, bf16), 3 hidden layers of 256
// (tanh), output = vMF natural parameters eta = kappa mu (3 per patch spin, 48
// used of 64).  The patch's 16 spins form 4 groups by sub-lattice
// ((py % 2) * 2 + px % 2; sites of one group share no bond); masks let the
// outputs of group g see the boundary and groups < g only, so
//   q(patch | boundary) = prod_g prod_{s in g} vMF(x_s; eta_s(boundary, groups < g)).
// All matrix products run on the tcgen05 GEMM (tc_gemm.cuh) in BF16 with FP32
// accumulation.
//
// Move (per colour, all chains at once): one forward pass on the old window
// gives log q(old) and group 0's parameters; three more passes sample groups 1-3
// on the updated window; then one warp per patch forms the exact energy change
// in FP64 from the simulation's neighbour lists (exchange, DMI, anisotropy,
// Zeeman -- the terms of calculate_energy, MonteCarlo/montecarlo_common.f90:431-865)
// and accepts with min(1, exp(-beta dE) q(old) / q(new)).  The boundary is not
// changed by the move, so q(old | boundary) is the reverse-move density and the
// chain keeps the Boltzmann distribution exactly.
//
// Training: windows of heat-bath configurations (teacher forcing), loss =
// mean negative log q of the patch, gradients by the hand-written backward pass
// (tcgen05 GEMMs with the tanh derivative fused into the epilogue), Adam on FP32
// master weights, masks re-applied after every step.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "sim.h"
#include "tc_gemm.cuh"
#include "tc_host.h"
#include "tc_mlp.cuh"

namespace uppasd {
namespace lp {

constexpr int kFeat = 192, kHid = 256, kOut = 64, kSpins = 16, kUsedOut = 48;
constexpr int kNW[4] = {kHid * kFeat, kHid * kHid, kHid * kHid, kOut * kHid};
constexpr int kNB[4] = {kHid, kHid, kHid, kOut};

__host__ __device__ constexpr int patch_group(int py, int px) { return (py & 1) * 2 + (px & 1); }

// feature f = pos * 3 + component, pos = wy * 8 + wx; interior (wy, wx in [2, 6)) has
// degree group + 1, the boundary degree 0
__host__ __device__ constexpr int feat_degree(int f) {
    const int pos = f / 3, wy = pos / 8, wx = pos % 8;
    return (wy >= 2 && wy < 6 && wx >= 2 && wx < 6) ? patch_group(wy - 2, wx - 2) + 1 : 0;
}

struct Params {
    // fp32 master weights and biases, masks, Adam moments, gradients (same layout)
    float *w[4], *b[4], *mask[4], *mw[4], *vw[4], *mb[4], *vb[4], *gw[4], *gb[4];
};

struct Bufs {
    __nv_bfloat16 *X, *H[3], *dO, *dH[3];     // [R x .]
    __nv_bfloat16 *Xt, *Ht[3], *dOt, *dHt[3]; // transposes [. x R]
    float *O;                                  // [R x 64]
    float *gW4t;                               // [256 x 64]
    __nv_bfloat16 *wb[4];                      // bf16 weights W (N x K)
    __nv_bfloat16 *wt[4];                      // bf16 transposes W^T (layers 2..4: K x N)
};

// ---------------------------------------------------------------------------- kernels

__global__ void k_cast_bf16(const float *src, __nv_bfloat16 *dst, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = __float2bfloat16_rn(src[i]);
}

// dst (cols x rows) = src (rows x cols)^T, fp32 -> bf16
__global__ void k_transpose_f32_bf16(const float *src, __nv_bfloat16 *dst, int rows, int cols) {
    __shared__ float t[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int r = r0 + j, c = c0 + threadIdx.x;
        t[j][threadIdx.x] = (r < rows && c < cols) ? src[(size_t)r * cols + c] : 0.f;
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int c = c0 + j, r = r0 + threadIdx.x;
        if (c < cols && r < rows) dst[(size_t)c * rows + r] = __float2bfloat16_rn(t[threadIdx.x][j]);
    }
}

// dst (cols x rows) = src (rows x cols)^T, bf16
__global__ void k_transpose_bf16(const __nv_bfloat16 *src, __nv_bfloat16 *dst, int rows, int cols) {
    __shared__ __nv_bfloat16 t[32][34];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int r = r0 + j, c = c0 + threadIdx.x;
        t[j][threadIdx.x] = (r < rows && c < cols) ? src[(size_t)r * cols + c] : __float2bfloat16_rn(0.f);
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int c = c0 + j, r = r0 + threadIdx.x;
        if (c < cols && r < rows) dst[(size_t)c * rows + r] = t[threadIdx.x][j];
    }
}

// column sums of a bf16 (rows x cols) matrix into fp32 out[cols]
__global__ void k_colsum(const __nv_bfloat16 *a, int rows, int cols, float *out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float s = 0.f;
    for (int r = blockIdx.y; r < rows; r += gridDim.y) s += __bfloat162float(a[(size_t)r * cols + c]);
    atomicAdd(out + c, s);
}

struct PatchGeom {
    int L, np;        // lattice edge, patches per colour per chain = (L/8)^2
    int half;         // L / 8: patches of one colour per row
    int colour;       // 0..3, or -1: rows run over all four colours (data collection)
};

// Row r -> chain k and patch origin (x0, y0).
__device__ __forceinline__ void patch_of_row(const PatchGeom &g, int r, int &k, int &x0, int &y0) {
    int c = g.colour, rr = r;
    const int per_chain = g.colour < 0 ? 4 * g.np : g.np;
    k = rr / per_chain;
    rr -= k * per_chain;
    if (c < 0) {
        c = rr / g.np;
        rr -= c * g.np;
    }
    const int I = 2 * (rr / g.half) + (c >> 1), J = 2 * (rr % g.half) + (c & 1);
    x0 = 4 * J;
    y0 = 4 * I;
}

__device__ __forceinline__ int wrap_site(int x, int y, int L) {
    x = x < 0 ? x + L : (x >= L ? x - L : x);
    y = y < 0 ? y + L : (y >= L ? y - L : y);
    return x + L * y;
}

// Windows of `rows` patches into X (rows x 192, bf16); optionally the old patch
// spins (rows x 48, FP32).  One thread per (row, window position).  The spins come
// from the FP32 mirror when `m` is given (the square-lattice path), else from e.
__global__ void k_gather(PatchGeom g, Vec3D e, const float4 *m, int natom, int rows, __nv_bfloat16 *X,
                         float *old_patch, float *win) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)rows * 64) return;
    const int r = (int)(t >> 6), pos = (int)(t & 63);
    int k, x0, y0;
    patch_of_row(g, r, k, x0, y0);
    const int wy = pos >> 3, wx = pos & 7;
    const int i = wrap_site(x0 - 2 + wx, y0 - 2 + wy, g.L);
    const size_t o = (size_t)k * natom + i;
    float v[3];
    if (m) {
        const float4 q = m[o];
        v[0] = q.x;
        v[1] = q.y;
        v[2] = q.z;
    } else {
        v[0] = (float)e.x[o];
        v[1] = (float)e.y[o];
        v[2] = (float)e.z[o];
    }
    __nv_bfloat16 *xr = X + (size_t)r * kFeat + pos * 3;
    xr[0] = __float2bfloat16_rn(v[0]);
    xr[1] = __float2bfloat16_rn(v[1]);
    xr[2] = __float2bfloat16_rn(v[2]);
    if (win) {
        // FP32 copy of the window for the acceptance kernel's bonds to the boundary
        float *wr = win + (size_t)r * kFeat + pos * 3;
        wr[0] = v[0];
        wr[1] = v[1];
        wr[2] = v[2];
    }
    if (old_patch && wy >= 2 && wy < 6 && wx >= 2 && wx < 6) {
        const int s = (wy - 2) * 4 + (wx - 2);
        float *op = old_patch + (size_t)r * 48 + 3 * s;
        op[0] = v[0];
        op[1] = v[1];
        op[2] = v[2];
    }
}

// log vMF(x; eta) = eta.x + log kappa - log(2 pi) - log(1 - e^{-2 kappa}) - kappa  (FP64)
__device__ __forceinline__ double log_vmf(const double eta[3], const double x[3]) {
    const double kap = sqrt(eta[0] * eta[0] + eta[1] * eta[1] + eta[2] * eta[2]);
    const double dot = eta[0] * x[0] + eta[1] * x[1] + eta[2] * x[2];
    if (kap < 1e-8) return dot - log(4.0 * kPi);
    return dot + log(kap) - log(2.0 * kPi) - log(-expm1(-2.0 * kap)) - kap;
}

// log vMF in FP32: the same function scores the sampled and the current patch, and
// the sampler itself is FP32.  A row's 16 terms are summed in FP32 (rounding ~1e-5,
// far below what the acceptance test resolves).
__device__ __forceinline__ float log_vmf_f(float ex, float ey, float ez, float x, float y, float z) {
    const float kap = sqrtf(ex * ex + ey * ey + ez * ez);
    const float dot = ex * x + ey * y + ez * z;
    if (kap < 1e-6f) return dot - 2.5310242469692907f;  // log(4 pi)
    return dot + logf(kap) - 1.8378770664093453f - logf(-expm1f(-2.0f * kap)) - kap;  // log(2 pi)
}

// Group g of every row, two rows per warp and one lane per patch spin: when g == 0
// the 16 lanes of a row score the current patch (log q(old)); then the lanes of
// group g draw their spins from vMF(eta), add their log density to log q(new),
// and write them to the new-patch buffer and into the window for the next pass.
__global__ void __launch_bounds__(128) k_vmf_group(int rows, int g, float eta_scale, const float *O,
                                                   __nv_bfloat16 *X, const float *old_patch, float *new_patch,
                                                   float *logq_old, float *logq_new, uint64_t seed,
                                                   const long long *dctr, int sub) {
    const int lane = threadIdx.x & 31;
    const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 4;  // rows % 8 == 0: whole warps stay in range
    const int s = lane & 15, py = s >> 2, px = s & 3;
    const long long ctr = *dctr * 16 + sub;  // device sweep counter: graph replays draw fresh numbers
    const float *o = O + (size_t)r * kOut;
    const float ex = eta_scale * o[3 * s], ey = eta_scale * o[3 * s + 1], ez = eta_scale * o[3 * s + 2];
    float t_old = 0.f, t_new = 0.f;
    if (g == 0) {
        const float *op = old_patch + (size_t)r * 48 + 3 * s;
        t_old = log_vmf_f(ex, ey, ez, op[0], op[1], op[2]);
    }
    if (patch_group(py, px) == g) {
        const float kap = sqrtf(ex * ex + ey * ey + ez * ez);
        const Philox4 w = philox_draw(seed, r, s, ctr, kStreamLearned);
        const float u1 = fmaf((float)w.x, 2.3283064365386963e-10f, 1.1641532182693481e-10f);
        const float u2 = fmaf((float)w.y, 2.3283064365386963e-10f, 1.1641532182693481e-10f);
        float mx, my, mz, ct;
        if (kap > 1e-6f) {
            mx = ex / kap;
            my = ey / kap;
            mz = ez / kap;
            // cos of the angle to mu: inverse CDF of exp(kappa t) on [-1, 1]
            const float e2 = expf(-2.0f * kap);
            ct = 1.0f + logf(fmaf(1.0f - e2, u1, e2)) / kap;
        } else {
            mx = 0.f;
            my = 0.f;
            mz = 1.f;
            ct = 1.0f - 2.0f * u1;
        }
        ct = fminf(1.0f, fmaxf(-1.0f, ct));
        const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
        // orthonormal pair perpendicular to mu
        float ax, ay, az;
        if (fabsf(mz) < 0.9f) {
            ax = -my;
            ay = mx;
            az = 0.f;
        } else {
            ax = 0.f;
            ay = -mz;
            az = my;
        }
        const float ia = rsqrtf(ax * ax + ay * ay + az * az);
        ax *= ia;
        ay *= ia;
        az *= ia;
        const float bx = my * az - mz * ay, by = mz * ax - mx * az, bz = mx * ay - my * ax;
        float sp, cp;
        sincospif(2.0f * u2, &sp, &cp);
        float nx = ct * mx + st * (cp * ax + sp * bx);
        float ny = ct * my + st * (cp * ay + sp * by);
        float nz = ct * mz + st * (cp * az + sp * bz);
        const float il = rsqrtf(nx * nx + ny * ny + nz * nz);
        nx *= il;
        ny *= il;
        nz *= il;
        t_new = log_vmf_f(ex, ey, ez, nx, ny, nz);
        float *np_ = new_patch + (size_t)r * 48 + 3 * s;
        np_[0] = nx;
        np_[1] = ny;
        np_[2] = nz;
        __nv_bfloat16 *xr = X + (size_t)r * kFeat + ((py + 2) * 8 + (px + 2)) * 3;
        xr[0] = __float2bfloat16_rn(nx);
        xr[1] = __float2bfloat16_rn(ny);
        xr[2] = __float2bfloat16_rn(nz);
    }
    // sums over the 16 lanes of the row
#pragma unroll
    for (int off = 8; off > 0; off >>= 1) {
        t_old += __shfl_xor_sync(0xffffffffu, t_old, off);
        t_new += __shfl_xor_sync(0xffffffffu, t_new, off);
    }
    if (s == 0) {
        if (g == 0) {
            logq_old[r] = t_old;
            logq_new[r] = t_new;
        } else {
            logq_new[r] += t_new;
        }
    }
}

// Accepted moves and their energy change summed per block (one warp per patch,
// lane 0 holds the warp's values): one atomic per block rather than one per patch,
// which serialised on the counters.  Every warp of the block must reach this.
__device__ __forceinline__ void block_count(int acc, double dE, unsigned long long *accepted, double *dE_sum) {
    __shared__ unsigned bacc[32];
    __shared__ double bde[32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        bacc[w] = acc ? 1u : 0u;
        bde[w] = acc ? dE : 0.0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned a = 0;
        double d = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
            a += bacc[q];
            d += bde[q];
        }
        if (a) {
            atomicAdd(accepted, (unsigned long long)a);
            atomicAdd(dE_sum, d);
        }
    }
}

// Uniform square-lattice couplings (SquareMC) for the patch energy.
struct SqCoup {
    float c[4], d[4][3], ext[3], mom;
};

// One warp per patch on a uniform square lattice: lanes 0-15 score the new patch,
// lanes 16-31 the old one (bonds leaving the patch in full, bonds inside it at one
// half, Zeeman on site); then the Metropolis-Hastings decision and write-back.
// Each lane's bond sum is FP32 (a bond term is at most |J| m ~ 500 T muB, rounded to
// ~3e-5), the patch sums and the decision FP64: the log acceptance carries an error
// of ~1e-5 / T[K], far below any statistical resolution.
__global__ void __launch_bounds__(256) k_accept_sq(PatchGeom g, SqCoup q, float4 *m, Vec3D e, Vec3D eM, int natom,
                                                   int rows,
                                                   const float *win, const float *old_patch, const float *new_patch,
                                                   const float *logq_old, const float *logq_new, float beta_mub,
                                                   const float *betak, uint64_t seed, const long long *dctr, int sub,
                                                   unsigned long long *accepted, double *dE_sum) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    // rows is a multiple of 128 and blocks hold 8 warps: every warp of the grid is a patch
    const int r = warp;
    const long long ctr = *dctr * 16 + sub;
    int k, x0, y0;
    patch_of_row(g, r, k, x0, y0);
    const int s = lane & 15, py = s >> 2, px = s & 3;
    const float *patch = (lane < 16 ? new_patch : old_patch) + (size_t)r * 48;
    const float fi[3] = {patch[3 * s], patch[3 * s + 1], patch[3 * s + 2]};
    const size_t off = (size_t)k * natom;
    float E = -(q.ext[0] * fi[0] + q.ext[1] * fi[1] + q.ext[2] * fi[2]);
    const int ddx[4] = {1, -1, 0, 0}, ddy[4] = {0, 0, 1, -1};
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        const int nx = px + ddx[d], ny = py + ddy[d];
        float ej[3], w;
        if (nx >= 0 && nx < 4 && ny >= 0 && ny < 4) {
            const int sj = ny * 4 + nx;
            ej[0] = patch[3 * sj];
            ej[1] = patch[3 * sj + 1];
            ej[2] = patch[3 * sj + 2];
            w = 0.5f;
        } else {
            // the boundary site from the window copy (no other patch of this colour touches it)
            const float *wv = win + (size_t)r * kFeat + ((ny + 2) * 8 + (nx + 2)) * 3;
            ej[0] = wv[0];
            ej[1] = wv[1];
            ej[2] = wv[2];
            w = 1.0f;
        }
        const float cx = fi[1] * ej[2] - fi[2] * ej[1], cy = fi[2] * ej[0] - fi[0] * ej[2],
                    cz = fi[0] * ej[1] - fi[1] * ej[0];
        E -= w * (q.c[d] * (fi[0] * ej[0] + fi[1] * ej[1] + fi[2] * ej[2]) +
                  (q.d[d][0] * cx + q.d[d][1] * cy + q.d[d][2] * cz));
    }
    E *= q.mom;
    // per spin new - old (lanes s and s + 16), then the sum over the patch; FP32
    // throughout, as GB300's FP64 pipe would set this kernel's time
    float dE = lane < 16 ? E : -E;
    dE += __shfl_xor_sync(0xffffffffu, dE, 16);
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) dE += __shfl_xor_sync(0xffffffffu, dE, o);
    int acc = 0;
    if (lane == 0) {
        const float loga = -(betak ? betak[k] : beta_mub) * dE + (logq_old[r] - logq_new[r]);
        const Philox4 w = philox_draw(seed, r, 16, ctr, kStreamLearned);
        const float u = u01_openf(w.z);
        acc = (loga >= 0.f || logf(u) < loga) ? 1 : 0;
    }
    acc = __shfl_sync(0xffffffffu, acc, 0);
    if (acc && lane < kSpins) {
        const size_t o = off + wrap_site(x0 + px, y0 + py, g.L);
        const double mm = (double)q.mom;
        const double ei[3] = {(double)fi[0], (double)fi[1], (double)fi[2]};
        m[o] = make_float4(fi[0], fi[1], fi[2], 0.f);
        e.x[o] = ei[0];
        e.y[o] = ei[1];
        e.z[o] = ei[2];
        eM.x[o] = mm * ei[0];
        eM.y[o] = mm * ei[1];
        eM.z[o] = mm * ei[2];
    }
    block_count(acc, (double)dE, accepted, dE_sum);
}

// Energy of patch spin `s` (site i) in one configuration: bonds to sites outside the
// patch in full, bonds inside the patch at one half, plus on-site terms.  Units: T muB.
// OLD: the configuration in the state (FP64, read from eM); otherwise the sampled
// patch (FP32 values, exact in FP64) with the state outside it.
template <bool OLD>
__device__ double patch_spin_energy(const HamDev &h, const Vec3D &eM, const double *mmom, int k, int i, int x0,
                                    int y0, int L, const float *patch /*48*/, int s) {
    const int N = h.natom;
    const size_t off = (size_t)k * N;
    const double mm = mmom[off + i];
    double mi[3];
    if (OLD) {
        mi[0] = eM.x[off + i];
        mi[1] = eM.y[off + i];
        mi[2] = eM.z[off + i];
    } else {
        mi[0] = (double)patch[3 * s] * mm;
        mi[1] = (double)patch[3 * s + 1] * mm;
        mi[2] = (double)patch[3 * s + 2] * mm;
    }
    const int ih = h.aham[i];
    double E = 0.0;
    for (int q = 0; q < h.nsize[i]; ++q) {
        const int j = h.nlist[(size_t)q * N + i];
        const int jx = j % L, jy = j / L;
        const int dx = (jx - x0 + L) % L, dy = (jy - y0 + L) % L;
        double mj[3], w = 1.0;
        if (dx < 4 && dy < 4) {
            w = 0.5;
            if (OLD) {
                mj[0] = eM.x[off + j];
                mj[1] = eM.y[off + j];
                mj[2] = eM.z[off + j];
            } else {
                const int sj = dy * 4 + dx;
                const double mmj = mmom[off + j];
                mj[0] = (double)patch[3 * sj] * mmj;
                mj[1] = (double)patch[3 * sj + 1] * mmj;
                mj[2] = (double)patch[3 * sj + 2] * mmj;
            }
        } else {
            mj[0] = eM.x[off + j];
            mj[1] = eM.y[off + j];
            mj[2] = eM.z[off + j];
        }
        const double c = h.ncoup[(size_t)q * h.nham + ih];
        E -= w * c * (mi[0] * mj[0] + mi[1] * mj[1] + mi[2] * mj[2]);
    }
    if (h.do_dm) {
        for (int q = 0; q < h.dmsize[i]; ++q) {
            const int j = h.dmlist[(size_t)q * N + i];
            const int jx = j % L, jy = j / L;
            const int dx = (jx - x0 + L) % L, dy = (jy - y0 + L) % L;
            double mj[3], w = 1.0;
            if (dx < 4 && dy < 4) {
                w = 0.5;
                if (OLD) {
                    mj[0] = eM.x[off + j];
                    mj[1] = eM.y[off + j];
                    mj[2] = eM.z[off + j];
                } else {
                    const int sj = dy * 4 + dx;
                    const double mmj = mmom[off + j];
                    mj[0] = (double)patch[3 * sj] * mmj;
                    mj[1] = (double)patch[3 * sj + 1] * mmj;
                    mj[2] = (double)patch[3 * sj + 2] * mmj;
                }
            } else {
                mj[0] = eM.x[off + j];
                mj[1] = eM.y[off + j];
                mj[2] = eM.z[off + j];
            }
            const size_t d = (size_t)q * h.nham + ih;
            // -D.(m_i x m_j): the energy whose gradient is the reference's m_j x D field
            const double cx = mi[1] * mj[2] - mi[2] * mj[1], cy = mi[2] * mj[0] - mi[0] * mj[2],
                         cz = mi[0] * mj[1] - mi[1] * mj[0];
            E -= w * (h.dmx[d] * cx + h.dmy[d] * cy + h.dmz[d] * cz);
        }
    }
    if (h.do_aniso && h.taniso[i] == 1) {
        const double t = mi[0] * h.eax[i] + mi[1] * h.eay[i] + mi[2] * h.eaz[i];
        E += h.k1[i] * (t * t) + h.k2[i] * (t * t * (t * t));
    }
    E -= h.ext.x[off + i] * mi[0] + h.ext.y[off + i] * mi[1] + h.ext.z[off + i] * mi[2];
    return E;
}

// One warp per patch: exact energy change, Metropolis-Hastings decision, write-back.
// tk: temperature per ensemble (K) or null (beta_mub for all)
__global__ void k_accept(PatchGeom g, HamDev h, Vec3D e, Vec3D eM, const double *mmom, int rows,
                         const float *new_patch, const float *logq_old, const float *logq_new, double beta_mub,
                         const double *tk, uint64_t seed, const long long *dctr, int sub, unsigned long long *accepted,
                         double *dE_sum) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    // rows is a multiple of 128 and blocks hold 8 warps: every warp of the grid is a patch
    const int r = warp;
    const long long ctr = *dctr * 16 + sub;
    int k, x0, y0;
    patch_of_row(g, r, k, x0, y0);
    double dE = 0.0;
    if (lane < kSpins) {
        const int py = lane >> 2, px = lane & 3;
        const int i = wrap_site(x0 + px, y0 + py, g.L);
        dE = patch_spin_energy<false>(h, eM, mmom, k, i, x0, y0, g.L, new_patch + (size_t)r * 48, lane) -
             patch_spin_energy<true>(h, eM, mmom, k, i, x0, y0, g.L, nullptr, lane);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dE += __shfl_xor_sync(0xffffffffu, dE, o);
    int acc = 0;
    if (lane == 0) {
        const double b = tk ? h.mub / (h.kbolt * tk[k]) : beta_mub;
        const double loga = -b * dE + (double)(logq_old[r] - logq_new[r]);
        const Philox4 w = philox_draw(seed, r, 16, ctr, kStreamLearned);
        const float u = u01_openf(w.z);
        acc = (loga >= 0.0 || (double)logf(u) < loga) ? 1 : 0;
    }
    acc = __shfl_sync(0xffffffffu, acc, 0);
    if (acc && lane < kSpins) {
        const int py = lane >> 2, px = lane & 3;
        const int i = wrap_site(x0 + px, y0 + py, g.L);
        const size_t o = (size_t)k * h.natom + i;
        const float *np_ = new_patch + (size_t)r * 48 + 3 * lane;
        const double mm = mmom[o];
        e.x[o] = (double)np_[0];
        e.y[o] = (double)np_[1];
        e.z[o] = (double)np_[2];
        eM.x[o] = mm * (double)np_[0];
        eM.y[o] = mm * (double)np_[1];
        eM.z[o] = mm * (double)np_[2];
    }
    block_count(acc, dE, accepted, dE_sum);
}

// Loss and output gradient: L = -(1/R) sum_rows sum_s log vMF(x_s; eta_s), eta = scale * O;
// dL/dO = -(scale/R) (x - A(kappa) mu), A = coth(kappa) - 1/kappa.
__global__ void k_loss_grad(int rows, float eta_scale, const float *O, const __nv_bfloat16 *X, __nv_bfloat16 *dO,
                            double *loss) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (r < rows) {
        const float *o = O + (size_t)r * kOut;
        __nv_bfloat16 *d = dO + (size_t)r * kOut;
        const double inv = 1.0 / rows;
        for (int s = 0; s < kSpins; ++s) {
            const int py = s >> 2, px = s & 3, pos = (py + 2) * 8 + (px + 2);
            const __nv_bfloat16 *xr = X + (size_t)r * kFeat + pos * 3;
            const double x[3] = {(double)__bfloat162float(xr[0]), (double)__bfloat162float(xr[1]),
                                 (double)__bfloat162float(xr[2])};
            const double eta[3] = {(double)eta_scale * o[3 * s], (double)eta_scale * o[3 * s + 1],
                                   (double)eta_scale * o[3 * s + 2]};
            l -= log_vmf(eta, x);
            const double kap = sqrt(eta[0] * eta[0] + eta[1] * eta[1] + eta[2] * eta[2]);
            // A(kappa) / kappa (the coefficient of eta), series below 1e-3
            const double a_over_k = kap < 1e-3 ? (1.0 / 3.0 - kap * kap / 45.0)
                                               : (1.0 / tanh(kap) - 1.0 / kap) / kap;
            for (int c = 0; c < 3; ++c)
                d[3 * s + c] = __float2bfloat16_rn((float)(-(double)eta_scale * inv * (x[c] - a_over_k * eta[c])));
        }
        for (int c = kUsedOut; c < kOut; ++c) d[c] = __float2bfloat16_rn(0.f);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && l != 0.0) atomicAdd(loss, l / rows);
}

// Adam step on one parameter array; masked entries stay exactly zero.
__global__ void k_adam(float *p, const float *gr, const float *mask, float *m, float *v, int n, float lr, float b1,
                       float b2, float c1, float c2, float eps, int transposed_rows, int transposed_cols) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // gradient stored transposed when transposed_rows > 0: parameter (r, c) of a
    // transposed_rows x transposed_cols matrix at gr[c * transposed_rows + r]
    float gi;
    if (transposed_rows > 0) {
        const int r = i / transposed_cols, c = i % transposed_cols;
        gi = gr[(size_t)c * transposed_rows + r];
    } else {
        gi = gr[i];
    }
    if (mask) gi *= mask[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    if (mask) pi *= mask[i];
    p[i] = pi;
}

__global__ void k_advance(long long *dctr) { *dctr += 1; }

// Random minibatch of dataset rows into X.
__global__ void k_sample_rows(const __nv_bfloat16 *D, long long count, int rows, uint64_t seed, long long ctr,
                              __nv_bfloat16 *X) {
    const int r = blockIdx.x;
    __shared__ long long src;
    if (threadIdx.x == 0) {
        const Philox4 w = philox_draw(seed, r, 17, ctr, kStreamLearned);
        const unsigned long long u = ((unsigned long long)w.x << 32) | w.y;
        src = (long long)(u % (unsigned long long)count);
    }
    __syncthreads();
    const uint4 *s = reinterpret_cast<const uint4 *>(D + (size_t)src * kFeat);
    uint4 *d = reinterpret_cast<uint4 *>(X + (size_t)r * kFeat);
    for (int q = threadIdx.x; q < kFeat * 2 / 16; q += blockDim.x) d[q] = s[q];
}

}  // namespace lp
}  // namespace uppasd

struct uppasd_gpu_proposal {
    uppasd_gpu_sim *sim = nullptr;
    int L = 0, max_rows = 0;
    float eta_scale = 1.f;
    uint64_t seed = 0;
    uppasd::lp::Params P{};
    uppasd::lp::Bufs B{};
    float *params = nullptr;   // one allocation for all fp32 parameter-sized arrays
    long long nparams = 0;
    // sampling
    float *old_patch = nullptr, *new_patch = nullptr, *logq_old = nullptr, *logq_new = nullptr;
    float *win = nullptr;  // FP32 copy of each row's window (rows x 192)
    unsigned long long *accepted = nullptr;
    double *dE_sum = nullptr, *loss = nullptr;
    int *err = nullptr;
    // dataset
    __nv_bfloat16 *data = nullptr;
    long long data_cap = 0, data_count = 0, data_next = 0;
    long long ctr = 0;             // Philox counter of minibatches (host)
    long long *dctr = nullptr;     // Philox counter of learned sweeps (device, advanced in-stream)
    int adam_t = 0;
    // prepared GEMMs: forward (rows R) for the current row count
    int prepared_rows = -1;
    uppasd::tc::Gemm fwd[4], bwd[3], wgr[4];
    // fused forward (tc_mlp.cuh): maps of the input rows and of the four bf16 weights
    int mlp_rows = -1;
    CUtensorMap mlp_x, mlp_w[4];
    // one learned sweep captured as a CUDA graph (rebuilt when T or the rows change)
    cudaGraphExec_t sweep_graph = nullptr;
    double graph_T = -1.0;
    int graph_rows = -1;
    bool warmed = false;
};

namespace {
using namespace uppasd;
using namespace uppasd::lp;

int cuda_fail(const char *what, cudaError_t e) {
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? UPPASD_GPU_ENOMEM : UPPASD_GPU_ECUDA;
}

void free_all(uppasd_gpu_proposal *p) {
    if (!p) return;
    cudaDeviceSynchronize();
    void *ptrs[] = {p->params, p->B.X, p->B.dO, p->B.Xt, p->B.dOt, p->B.O, p->B.gW4t, p->old_patch,
                    p->new_patch, p->logq_old, p->logq_new, p->accepted, p->dE_sum, p->loss, p->err, p->data,
                    p->dctr, p->win};
    if (p->sweep_graph) cudaGraphExecDestroy(p->sweep_graph);
    for (void *q : ptrs) cudaFree(q);
    for (int l = 0; l < 3; ++l) {
        cudaFree(p->B.H[l]);
        cudaFree(p->B.dH[l]);
        cudaFree(p->B.Ht[l]);
        cudaFree(p->B.dHt[l]);
    }
    for (int l = 0; l < 4; ++l) {
        cudaFree(p->B.wb[l]);
        cudaFree(p->B.wt[l]);
    }
    delete p;
}

// MADE masks: hidden degrees h % 4; input degree by feat_degree; outputs of group g see d_h <= g.
void build_masks(std::vector<float> mask[4]) {
    mask[0].assign((size_t)kHid * kFeat, 0.f);
    for (int hh = 0; hh < kHid; ++hh)
        for (int f = 0; f < kFeat; ++f) mask[0][(size_t)hh * kFeat + f] = feat_degree(f) <= (hh & 3) ? 1.f : 0.f;
    for (int l = 1; l < 3; ++l) {
        mask[l].assign((size_t)kHid * kHid, 0.f);
        for (int a = 0; a < kHid; ++a)
            for (int bb = 0; bb < kHid; ++bb) mask[l][(size_t)a * kHid + bb] = (bb & 3) <= (a & 3) ? 1.f : 0.f;
    }
    mask[3].assign((size_t)kOut * kHid, 0.f);
    for (int o = 0; o < kUsedOut; ++o) {
        const int s = o / 3, grp = patch_group(s >> 2, s & 3);
        for (int hh = 0; hh < kHid; ++hh) mask[3][(size_t)o * kHid + hh] = (hh & 3) <= grp ? 1.f : 0.f;
    }
}

int sync_weights(uppasd_gpu_proposal *p, cudaStream_t st) {
    const int K[4] = {kFeat, kHid, kHid, kHid}, N[4] = {kHid, kHid, kHid, kOut};
    for (int l = 0; l < 4; ++l) {
        const int n = kNW[l];
        k_cast_bf16<<<(n + 255) / 256, 256, 0, st>>>(p->P.w[l], p->B.wb[l], n);
        if (l >= 1) {
            dim3 grid((K[l] + 31) / 32, (N[l] + 31) / 32);
            k_transpose_f32_bf16<<<grid, dim3(32, 8), 0, st>>>(p->P.w[l], p->B.wt[l], N[l], K[l]);
        }
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? UPPASD_GPU_OK : cuda_fail("proposal weights", e);
}

// Prepare the GEMMs for `rows` rows (forward, backward data, weight gradients).
int prepare(uppasd_gpu_proposal *p, int rows) {
    if (p->prepared_rows == rows) return UPPASD_GPU_OK;
    auto &B = p->B;
    int rc = 0;
    rc = rc ? rc : tc::gemm_prepare(p->fwd[0], B.X, B.wb[0], rows, kHid, kFeat, tc::kEpiBiasTanhBF16, 128, 2);
    rc = rc ? rc : tc::gemm_prepare(p->fwd[1], B.H[0], B.wb[1], rows, kHid, kHid, tc::kEpiBiasTanhBF16, 128, 2);
    rc = rc ? rc : tc::gemm_prepare(p->fwd[2], B.H[1], B.wb[2], rows, kHid, kHid, tc::kEpiBiasTanhBF16, 128, 2);
    rc = rc ? rc : tc::gemm_prepare(p->fwd[3], B.H[2], B.wb[3], rows, kOut, kHid, tc::kEpiBiasF32, 64, 2);
    // backward data: dH3 = (dO W4) (1 - H3^2), dH2 = (dH3 W3) (1 - H2^2), dH1 = (dH2 W2) (1 - H1^2)
    rc = rc ? rc : tc::gemm_prepare(p->bwd[2], B.dO, B.wt[3], rows, kHid, kOut, tc::kEpiDTanhBF16, 128, 2);
    rc = rc ? rc : tc::gemm_prepare(p->bwd[1], B.dH[2], B.wt[2], rows, kHid, kHid, tc::kEpiDTanhBF16, 128, 2);
    rc = rc ? rc : tc::gemm_prepare(p->bwd[0], B.dH[1], B.wt[1], rows, kHid, kHid, tc::kEpiDTanhBF16, 128, 2);
    // weight gradients (K = rows): gW1 = dH1^T X, gW2 = dH2^T H1, gW3 = dH3^T H2, gW4^T = H3^T dO
    rc = rc ? rc : tc::gemm_prepare(p->wgr[0], B.dHt[0], B.Xt, kHid, kFeat, rows, tc::kEpiStoreF32, 64);
    rc = rc ? rc : tc::gemm_prepare(p->wgr[1], B.dHt[1], B.Ht[0], kHid, kHid, rows, tc::kEpiStoreF32, 128);
    rc = rc ? rc : tc::gemm_prepare(p->wgr[2], B.dHt[2], B.Ht[1], kHid, kHid, rows, tc::kEpiStoreF32, 128);
    rc = rc ? rc : tc::gemm_prepare(p->wgr[3], B.Ht[2], B.dOt, kHid, kOut, rows, tc::kEpiStoreF32, 64);
    if (!rc) p->prepared_rows = rows;
    return rc;
}

int forward(uppasd_gpu_proposal *p, cudaStream_t st) {
    auto &B = p->B;
    int rc = tc::gemm_run(p->fwd[0], p->P.b[0], nullptr, nullptr, B.H[0], p->err, st);
    if (!rc) rc = tc::gemm_run(p->fwd[1], p->P.b[1], nullptr, nullptr, B.H[1], p->err, st);
    if (!rc) rc = tc::gemm_run(p->fwd[2], p->P.b[2], nullptr, nullptr, B.H[2], p->err, st);
    if (!rc) rc = tc::gemm_run(p->fwd[3], p->P.b[3], nullptr, B.O, nullptr, p->err, st);
    return rc;
}

// The whole forward pass of the rows in B.X (fused kernel) into B.O.
int forward_fused(uppasd_gpu_proposal *p, int rows, cudaStream_t st) {
    auto &B = p->B;
    if (rows <= 0 || rows % 128 || rows > p->max_rows) {
        set_error("proposal forward: rows must be a positive multiple of 128 within the buffers");
        return UPPASD_GPU_EINVAL;
    }
    if (p->mlp_rows != rows) {
        const int nrow[4] = {kHid, kHid, kHid, kOut}, ncol[4] = {kFeat, kHid, kHid, kHid};
        int rc = tc::make_map(&p->mlp_x, B.X, rows, kFeat, 128);
        for (int l = 0; l < 4 && !rc; ++l) rc = tc::make_map(&p->mlp_w[l], B.wb[l], nrow[l], ncol[l], nrow[l]);
        if (rc) return rc;
        p->mlp_rows = rows;
    }
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(tc::tc_mlp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)tc::mlp_smem_bytes());
        if (e != cudaSuccess) return cuda_fail("proposal forward attribute", e);
        attr_set = true;
    }
    tc::MlpArgs a{};
    for (int l = 0; l < 4; ++l) a.bias[l] = p->P.b[l];
    a.out = B.O;
    a.rows = rows;
    a.err = p->err;
    tc::tc_mlp_kernel<<<rows / 128, tc::kMlpThreads, tc::mlp_smem_bytes(), st>>>(p->mlp_x, p->mlp_w[0], p->mlp_w[1],
                                                                                  p->mlp_w[2], p->mlp_w[3], a);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? UPPASD_GPU_OK : cuda_fail("proposal forward", e);
}

void transpose(const __nv_bfloat16 *src, __nv_bfloat16 *dst, int rows, int cols, cudaStream_t st) {
    dim3 grid((cols + 31) / 32, (rows + 31) / 32);
    k_transpose_bf16<<<grid, dim3(32, 8), 0, st>>>(src, dst, rows, cols);
}

// Loss (into p->loss, accumulated) and gradients (P.gw, P.gb; gW4 transposed in B.gW4t)
// of the rows in B.X.
int loss_and_grad(uppasd_gpu_proposal *p, int rows, cudaStream_t st) {
    auto &B = p->B;
    int rc = prepare(p, rows);
    if (!rc) rc = forward(p, st);
    if (rc) return rc;
    k_loss_grad<<<(rows + 127) / 128, 128, 0, st>>>(rows, p->eta_scale, B.O, B.X, B.dO, p->loss);
    rc = tc::gemm_run(p->bwd[2], nullptr, B.H[2], nullptr, B.dH[2], p->err, st);
    if (!rc) rc = tc::gemm_run(p->bwd[1], nullptr, B.H[1], nullptr, B.dH[1], p->err, st);
    if (!rc) rc = tc::gemm_run(p->bwd[0], nullptr, B.H[0], nullptr, B.dH[0], p->err, st);
    if (rc) return rc;
    transpose(B.X, B.Xt, rows, kFeat, st);
    for (int l = 0; l < 3; ++l) {
        transpose(B.H[l], B.Ht[l], rows, kHid, st);
        transpose(B.dH[l], B.dHt[l], rows, kHid, st);
    }
    transpose(B.dO, B.dOt, rows, kOut, st);
    rc = tc::gemm_run(p->wgr[0], nullptr, nullptr, p->P.gw[0], nullptr, p->err, st);
    if (!rc) rc = tc::gemm_run(p->wgr[1], nullptr, nullptr, p->P.gw[1], nullptr, p->err, st);
    if (!rc) rc = tc::gemm_run(p->wgr[2], nullptr, nullptr, p->P.gw[2], nullptr, p->err, st);
    if (!rc) rc = tc::gemm_run(p->wgr[3], nullptr, nullptr, B.gW4t, nullptr, p->err, st);
    if (rc) return rc;
    for (int l = 0; l < 4; ++l) cudaMemsetAsync(p->P.gb[l], 0, kNB[l] * sizeof(float), st);
    const __nv_bfloat16 *dsrc[4] = {B.dH[0], B.dH[1], B.dH[2], B.dO};
    for (int l = 0; l < 4; ++l) {
        dim3 grid((kNB[l] + 127) / 128, 64);
        k_colsum<<<grid, 128, 0, st>>>(dsrc[l], rows, kNB[l], p->P.gb[l]);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? UPPASD_GPU_OK : cuda_fail("proposal backward", e);
}

int check_err(uppasd_gpu_proposal *p, cudaStream_t st) {
    cudaError_t e = cudaStreamSynchronize(st);
    int h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, p->err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail("proposal", e);
    if (h) {
        set_error("proposal: a tensor-core pipeline wait ran past its limit (code " + std::to_string(h) + ")");
        return UPPASD_GPU_ESTATE;
    }
    return UPPASD_GPU_OK;
}

PatchGeom geom(const uppasd_gpu_proposal *p, int colour) {
    PatchGeom g;
    g.L = p->L;
    g.half = p->L / 8;
    g.np = g.half * g.half;
    g.colour = colour;
    return g;
}

// One learned sweep (the four patch colours) enqueued on `st`; capturable.
int enqueue_sweep(uppasd_gpu_proposal *p, int rows, double beta_mub, bool per_ensemble, cudaStream_t st) {
    Sim &s = p->sim->s;
    if (s.ham.do_dip) {
        set_error("learned moves: the dipolar field is not taken; set_dipole(0) first, or use mc_run");
        return UPPASD_GPU_EUNSUPPORTED;
    }
    const long long nt = (long long)rows * 64;
    int rc;
    for (int c = 0; c < 4; ++c) {
        PatchGeom g = geom(p, c);
        // the square-lattice path reads the FP32 mirror (made ready by the caller)
        const float4 *mirror = s.sq.L == p->L ? s.sqm : nullptr;
        k_gather<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(g, s.e, mirror, s.ham.natom, rows, p->B.X,
                                                                p->old_patch, p->win);
        for (int grp = 0; grp < 4; ++grp) {
            if ((rc = forward_fused(p, rows, st))) return rc;
            k_vmf_group<<<rows / 8, 128, 0, st>>>(rows, grp, p->eta_scale, p->B.O, p->B.X, p->old_patch,
                                                   p->new_patch, p->logq_old, p->logq_new, p->seed, p->dctr, c * 4 + grp);
        }
        if (s.sq.L == p->L) {
            SqCoup q;
            for (int d = 0; d < 4; ++d) {
                q.c[d] = s.sq.c[d];
                for (int cc = 0; cc < 3; ++cc) q.d[d][cc] = s.sq.d[d][cc];
            }
            for (int cc = 0; cc < 3; ++cc) q.ext[cc] = s.sq.ext[cc];
            q.mom = s.sq.mom;
            k_accept_sq<<<(rows * 32 + 255) / 256, 256, 0, st>>>(g, q, s.sqm, s.e, s.eM, s.ham.natom, rows, p->win,
                                                                  p->old_patch,
                                                                  p->new_patch, p->logq_old, p->logq_new, beta_mub,
                                                                  per_ensemble ? s.betak : nullptr, p->seed, p->dctr,
                                                                  c, p->accepted, p->dE_sum);
        } else {
            k_accept<<<(rows * 32 + 255) / 256, 256, 0, st>>>(g, s.ham, s.e, s.eM, s.llg.mmom, rows,
                                                               p->new_patch, p->logq_old, p->logq_new, beta_mub,
                                                               per_ensemble ? s.tk : nullptr, p->seed, p->dctr, c,
                                                               p->accepted, p->dE_sum);
        }
    }
    k_advance<<<1, 1, 0, st>>>(p->dctr);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? UPPASD_GPU_OK : cuda_fail("proposal sweep", e);
}

}  // namespace

extern "C" {

int uppasd_gpu_proposal_create(uppasd_gpu_sim *sim, int32_t L, float eta_scale, int32_t data_capacity,
                               uint64_t seed, uppasd_gpu_proposal **out) {
    if (!sim || !out || L < 8 || L % 8 || !(eta_scale > 0.f) || data_capacity < 0) {
        set_error("proposal_create: need a simulation, L % 8 == 0, eta_scale > 0");
        return UPPASD_GPU_EINVAL;
    }
    *out = nullptr;
    const Sim &s = sim->s;
    if (s.ham.do_jtensor) {
        set_error("proposal_create: the exchange is a tensor; learned patch moves cover scalar exchange");
        return UPPASD_GPU_EUNSUPPORTED;
    }
    if (s.ham.natom != L * L) {
        set_error("proposal_create: the simulation is not an L x L square lattice with one atom per cell");
        return UPPASD_GPU_EINVAL;
    }
    const int rows_colour = s.ham.mensemble * (L / 8) * (L / 8);
    if (rows_colour % 128) {
        set_error("proposal_create: Mensemble * (L/8)^2 must be a multiple of 128");
        return UPPASD_GPU_EINVAL;
    }
    uppasd_gpu_proposal *p = new (std::nothrow) uppasd_gpu_proposal();
    if (!p) return UPPASD_GPU_ENOMEM;
    p->sim = sim;
    p->L = L;
    p->eta_scale = eta_scale;
    p->seed = seed;
    p->max_rows = std::max(rows_colour, 16384);
    p->max_rows = (p->max_rows + 127) / 128 * 128;
    const int R = p->max_rows;
    // parameter-sized arrays: w, b, mask(w only), m, v (w and b), gradients
    long long nw = 0, nb = 0;
    for (int l = 0; l < 4; ++l) {
        nw += kNW[l];
        nb += kNB[l];
    }
    p->nparams = nw + nb;
    cudaError_t e = cudaMalloc(&p->params, (size_t)(nw * 6 + nb * 5) * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(p->params, 0, (size_t)(nw * 6 + nb * 5) * sizeof(float));
    if (e == cudaSuccess) {
        float *q = p->params;
        for (int l = 0; l < 4; ++l) { p->P.w[l] = q; q += kNW[l]; }
        for (int l = 0; l < 4; ++l) { p->P.b[l] = q; q += kNB[l]; }
        for (int l = 0; l < 4; ++l) { p->P.mask[l] = q; q += kNW[l]; }
        for (int l = 0; l < 4; ++l) { p->P.mw[l] = q; q += kNW[l]; }
        for (int l = 0; l < 4; ++l) { p->P.vw[l] = q; q += kNW[l]; }
        for (int l = 0; l < 4; ++l) { p->P.mb[l] = q; q += kNB[l]; }
        for (int l = 0; l < 4; ++l) { p->P.vb[l] = q; q += kNB[l]; }
        for (int l = 0; l < 4; ++l) { p->P.gw[l] = q; q += kNW[l]; }
        for (int l = 0; l < 4; ++l) { p->P.gb[l] = q; q += kNB[l]; }
        (void)q;
    }
    auto al = [&](void **q, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(q, bytes);
        if (e == cudaSuccess) e = cudaMemset(*q, 0, bytes);
    };
    auto &B = p->B;
    al((void **)&B.X, (size_t)R * kFeat * 2);
    al((void **)&B.Xt, (size_t)R * kFeat * 2);
    al((void **)&B.dO, (size_t)R * kOut * 2);
    al((void **)&B.dOt, (size_t)R * kOut * 2);
    al((void **)&B.O, (size_t)R * kOut * 4);
    al((void **)&B.gW4t, (size_t)kHid * kOut * 4);
    for (int l = 0; l < 3; ++l) {
        al((void **)&B.H[l], (size_t)R * kHid * 2);
        al((void **)&B.dH[l], (size_t)R * kHid * 2);
        al((void **)&B.Ht[l], (size_t)R * kHid * 2);
        al((void **)&B.dHt[l], (size_t)R * kHid * 2);
    }
    for (int l = 0; l < 4; ++l) {
        al((void **)&B.wb[l], (size_t)kNW[l] * 2);
        al((void **)&B.wt[l], (size_t)kNW[l] * 2);
    }
    al((void **)&p->old_patch, (size_t)R * 48 * 4);
    al((void **)&p->new_patch, (size_t)R * 48 * 4);
    al((void **)&p->logq_old, (size_t)R * 4);
    al((void **)&p->win, (size_t)R * kFeat * 4);
    al((void **)&p->logq_new, (size_t)R * 4);
    al((void **)&p->accepted, sizeof(unsigned long long));
    al((void **)&p->dE_sum, sizeof(double));
    al((void **)&p->loss, sizeof(double));
    al((void **)&p->err, sizeof(int));
    al((void **)&p->dctr, sizeof(long long));
    p->data_cap = data_capacity;
    if (data_capacity > 0) al((void **)&p->data, (size_t)data_capacity * kFeat * 2);
    if (e != cudaSuccess) {
        int rc = cuda_fail("proposal_create", e);
        free_all(p);
        return rc;
    }
    // masks and initial weights (seeded; masked entries zero)
    std::vector<float> mask[4];
    build_masks(mask);
    const int fan_in[4] = {kFeat, kHid, kHid, kHid};
    for (int l = 0; l < 4 && e == cudaSuccess; ++l) {
        std::vector<float> w(kNW[l]);
        const float sc = (l == 3 ? 0.1f : 1.0f) / std::sqrt((float)fan_in[l]);
        for (int i = 0; i < kNW[l]; ++i) {
            const Philox4 r = philox_draw(seed, i, l, 0, kStreamLearned + 2u);
            const double u1 = u01_open(r.x), u2 = u01_open(r.y);
            const double z = sqrt(-2.0 * log(u1)) * cos(2.0 * kPi * u2);
            w[i] = (float)(z * sc) * mask[l][i];
        }
        e = cudaMemcpy(p->P.w[l], w.data(), kNW[l] * 4, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(p->P.mask[l], mask[l].data(), kNW[l] * 4, cudaMemcpyHostToDevice);
    }
    int rc = e == cudaSuccess ? sync_weights(p, sim->s.stream) : cuda_fail("proposal_create", e);
    // uniform square couplings select the structured energy kernel; anything else
    // (anisotropy, site-dependent couplings) uses the neighbour-list kernel
    if (!rc && sim->s.sq.L != L && square_recognise(sim->s, L) != UPPASD_GPU_OK) sim->s.sq.L = 0;
    if (!rc) rc = check_err(p, sim->s.stream);
    if (rc) {
        free_all(p);
        return rc;
    }
    *out = p;
    return UPPASD_GPU_OK;
}

int uppasd_gpu_proposal_destroy(uppasd_gpu_proposal *p) {
    if (!p) {
        set_error("proposal_destroy: null handle");
        return UPPASD_GPU_EINVAL;
    }
    free_all(p);
    return UPPASD_GPU_OK;
}

int uppasd_gpu_proposal_nparams(uppasd_gpu_proposal *p, int64_t *n) {
    if (!p || !n) {
        set_error("proposal_nparams: null argument");
        return UPPASD_GPU_EINVAL;
    }
    *n = p->nparams;
    return UPPASD_GPU_OK;
}

// Parameter vector layout: W1 (256x192), W2, W3 (256x256), W4 (64x256), then b1, b2, b3, b4.
int uppasd_gpu_proposal_get_params(uppasd_gpu_proposal *p, float *out) {
    if (!p || !out) {
        set_error("proposal_get_params: null argument");
        return UPPASD_GPU_EINVAL;
    }
    cudaError_t e = cudaStreamSynchronize(p->sim->s.stream);
    if (e == cudaSuccess) e = cudaMemcpy(out, p->params, p->nparams * sizeof(float), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? UPPASD_GPU_OK : cuda_fail("proposal_get_params", e);
}

int uppasd_gpu_proposal_set_params(uppasd_gpu_proposal *p, const float *in) {
    if (!p || !in) {
        set_error("proposal_set_params: null argument");
        return UPPASD_GPU_EINVAL;
    }
    // masked weights must be zero
    std::vector<float> mask[4];
    build_masks(mask);
    long long o = 0;
    for (int l = 0; l < 4; ++l) {
        for (int i = 0; i < kNW[l]; ++i)
            if (mask[l][i] == 0.f && in[o + i] != 0.f) {
                set_error("proposal_set_params: a masked (non-autoregressive) weight is non-zero");
                return UPPASD_GPU_EINVAL;
            }
        o += kNW[l];
    }
    cudaStream_t st = p->sim->s.stream;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaMemcpy(p->params, in, p->nparams * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail("proposal_set_params", e);
    int rc = sync_weights(p, st);
    return rc ? rc : check_err(p, st);
}

int uppasd_gpu_proposal_get_masks(uppasd_gpu_proposal *p, float *out) {
    if (!p || !out) {
        set_error("proposal_get_masks: null argument");
        return UPPASD_GPU_EINVAL;
    }
    std::vector<float> mask[4];
    build_masks(mask);
    long long o = 0;
    for (int l = 0; l < 4; ++l) {
        std::memcpy(out + o, mask[l].data(), kNW[l] * sizeof(float));
        o += kNW[l];
    }
    return UPPASD_GPU_OK;
}

// Outputs (rows x 64, fp32 = eta / eta_scale) for explicit inputs (rows x 192, fp32 rounded to bf16).
int uppasd_gpu_proposal_forward(uppasd_gpu_proposal *p, const float *x, int32_t rows, float *out) {
    if (!p || !x || !out || rows <= 0 || rows % 128 || rows > p->max_rows) {
        set_error("proposal_forward: rows must be a positive multiple of 128 within the buffers");
        return UPPASD_GPU_EINVAL;
    }
    cudaStream_t st = p->sim->s.stream;
    float *dx = nullptr;
    cudaError_t e = cudaMalloc(&dx, (size_t)rows * kFeat * 4);
    if (e == cudaSuccess) e = cudaMemcpy(dx, x, (size_t)rows * kFeat * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(dx);
        return cuda_fail("proposal_forward", e);
    }
    k_cast_bf16<<<(rows * kFeat + 255) / 256, 256, 0, st>>>(dx, p->B.X, rows * kFeat);
    int rc = forward_fused(p, rows, st);
    if (!rc) rc = check_err(p, st);
    if (!rc) {
        e = cudaMemcpy(out, p->B.O, (size_t)rows * kOut * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cuda_fail("proposal_forward", e);
    }
    cudaFree(dx);
    return rc;
}

// Loss and gradient (parameter-vector layout) for explicit inputs; no update.
int uppasd_gpu_proposal_loss_grad(uppasd_gpu_proposal *p, const float *x, int32_t rows, double *loss, float *grad) {
    if (!p || !x || !loss || !grad || rows <= 0 || rows % 128 || rows > p->max_rows) {
        set_error("proposal_loss_grad: rows must be a positive multiple of 128 within the buffers");
        return UPPASD_GPU_EINVAL;
    }
    cudaStream_t st = p->sim->s.stream;
    float *dx = nullptr;
    cudaError_t e = cudaMalloc(&dx, (size_t)rows * kFeat * 4);
    if (e == cudaSuccess) e = cudaMemcpy(dx, x, (size_t)rows * kFeat * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemsetAsync(p->loss, 0, sizeof(double), st);
    if (e != cudaSuccess) {
        cudaFree(dx);
        return cuda_fail("proposal_loss_grad", e);
    }
    k_cast_bf16<<<(rows * kFeat + 255) / 256, 256, 0, st>>>(dx, p->B.X, rows * kFeat);
    int rc = loss_and_grad(p, rows, st);
    if (!rc) rc = check_err(p, st);
    if (!rc) {
        // gW4 is held transposed (256 x 64): bring it back to W4's (64 x 256) layout
        std::vector<float> g4t((size_t)kHid * kOut);
        long long o = 0;
        for (int l = 0; l < 3 && e == cudaSuccess; ++l) {
            e = cudaMemcpy(grad + o, p->P.gw[l], kNW[l] * 4, cudaMemcpyDeviceToHost);
            o += kNW[l];
        }
        if (e == cudaSuccess) e = cudaMemcpy(g4t.data(), p->B.gW4t, g4t.size() * 4, cudaMemcpyDeviceToHost);
        for (int oo = 0; oo < kOut; ++oo)
            for (int hh = 0; hh < kHid; ++hh) grad[o + (size_t)oo * kHid + hh] = g4t[(size_t)hh * kOut + oo];
        o += kNW[3];
        for (int l = 0; l < 4 && e == cudaSuccess; ++l) {
            e = cudaMemcpy(grad + o, p->P.gb[l], kNB[l] * 4, cudaMemcpyDeviceToHost);
            o += kNB[l];
        }
        if (e == cudaSuccess) e = cudaMemcpy(loss, p->loss, sizeof(double), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cuda_fail("proposal_loss_grad", e);
        // W4's masked gradient entries read as zero from the host side too
        std::vector<float> mask[4];
        build_masks(mask);
        long long ow = kNW[0] + kNW[1] + kNW[2];
        for (int i = 0; i < kNW[3]; ++i) grad[ow + i] *= mask[3][i];
        ow = 0;
        for (int l = 0; l < 3; ++l) {
            for (int i = 0; i < kNW[l]; ++i) grad[ow + i] *= mask[l][i];
            ow += kNW[l];
        }
    }
    cudaFree(dx);
    return rc;
}

// Append the windows of every patch of every chain (the simulation's current spins).
int uppasd_gpu_proposal_collect(uppasd_gpu_proposal *p) {
    if (!p || p->data_cap <= 0) {
        set_error("proposal_collect: created without a dataset buffer");
        return UPPASD_GPU_EINVAL;
    }
    Sim &s = p->sim->s;
    if (const int rc = sync_state(s)) return rc;  // precision 4: e from its master first
    const int rows = s.ham.mensemble * 4 * (p->L / 8) * (p->L / 8);
    if (rows > p->data_cap) {
        set_error("proposal_collect: the dataset buffer holds fewer rows than one snapshot");
        return UPPASD_GPU_EINVAL;
    }
    // ring buffer: write in one or two pieces
    long long at = p->data_next;
    if (at + rows > p->data_cap) at = 0;
    PatchGeom g = geom(p, -1);
    const long long nt = (long long)rows * 64;
    const bool sq = s.sq.L == p->L;
    if (sq) {
        if (const int rc = square_mirror_ready(s)) return rc;
    }
    k_gather<<<(unsigned)((nt + 255) / 256), 256, 0, s.stream>>>(g, s.e, sq ? s.sqm : nullptr, s.ham.natom, rows,
                                                                 p->data + (size_t)at * kFeat, nullptr, nullptr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail("proposal_collect", e);
    p->data_next = at + rows;
    p->data_count = std::min(p->data_cap, std::max(p->data_count, p->data_next));
    return UPPASD_GPU_OK;
}

// nsteps Adam steps on random minibatches of `rows` dataset rows; losses[i] per step (or NULL).
int uppasd_gpu_proposal_train(uppasd_gpu_proposal *p, int32_t nsteps, int32_t rows, float lr, double *losses) {
    if (!p || nsteps < 0 || rows <= 0 || rows % 128 || rows > p->max_rows || !(lr > 0.f)) {
        set_error("proposal_train: rows must be a positive multiple of 128 within the buffers, lr > 0");
        return UPPASD_GPU_EINVAL;
    }
    if (p->data_count <= 0) {
        set_error("proposal_train: empty dataset (call proposal_collect first)");
        return UPPASD_GPU_ESTATE;
    }
    cudaStream_t st = p->sim->s.stream;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int it = 0; it < nsteps; ++it) {
        cudaError_t e = cudaMemsetAsync(p->loss, 0, sizeof(double), st);
        if (e != cudaSuccess) return cuda_fail("proposal_train", e);
        k_sample_rows<<<rows, 32, 0, st>>>(p->data, p->data_count, rows, p->seed, p->ctr++, p->B.X);
        int rc = loss_and_grad(p, rows, st);
        if (rc) return rc;
        p->adam_t++;
        const float c1 = 1.f - std::pow(b1, (float)p->adam_t), c2 = 1.f - std::pow(b2, (float)p->adam_t);
        for (int l = 0; l < 4; ++l) {
            const int n = kNW[l];
            const float *g = l == 3 ? p->B.gW4t : p->P.gw[l];
            // W4's gradient is held transposed (256 x 64)
            k_adam<<<(n + 255) / 256, 256, 0, st>>>(p->P.w[l], g, p->P.mask[l], p->P.mw[l], p->P.vw[l], n, lr, b1,
                                                     b2, c1, c2, eps, l == 3 ? kOut : 0, l == 3 ? kHid : 0);
            k_adam<<<(kNB[l] + 255) / 256, 256, 0, st>>>(p->P.b[l], p->P.gb[l], nullptr, p->P.mb[l], p->P.vb[l],
                                                          kNB[l], lr, b1, b2, c1, c2, eps, 0, 0);
        }
        rc = sync_weights(p, st);
        if (rc) return rc;
        if (losses) {
            e = cudaMemcpyAsync(losses + it, p->loss, sizeof(double), cudaMemcpyDeviceToHost, st);
            if (e != cudaSuccess) return cuda_fail("proposal_train", e);
        }
    }
    return check_err(p, st);
}

// nsweeps learned sweeps (4 patch colours each) at `temperature` on the simulation's spins.
int uppasd_gpu_proposal_sweep(uppasd_gpu_proposal *p, double temperature, int64_t nsweeps, int64_t *accepted,
                              int64_t *proposed, double *dE_accepted) {
    return uppasd_gpu_proposal_mix(p, temperature, nsweeps, 0, accepted, proposed, dE_accepted);
}

}  // extern "C"

namespace {
// ncycles of (hb_per_cycle structured heat-bath sweeps, then one learned sweep), all
// enqueued on the simulation's stream; one synchronisation at the end.  temps: one
// temperature per ensemble, or null for `temperature`.
int proposal_mix(uppasd_gpu_proposal *p, double temperature, const double *temps, int64_t ncycles,
                 int32_t hb_per_cycle, int64_t *accepted, int64_t *proposed, double *dE_accepted) {
    if (!p || !(temps || temperature > 0.0) || ncycles < 0 || hb_per_cycle < 0) {
        set_error("proposal_mix: bad arguments");
        return UPPASD_GPU_EINVAL;
    }
    Sim &s = p->sim->s;
    if (const int rc = sync_state(s)) return rc;  // precision 4: e from its master first
    const bool per_ens = temps != nullptr;
    if (per_ens) {
        const int rc0 = set_ensemble_temps(s, temps);
        if (rc0) return rc0;
        temperature = -1.0;  // the graph's key: per-ensemble temperatures (read on the device)
    }
    if (s.ham.do_jtensor) {
        set_error("proposal_mix: the exchange became a tensor after the proposal was created");
        return UPPASD_GPU_EUNSUPPORTED;
    }
    cudaStream_t st = s.stream;
    const int rows = s.ham.mensemble * (p->L / 8) * (p->L / 8);
    int rc = prepare(p, rows);
    if (rc) return rc;
    cudaError_t e = cudaMemsetAsync(p->accepted, 0, sizeof(unsigned long long), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(p->dE_sum, 0, sizeof(double), st);
    if (e != cudaSuccess) return cuda_fail("proposal_mix", e);
    const double beta_mub = per_ens ? 0.0 : s.ham.mub / (s.ham.kbolt * temperature);
    s.mix.valid = 0;  // the precision-3 LLG mirror does not follow the learned moves
    if (s.sq.L == p->L) {
        // learned moves on the square lattice read and write the FP32 mirror as well
        if ((rc = square_mirror_ready(s))) return rc;
    } else {
        square_mirror_stale(s);  // the neighbour-list path writes e / eM only
    }
    int64_t done = 0;
    auto heat_bath = [&]() -> int {
        return hb_per_cycle > 0 ? square_sweeps(s, p->L, temperature, per_ens ? s.betak : nullptr, hb_per_cycle) : 0;
    };
    if (ncycles > 0 && !p->warmed) {
        // first sweep eagerly: sets the GEMM kernels' shared-memory attributes before any capture
        if ((rc = heat_bath()) || (rc = enqueue_sweep(p, rows, beta_mub, per_ens, st))) return rc;
        p->warmed = true;
        done = 1;
    }
    if (done < ncycles && (!p->sweep_graph || p->graph_T != temperature || p->graph_rows != rows)) {
        if (p->sweep_graph) cudaGraphExecDestroy(p->sweep_graph);
        p->sweep_graph = nullptr;
        cudaGraph_t g = nullptr;
        e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_fail("proposal_mix capture", e);
        rc = enqueue_sweep(p, rows, beta_mub, per_ens, st);
        e = cudaStreamEndCapture(st, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&p->sweep_graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail("proposal_mix graph", e);
        p->graph_T = temperature;
        p->graph_rows = rows;
    }
    for (; done < ncycles; ++done) {
        if ((rc = heat_bath())) return rc;
        e = cudaGraphLaunch(p->sweep_graph, st);
        if (e != cudaSuccess) return cuda_fail("proposal_mix graph launch", e);
    }
    rc = check_err(p, st);
    if (rc) return rc;
    unsigned long long a = 0;
    double de = 0.0;
    e = cudaMemcpy(&a, p->accepted, sizeof(a), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&de, p->dE_sum, sizeof(de), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail("proposal_mix", e);
    if (accepted) *accepted = (int64_t)a;
    if (proposed) *proposed = (int64_t)rows * 4 * ncycles;
    if (dE_accepted) *dE_accepted = de * s.ham.mub;
    return UPPASD_GPU_OK;
}
}  // namespace

extern "C" {

int uppasd_gpu_proposal_mix(uppasd_gpu_proposal *p, double temperature, int64_t ncycles, int32_t hb_per_cycle,
                            int64_t *accepted, int64_t *proposed, double *dE_accepted) {
    if (!(temperature > 0.0)) {
        set_error("proposal_mix: temperature must be > 0");
        return UPPASD_GPU_EINVAL;
    }
    return proposal_mix(p, temperature, nullptr, ncycles, hb_per_cycle, accepted, proposed, dE_accepted);
}

int uppasd_gpu_proposal_mix_temps(uppasd_gpu_proposal *p, const double *temps, int64_t ncycles, int32_t hb_per_cycle,
                                  int64_t *accepted, int64_t *proposed, double *dE_accepted) {
    if (!temps) {
        set_error("proposal_mix_temps: temperatures required");
        return UPPASD_GPU_EINVAL;
    }
    return proposal_mix(p, 0.0, temps, ncycles, hb_per_cycle, accepted, proposed, dE_accepted);
}

}  // extern "C"
