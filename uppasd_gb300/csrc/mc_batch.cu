// mc_batch.cu -- many Monte Carlo replicas (temperatures x system sizes of
// uneven atom counts) advanced by one persistent launch.
//
// Replica r is a periodic bcc Heisenberg ferromagnet of L^3 conventional cells
// with two exchange shells (J1 on the 8 nearest, J2 on the 6 next-nearest
// neighbours) and an optional uniform Zeeman field.  Two shells admit the
// 4-colour checkerboard (sublattice b x cell parity p): sites of one colour
// share no bond, so a colour updates concurrently.  The sweep order per replica
// is colours (0,0), (0,1), (1,0), (1,1) -- the same chain as the per-colour
// launches of mc.cu and the oracle's checkerboard sweep, with the same Philox
// counters (site, replica, sweep).
//
// HBM layout: per replica four arrays, one per colour, of L^3/2 float4 unit
// spins (w unused), cell (x,y,z) of colour (b,p) at ((z*L + y)*L + x) / 2.  A
// colour's own sites are contiguous, and every neighbour read of a warp is a
// contiguous run in one of the other colour arrays.  No ghost cells: periodic
// wrap by index arithmetic.  The 5.2 M spins of the 64-replica sweep take 83 MB,
// which can stay resident in the 126 MB L2 across sweeps.
//
// Launch: cooperative (all CTAs co-resident).  Replica r owns a contiguous
// group of CTAs (the count per replica is the tile the autotuner picks); a group
// meets at a group barrier after every colour.  The barrier is a 64-bit arrive
// counter per replica with a bounded wait: past the limit a CTA records an
// error and returns, so a launch always ends.
//
// Observables come free with the sweep: updating site i with its neighbours
// fixed changes the energy by exactly -m (e_i' - e_i).(h_i + B) and the moment
// by m (e_i' - e_i).  Each CTA sums these per sweep (FP32 per thread, FP64
// across threads) into a per-(replica, sweep) slot; a scan kernel after the
// launch turns the deltas plus an exact FP64 recount of the starting state into
// the per-sweep energy and magnetisation series, FP64 moments of them, and the
// ring buffer the autocorrelation analysis reads.
//
// Single-spin updates follow the reference: heat bath = flip_h
// (MonteCarlo/montecarlo_common.f90:371-422), Metropolis = choose_random_flip +
// calculate_energy + flip_a (montecarlo_common.f90:25-79, 139-200, 431-865),
// Gaussian width delta = (2/25) (kB T / muB)^0.2 (MonteCarlo/montecarlo.f90:142);
// observables are those of calc_mavrg and calc_energy (Measurement/measurements.f90:211-235,
// Hamiltonian/energy.f90:60-405) accumulated like calc_and_print_cumulant
// (Measurement/prn_averages.f90:919-1095).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "common.cuh"
#include "sim.h"

namespace uppasd {
namespace {

constexpr int kMBMaxThreads = 256;
constexpr int kBarStride = 16;  // 64-bit arrive counters 128 B apart

struct MBRep {
    int L, Lh;              // cells per edge, L/2
    unsigned mL, mLh;       // ceil(2^32 / L), ceil(2^32 / Lh): division by multiply-high
    long long nhalf;        // L^3/2: sites per colour
    long long off;          // float4 offset of the replica's four colour arrays in the pool
    float c1, c2;           // J fc2 / m per shell: field in Tesla from unit-vector neighbours
    float ext[3];           // Zeeman field (T)
    float beta_mu;          // muB m / (kB T)
    float delta;            // Gaussian trial width
    int heatbath;           // 1 heat bath, 0 Metropolis
    int cta_first, cta_count;
    double e_scale;         // unit-vector energy sum -> mRy per atom: m muB / mRy / N
    double m_scale;         // unit-vector moment sum -> muB per atom: m / N
    int slot;               // temperature slot held (replica exchange moves slots between replicas)
};

struct MBParams {
    const MBRep *reps;
    const int *cta_rep;
    int nrep;
    float4 *pool;
    unsigned long long *bar;  // per replica arrive counter (stride kBarStride)
    int *err;
    double *delta;            // [nrep][max_spl][4]: dE, dMx, dMy, dMz of each sweep (unit-vector sums)
    int max_spl;
    double *base;             // [nrep][4]: E, Mx, My, Mz of the state at launch start (unit-vector sums)
    double *acc;              // [nrep][10]: n, E, E^2, |M|, M^2, M^4, Mx, My, Mz, |M|^3
    double *last;             // [nrep][4]: E (mRy/atom), Mx, My, Mz (muB/atom) after the last sweep
    double *series;           // [nrep][series_len][2]: E, |M| ring buffer
    int series_len;
    long long *nsample;       // per replica
    const int *measuring;     // device flag: accumulate moments and series
    long long *sweep_ctr;     // device sweep counter (Philox step)
    long long *rep_ns;        // per replica: ns the group spent in the last launch
    uint64_t seed;
    int rep_id0;              // id of replica 0 in the Philox counters (a share of a larger table)
    long long spin_limit;
    // replica exchange (parallel tempering) between adjacent temperatures of one size
    int *rep_of_slot;             // replica currently at each temperature slot
    const double *slot_beta;      // 1 / (kB T) of each slot (1/J)
    const int2 *pairs;            // (slot a, slot b) ladder neighbours: even pairs then odd pairs
    int npair[2];                 // number of even / odd pairs
    long long *pt_ctr;            // exchange counter (parity of the next attempt)
    unsigned long long *pt_att, *pt_acc;  // attempts / accepts per pair (pairs array order)
};

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *a) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(a) : "memory");
    return v;
}

__device__ __forceinline__ long long globaltimer_ns() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Barrier of the `n` CTAs of one replica; thread 0 of each CTA arrives once.
// Returns false when the wait ran past the limit (error recorded).
__device__ __forceinline__ bool group_barrier(const MBParams &p, int r, int n) {
    __shared__ int failed;
    __syncthreads();
    if (n == 1) return true;  // a one-CTA group: the CTA barrier orders its own global accesses
    if (threadIdx.x == 0) {
        failed = 0;
        unsigned long long *ctr = p.bar + (size_t)r * kBarStride;
        __threadfence();
        const unsigned long long old = atomicAdd(ctr, 1ull);
        const unsigned long long target = (old / (unsigned long long)n + 1ull) * (unsigned long long)n;
        long long it = 0, t0 = 0;
        if (p.spin_limit == 1) {
            // the error path on demand: every CTA of the group gives up at its arrival,
            // so none of them waits for another
            atomicExch(p.err, 1);
            failed = 1;
        }
        while (!failed && ld_acquire_u64(ctr) < target) {
            // give up after spin_limit polls that found the barrier incomplete, or after
            // about two seconds, whichever comes first (the clock is read from poll 64 on)
            ++it;
            if (it == 64) t0 = globaltimer_ns();
            if (it >= p.spin_limit || (it > 64 && (it & 63) == 0 && globaltimer_ns() - t0 > 2000000000LL)) {
                atomicExch(p.err, 1);
                failed = 1;
                break;
            }
            __nanosleep(32);
        }
        __threadfence();
    }
    __syncthreads();
    return failed == 0;
}


// Exchange field on site (b, x, y, z) of parity p and colour-array index t, in Tesla,
// from the unit-vector neighbours; `rep` points at the replica's four colour arrays.
// A neighbour's index is t plus independent x, y, z index steps (periodic wrap folded
// into the step), so the 14 loads need no per-neighbour index arithmetic.
__device__ __forceinline__ float3 exchange_field(const float4 *rep, const MBRep &R, int b, int p, int x, int y,
                                                 int z, int t) {
    const int L = R.L, Lh = R.Lh, nh = (int)R.nhalf, P = L * Lh;
    const int xm = x == 0 ? Lh - 1 : (x & 1) - 1;  // index step of (x-1) >> 1
    const int xp = x == L - 1 ? 1 - Lh : (x & 1);  // index step of (x+1) >> 1
    const int ym = y == 0 ? P - Lh : -Lh;
    const int yp = y == L - 1 ? Lh - P : Lh;
    const int zm = z == 0 ? nh - P : -P;
    const int zp = z == L - 1 ? P - nh : P;
    // nearest: the other sublattice's cells {x, x-1}^3 (b = 0) or {x, x+1}^3 (b = 1);
    // an even number of steps keeps parity p
    const int dx = b ? xp : xm, dy = b ? yp : ym, dz = b ? zp : zm;
    const float4 *ev = rep + (2 * (1 - b) + p) * nh + t;
    const float4 *od = rep + (2 * (1 - b) + (p ^ 1)) * nh + t;
    const float4 v0 = ev[0], v1 = od[dx], v2 = od[dy], v3 = od[dz];
    const float4 v4 = ev[dx + dy], v5 = ev[dx + dz], v6 = ev[dy + dz], v7 = od[dx + dy + dz];
    const float sx = ((v0.x + v1.x) + (v2.x + v3.x)) + ((v4.x + v5.x) + (v6.x + v7.x));
    const float sy = ((v0.y + v1.y) + (v2.y + v3.y)) + ((v4.y + v5.y) + (v6.y + v7.y));
    const float sz = ((v0.z + v1.z) + (v2.z + v3.z)) + ((v4.z + v5.z) + (v6.z + v7.z));
    // next-nearest: same sublattice, opposite parity
    const float4 *nn = rep + (2 * b + (p ^ 1)) * nh + t;
    const float4 n0 = nn[xm], n1 = nn[xp], n2 = nn[ym], n3 = nn[yp], n4 = nn[zm], n5 = nn[zp];
    const float tx = ((n0.x + n1.x) + (n2.x + n3.x)) + (n4.x + n5.x);
    const float ty = ((n0.y + n1.y) + (n2.y + n3.y)) + (n4.y + n5.y);
    const float tz = ((n0.z + n1.z) + (n2.z + n3.z)) + (n4.z + n5.z);
    return make_float3(fmaf(R.c1, sx, R.c2 * tx), fmaf(R.c1, sy, R.c2 * ty), fmaf(R.c1, sz, R.c2 * tz));
}

// (0,1) uniform from a full 32-bit Philox word (the FP64 path's u01_open, rounded to FP32)
__device__ __forceinline__ float u01_full(uint32_t w) {
    const float k32 = 2.3283064365386963e-10f;
    return fmaf((float)w, k32, 0.5f * k32);
}

// flip_h in FP32: draw the new direction from exp(x cos(theta)) about the local field.
// 1 - cos(theta) = -ln((1 - e^-2x) q + e^-2x + tol) / x is formed directly, and the
// field frame from the field's own components (sin of its polar angle from
// |(zx, zy)|, not from 1 - cos^2), so the frame stays orthonormal in FP32.
__device__ __forceinline__ float3 heat_bath_draw(float3 h, float beta_mu, float q, float fp) {
    const float zx = beta_mu * h.x, zy = beta_mu * h.y, zz = beta_mu * h.z;
    const float rxy = sqrtf(zx * zx + zy * zy);
    const float zarg = sqrtf(fmaf(rxy, rxy, zz * zz));
    const float izarg = 1.0f / zarg;
    const float zct = zz * izarg, zst = rxy * izarg;
    const float zcp = rxy > 0.0f ? zx / rxy : 1.0f, zsp = rxy > 0.0f ? zy / rxy : 0.0f;
    const float e2 = __expf(-2.0f * zarg);
    const float omc = fminf(2.0f, fmaxf(0.0f, -__logf(fmaf(1.0f - e2, q, e2) + 1e-14f) * izarg));
    const float ct = 1.0f - omc;
    const float st = sqrtf(omc * (2.0f - omc));
    float sp, cp;
    __sincosf(3.14159265358979f * (2.0f * fp - 1.0f), &sp, &cp);  // argument in [-pi, pi]
    const float s0 = st * cp, s1 = st * sp;
    const float nx = zcp * zct * s0 - zsp * s1 + zcp * zst * ct;
    const float ny = zsp * zct * s0 + zcp * s1 + zsp * zst * ct;
    const float nz = -zst * s0 + zct * ct;
    const float il = rsqrtf(nx * nx + ny * ny + nz * nz);
    return make_float3(nx * il, ny * il, nz * il);
}

// floor(n / d) for n < 2^31 with m = ceil(2^32 / d): the multiply-high estimate is exact or one too large
__device__ __forceinline__ int fast_div(int n, int d, unsigned m) {
    int q = (int)__umulhi((unsigned)n, m);
    return q * d > n ? q - 1 : q;
}

__device__ __forceinline__ void colour_cell(const MBRep &R, int parity, int t, int &x, int &y, int &z) {
    const int row = fast_div(t, R.Lh, R.mLh);
    const int xh = t - row * R.Lh;
    z = fast_div(row, R.L, R.mL);
    y = row - z * R.L;
    x = 2 * xh + ((parity + y + z) & 1);
}

enum : int { kMixed = 0, kHeatBath = 1, kMetropolis = 2 };

// One trial (or heat-bath draw) on site (b, x, y, z): accumulates the energy change
// (unit-vector units, -(e'-e).h) and the moment change when the spin changes.
template <int KIND>
__device__ __forceinline__ void update_site(const MBParams &p, const MBRep &R, const float4 *rep, int r,
                                            long long sweep, int b, int par, int x, int y, int z, int t,
                                            float4 *own, float &dE, float3 &dM) {
    const int site = b + 2 * (x + R.L * (y + R.L * z));
    const Philox4 w = philox_draw(p.seed, site, r + p.rep_id0, sweep, kStreamMC);
    const float3 hx = exchange_field(rep, R, b, par, x, y, z, t);
    const float3 h = make_float3(hx.x + R.ext[0], hx.y + R.ext[1], hx.z + R.ext[2]);
    const float4 cur = *own;
    float3 nm;
    if (KIND == kHeatBath || (KIND == kMixed && R.heatbath)) {
        nm = heat_bath_draw(h, R.beta_mu, u01_full(w.x), u01_full(w.y));
    } else {
        const float u0 = u01_full(w.x);
        const int ftype = (int)floorf(3.0f * u0);
        if (ftype == 0) {
            const float ct = 1.0f - 2.0f * u01_full(w.z);
            const float st = sqrtf(fmaxf(1.0f - ct * ct, 0.0f));
            float sp, cp;
            sincospif(2.0f * u01_full(w.y), &sp, &cp);
            nm = make_float3(st * cp, st * sp, ct);
        } else if (ftype == 1) {
            float g[3];
            normal3_f32(p.seed, site, r + p.rep_id0, sweep, kStreamMCGauss, g);
            const float ax = fmaf(g[0], R.delta, cur.x), ay = fmaf(g[1], R.delta, cur.y),
                        az = fmaf(g[2], R.delta, cur.z);
            const float il = rsqrtf(ax * ax + ay * ay + az * az);
            nm = make_float3(ax * il, ay * il, az * il);
        } else {
            nm = make_float3(-cur.x, -cur.y, -cur.z);
        }
        // beta * dE = beta muB m (e - e').h
        const float bde = R.beta_mu * ((cur.x - nm.x) * h.x + (cur.y - nm.y) * h.y + (cur.z - nm.z) * h.z);
        if (!(bde <= 0.0f || u01_full(w.w) < __expf(-bde))) return;
    }
    const float ddx = nm.x - cur.x, ddy = nm.y - cur.y, ddz = nm.z - cur.z;
    dE -= ddx * h.x + ddy * h.y + ddz * h.z;
    dM.x += ddx;
    dM.y += ddy;
    dM.z += ddz;
    *own = make_float4(nm.x, nm.y, nm.z, 0.f);
}

// MINB: minimum resident CTAs per SM the register allocation is built for (the
// autotuner picks among the builds).
template <int KIND, int MINB>
__global__ void __launch_bounds__(kMBMaxThreads, MINB) mb_sweeps(MBParams p, int nsweeps) {
    __shared__ float wred[kMBMaxThreads / 32][4];
    const int r = p.cta_rep[blockIdx.x];
    const MBRep R = p.reps[r];
    float4 *rep = p.pool + R.off;
    const int g = blockIdx.x - R.cta_first;
    const int gthreads = R.cta_count * blockDim.x;
    const int gtid = g * blockDim.x + threadIdx.x;
    const int nh = (int)R.nhalf;
    const long long sweep0 = *(volatile long long *)p.sweep_ctr;
    const long long t_start = globaltimer_ns();
    for (int sw = 0; sw < nsweeps; ++sw) {
        const long long sweep = sweep0 + sw;
        float dE = 0.f;
        float3 dM = make_float3(0.f, 0.f, 0.f);
        for (int c = 0; c < 4; ++c) {
            const int b = c >> 1, par = c & 1;
            float4 *arr = rep + c * nh;
            for (int t = gtid; t < nh; t += gthreads) {
                int x, y, z;
                colour_cell(R, par, t, x, y, z);
                update_site<KIND>(p, R, rep, r, sweep, b, par, x, y, z, t, arr + t, dE, dM);
            }
            if (c == 3) {
                // per-CTA partial sums of this sweep's changes, one FP64 atomic per CTA and quantity
                float v[4] = {dE, dM.x, dM.y, dM.z};
#pragma unroll
                for (int q = 0; q < 4; ++q) {
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
                }
                if ((threadIdx.x & 31) == 0) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) wred[threadIdx.x >> 5][q] = v[q];
                }
                __syncthreads();
                if (threadIdx.x < 4) {
                    double s = 0.0;
                    for (int wi = 0; wi < (int)(blockDim.x >> 5); ++wi) s += (double)wred[wi][threadIdx.x];
                    atomicAdd(p.delta + ((size_t)r * p.max_spl + sw) * 4 + threadIdx.x, s);
                }
            }
            if (!group_barrier(p, r, R.cta_count)) return;
        }
    }
    if (g == 0 && threadIdx.x == 0) p.rep_ns[r] = globaltimer_ns() - t_start;
}

// Exact FP64 recount of E and M of the current state (unit-vector sums), per replica.
__global__ void __launch_bounds__(kMBMaxThreads) mb_recount(MBParams p) {
    __shared__ double wred[kMBMaxThreads / 32][4];
    const int r = p.cta_rep[blockIdx.x];
    const MBRep R = p.reps[r];
    const float4 *rep = p.pool + R.off;
    const int g = blockIdx.x - R.cta_first;
    const int gthreads = R.cta_count * blockDim.x;
    const int nh = (int)R.nhalf;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int c = 0; c < 4; ++c) {
        const int b = c >> 1, par = c & 1;
        const float4 *arr = rep + c * nh;
        for (int t = g * blockDim.x + threadIdx.x; t < nh; t += gthreads) {
            int x, y, z;
            colour_cell(R, par, t, x, y, z);
            const float4 e = arr[t];
            const float3 hx = exchange_field(rep, R, b, par, x, y, z, t);
            v[0] += -0.5 * ((double)e.x * hx.x + (double)e.y * hx.y + (double)e.z * hx.z) -
                    ((double)e.x * R.ext[0] + (double)e.y * R.ext[1] + (double)e.z * R.ext[2]);
            v[1] += e.x;
            v[2] += e.y;
            v[3] += e.z;
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) wred[threadIdx.x >> 5][q] = v[q];
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double s = 0.0;
        for (int wi = 0; wi < (int)(blockDim.x >> 5); ++wi) s += wred[wi][threadIdx.x];
        atomicAdd(p.base + 4 * r + threadIdx.x, s);
    }
}

// One warp per replica: prefix-sum the launch's per-sweep changes onto the recounted
// start, form E (mRy/atom) and M (muB/atom) per sweep, accumulate their moments and
// the series when measuring, clear the slots, advance the sweep counter.
__global__ void mb_scan(MBParams p, int nsweeps) {
    const int r = blockIdx.x, lane = threadIdx.x;
    const MBRep R = p.reps[r];
    const int sl = R.slot;  // statistics and series belong to the temperature, not the replica
    const bool meas = *p.measuring != 0;
    double run[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) run[q] = p.base[4 * r + q];
    double s[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const long long n0 = p.nsample[sl];
    for (int c0 = 0; c0 < nsweeps; c0 += 32) {
        const int sw = c0 + lane;
        double d[4] = {0.0, 0.0, 0.0, 0.0};
        if (sw < nsweeps) {
            double *slot = p.delta + ((size_t)r * p.max_spl + sw) * 4;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                d[q] = slot[q];
                slot[q] = 0.0;
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double u = __shfl_up_sync(0xffffffffu, d[q], o);
                if (lane >= o) d[q] += u;
            }
        }
        if (sw < nsweeps) {
            const double E = (run[0] + d[0]) * R.e_scale;
            const double Mx = (run[1] + d[1]) * R.m_scale, My = (run[2] + d[2]) * R.m_scale,
                         Mz = (run[3] + d[3]) * R.m_scale;
            const double M2 = Mx * Mx + My * My + Mz * Mz, Ma = sqrt(M2);
            if (meas) {
                s[0] += 1.0;
                s[1] += E;
                s[2] += E * E;
                s[3] += Ma;
                s[4] += M2;
                s[5] += M2 * M2;
                s[6] += Mx;
                s[7] += My;
                s[8] += Mz;
                s[9] += M2 * Ma;
                if (p.series_len > 0) {
                    double *o = p.series + 2 * ((size_t)sl * p.series_len + (size_t)((n0 + sw) % p.series_len));
                    o[0] = E;
                    o[1] = Ma;
                }
            }
            if (sw == nsweeps - 1) {
                p.last[4 * r] = E;
                p.last[4 * r + 1] = Mx;
                p.last[4 * r + 2] = My;
                p.last[4 * r + 3] = Mz;
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) run[q] += __shfl_sync(0xffffffffu, d[q], 31);
    }
#pragma unroll
    for (int q = 0; q < 10; ++q) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_down_sync(0xffffffffu, s[q], o);
    }
    if (lane == 0) {
        if (meas) {
            for (int q = 0; q < 10; ++q) p.acc[10 * sl + q] += s[q];
            p.nsample[sl] = n0 + nsweeps;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) p.base[4 * r + q] = 0.0;
        if (r == 0) *p.sweep_ctr += nsweeps;
    }
}

// Replica exchange between adjacent temperatures of one ladder (one system size),
// even pairs and odd pairs on alternate calls: swap with probability
// min(1, exp((beta_a - beta_b)(E_a - E_b))), E the total energy of the replica
// holding each slot after its last sweep (pt_driver.f90:58-367 restated on the
// batch).  A swap exchanges the temperature parameters of the two replicas; the
// spins stay where they are.  One thread per pair; pairs of one parity are disjoint.
__global__ void mb_swap(MBParams p, MBRep *reps) {
    const long long c = *p.pt_ctr;
    const int par = (int)(c & 1);
    const int n = p.npair[par], first = par ? p.npair[0] : 0;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        const int2 pr = p.pairs[first + q];
        const int ra = p.rep_of_slot[pr.x], rb = p.rep_of_slot[pr.y];
        const MBRep A = reps[ra], B = reps[rb];
        const double ea = p.last[4 * ra] * (double)(4 * A.nhalf) * kMry;
        const double eb = p.last[4 * rb] * (double)(4 * B.nhalf) * kMry;
        const double x = (p.slot_beta[pr.x] - p.slot_beta[pr.y]) * (ea - eb);
        const Philox4 w = philox_draw(p.seed, first + q, 0, c, kStreamLearned + 3u);
        atomicAdd(p.pt_att + first + q, 1ull);
        if (x >= 0.0 || log(u01_open(w.x)) < x) {
            atomicAdd(p.pt_acc + first + q, 1ull);
            reps[ra].beta_mu = B.beta_mu;
            reps[ra].delta = B.delta;
            reps[ra].slot = B.slot;
            reps[rb].beta_mu = A.beta_mu;
            reps[rb].delta = A.delta;
            reps[rb].slot = A.slot;
            p.rep_of_slot[pr.x] = rb;
            p.rep_of_slot[pr.y] = ra;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) *p.pt_ctr = c + 1;
}

}  // namespace
}  // namespace uppasd

struct uppasd_gpu_mcbatch {
    std::vector<uppasd::MBRep> reps;
    std::vector<int> cta_of_rep;
    uppasd::MBParams p{};
    uppasd::MBRep *reps_d = nullptr;
    int *cta_rep_d = nullptr;
    int *measuring_d = nullptr;
    int ctas = 0, threads = 256;
    int kind = 0;   // kMixed / kHeatBath / kMetropolis
    int build = 0;  // register build (index into kRegBuilds)
    long long total_sites = 0, pool_f4 = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaGraphExec_t graph = nullptr;
    int graph_sweeps = 0;
    int measuring_h = 0;
    // replica exchange
    bool exchange = false;
    std::vector<double> temperature;   // per slot
    int *rep_of_slot_d = nullptr;
    double *slot_beta_d = nullptr;
    int2 *pairs_d = nullptr;
    long long *pt_ctr_d = nullptr;
    unsigned long long *pt_att_d = nullptr, *pt_acc_d = nullptr;
    std::vector<int2> pairs_h;
};

namespace {
using uppasd::MBRep;
using uppasd::set_error;

void mb_free(uppasd_gpu_mcbatch *b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    void *ptrs[] = {b->reps_d,  b->cta_rep_d, b->measuring_d, b->p.pool,      b->p.bar,       b->p.err,
                    b->p.delta, b->p.base,    b->p.acc,       b->p.last,      b->p.series,    b->p.nsample,
                    b->p.sweep_ctr, b->p.rep_ns, b->rep_of_slot_d, b->slot_beta_d, b->pairs_d, b->pt_ctr_d,
                    b->pt_att_d, b->pt_acc_d};
    for (void *q : ptrs) cudaFree(q);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int cuda_fail(const char *what, cudaError_t e) {
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? UPPASD_GPU_ENOMEM : UPPASD_GPU_ECUDA;
}

// CTA counts proportional to `work`, at least one each, summing to `ctas`.
std::vector<int> proportional(const std::vector<double> &work, int ctas) {
    const int n = (int)work.size();
    std::vector<int> c(n, 1);
    double tot = 0;
    for (double w : work) tot += w;
    for (int left = ctas - n; left > 0; --left) {
        int best = 0;
        double bestd = -1e300;
        for (int i = 0; i < n; ++i) {
            const double d = (double)ctas * work[i] / tot - c[i];
            if (d > bestd) {
                bestd = d;
                best = i;
            }
        }
        c[best]++;
    }
    return c;
}

using SweepKernel = void (*)(uppasd::MBParams, int);
constexpr int kRegBuilds[3] = {1, 3, 4};  // MINB of the register builds

template <int KIND>
SweepKernel sweep_kernel_k(int build) {
    return build == 2 ? uppasd::mb_sweeps<KIND, kRegBuilds[2]>
           : build == 1 ? uppasd::mb_sweeps<KIND, kRegBuilds[1]>
                        : uppasd::mb_sweeps<KIND, kRegBuilds[0]>;
}

SweepKernel sweep_kernel(int kind, int build) {
    return kind == uppasd::kHeatBath     ? sweep_kernel_k<uppasd::kHeatBath>(build)
           : kind == uppasd::kMetropolis ? sweep_kernel_k<uppasd::kMetropolis>(build)
                                         : sweep_kernel_k<uppasd::kMixed>(build);
}

int max_coresident(int kind, int build, int threads, int *ctas_per_sm_max, int *nsm) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm_max, sweep_kernel(kind, build), threads, 0);
    if (e != cudaSuccess) return cuda_fail("mcbatch occupancy", e);
    if (*ctas_per_sm_max <= 0) {
        set_error("mcbatch: kernel does not fit on an SM at this block size");
        return UPPASD_GPU_EINVAL;
    }
    return UPPASD_GPU_OK;
}

// Install a schedule: register build, `threads` per CTA and `per_rep[i]` CTAs for replica i.
int install(uppasd_gpu_mcbatch *b, int build, int threads, const std::vector<int> &per_rep) {
    int occ = 0, nsm = 0, rc;
    if (build < 0 || build > 2) {
        set_error("mcbatch: register build must be 0, 1 or 2");
        return UPPASD_GPU_EINVAL;
    }
    if ((rc = max_coresident(b->kind, build, threads, &occ, &nsm))) return rc;
    long long tot = 0;
    for (int c : per_rep) {
        if (c < 1) {
            set_error("mcbatch: every replica needs at least one CTA");
            return UPPASD_GPU_EINVAL;
        }
        tot += c;
    }
    if (tot > (long long)occ * nsm) {
        set_error("mcbatch: schedule exceeds the co-resident CTA count (" + std::to_string((long long)occ * nsm) +
                  ")");
        return UPPASD_GPU_EINVAL;
    }
    cudaError_t es = cudaStreamSynchronize(b->stream);
    // the device copy holds the current temperature of each replica (exchange moves them)
    if (es == cudaSuccess)
        es = cudaMemcpy(b->reps.data(), b->reps_d, b->reps.size() * sizeof(MBRep), cudaMemcpyDeviceToHost);
    if (es != cudaSuccess) return cuda_fail("mcbatch schedule", es);
    std::vector<int> map;
    map.reserve((size_t)tot);
    for (size_t i = 0; i < b->reps.size(); ++i) {
        b->reps[i].cta_first = (int)map.size();
        b->reps[i].cta_count = per_rep[i];
        for (int q = 0; q < per_rep[i]; ++q) map.push_back((int)i);
    }
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_fail("mcbatch schedule", e);
    // the arrive counters count in multiples of the group size: restart them for the new groups
    e = cudaMemset(b->p.bar, 0, b->reps.size() * uppasd::kBarStride * sizeof(unsigned long long));
    if (e != cudaSuccess) return cuda_fail("mcbatch schedule", e);
    cudaFree(b->cta_rep_d);
    b->cta_rep_d = nullptr;
    if ((e = cudaMalloc(&b->cta_rep_d, map.size() * sizeof(int))) != cudaSuccess ||
        (e = cudaMemcpy(b->cta_rep_d, map.data(), map.size() * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(b->reps_d, b->reps.data(), b->reps.size() * sizeof(MBRep), cudaMemcpyHostToDevice)) !=
            cudaSuccess)
        return cuda_fail("mcbatch schedule", e);
    b->p.cta_rep = b->cta_rep_d;
    b->ctas = (int)map.size();
    b->threads = threads;
    b->build = build;
    b->cta_of_rep = per_rep;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return UPPASD_GPU_OK;
}

// recount -> persistent sweeps -> scan, on b->stream (capturable)
int enqueue_chunk(uppasd_gpu_mcbatch *b, int n) {
    uppasd::MBParams p = b->p;
    uppasd::mb_recount<<<b->ctas, b->threads, 0, b->stream>>>(p);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(b->ctas);
    cfg.blockDim = dim3(b->threads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = b->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, sweep_kernel(b->kind, b->build), p, n);
    if (e != cudaSuccess) return cuda_fail("mcbatch sweep launch", e);
    uppasd::mb_scan<<<p.nrep, 32, 0, b->stream>>>(p, n);
    if (b->exchange) uppasd::mb_swap<<<1, 256, 0, b->stream>>>(p, b->reps_d);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail("mcbatch launch", e);
    return UPPASD_GPU_OK;
}

// polls of a group barrier's wait by default: beyond any real wait; the wait's own time
// limit (about two seconds) is what ends a stalled group
constexpr long long kDefaultSpinLimit = 1LL << 40;

// Initial state: uniform on the sphere, Philox (site, replica id, 0, stream
// kStreamLearned + 1), replica ids rep_id0, rep_id0 + 1, ...
int draw_initial_state(uppasd_gpu_mcbatch *b) {
    std::vector<float4> h((size_t)b->pool_f4);
    const uint64_t seed = b->p.seed;
    for (size_t i = 0; i < b->reps.size(); ++i) {
        const MBRep &R = b->reps[i];
        const int id = (int)i + b->p.rep_id0;
        for (int c = 0; c < 4; ++c)
            for (long long t = 0; t < R.nhalf; ++t) {
                const int bb = c >> 1, par = c & 1;
                const long long row = t / R.Lh;
                const int xh = (int)(t - row * R.Lh), z = (int)(row / R.L), y = (int)(row - (long long)z * R.L);
                const int x = 2 * xh + ((par + y + z) & 1);
                const long long site = bb + 2LL * (x + (long long)R.L * (y + (long long)R.L * z));
                const uppasd::Philox4 w = uppasd::philox_draw(seed, site, id, 0, uppasd::kStreamLearned + 1u);
                const double ct = 1.0 - 2.0 * uppasd::u01_open(w.x), st = sqrt(std::max(0.0, 1.0 - ct * ct));
                const double ph = 2.0 * uppasd::kPi * uppasd::u01_open(w.y);
                h[(size_t)(R.off + c * R.nhalf + t)] =
                    make_float4((float)(st * cos(ph)), (float)(st * sin(ph)), (float)ct, 0.f);
            }
    }
    cudaError_t e = cudaMemcpy(b->p.pool, h.data(), (size_t)b->pool_f4 * sizeof(float4), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail("mcbatch initial state", e);
    return UPPASD_GPU_OK;
}

int check_err(uppasd_gpu_mcbatch *b) {
    cudaError_t e = cudaStreamSynchronize(b->stream);
    int err = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&err, b->p.err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail("mcbatch", e);
    if (err) {
        // the groups that gave up left their arrive counters out of step: start every
        // counter and the flag afresh, so that the next launch's barriers line up again
        const int zero = 0;
        e = cudaMemset(b->p.bar, 0, b->reps.size() * uppasd::kBarStride * sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMemcpy(b->p.err, &zero, sizeof(int), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail("mcbatch barrier reset", e);
        set_error("mcbatch: a replica group barrier wait ran past its limit");
        return UPPASD_GPU_ESTATE;
    }
    return UPPASD_GPU_OK;
}

int set_measuring(uppasd_gpu_mcbatch *b, int m) {
    if (b->measuring_h == m) return UPPASD_GPU_OK;
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e == cudaSuccess) e = cudaMemcpy(b->measuring_d, &m, sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail("mcbatch measuring flag", e);
    b->measuring_h = m;
    return UPPASD_GPU_OK;
}

int run_sweeps(uppasd_gpu_mcbatch *b, long long nsweeps, int spl) {
    int rc;
    const long long whole = nsweeps / spl;
    const int rest = (int)(nsweeps - whole * spl);
    if (whole > 0) {
        if (!b->graph || b->graph_sweeps != spl) {
            if (b->graph) cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return cuda_fail("mcbatch capture", e);
            rc = enqueue_chunk(b, spl);
            e = cudaStreamEndCapture(b->stream, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
            if (g) cudaGraphDestroy(g);
            if (e != cudaSuccess) return cuda_fail("mcbatch graph", e);
            b->graph_sweeps = spl;
        }
        for (long long i = 0; i < whole; ++i) {
            cudaError_t e = cudaGraphLaunch(b->graph, b->stream);
            if (e != cudaSuccess) return cuda_fail("mcbatch graph launch", e);
        }
    }
    if (rest > 0 && (rc = enqueue_chunk(b, rest))) return rc;
    return UPPASD_GPU_OK;
}

// ---- autotuner ---------------------------------------------------------------
// For each register build (kRegBuilds), block size (64, 128, 256) and CTAs per SM
// (1 .. occupancy): start from
// CTA counts proportional to the replicas' sites, then rebalance from the
// per-group times the kernel records (work_i ~ t_i n_i, n_i proportional to
// work_i), keeping the fastest measured schedule.  Results are cached per device
// and replica table in a text file, one line per key.

std::string tune_key(const uppasd_gpu_mcbatch *b) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp pr{};
    cudaGetDeviceProperties(&pr, dev);
    std::ostringstream k;
    k << "mcbatch-v2|" << pr.name << "|" << pr.multiProcessorCount << "|";
    for (const MBRep &R : b->reps) k << R.L << (R.heatbath ? 'H' : 'M') << ",";
    std::string s = k.str();
    for (char &c : s)
        if (c == ' ') c = '_';
    return s;
}

bool cache_lookup(const char *path, const std::string &key, int nrep, int *build, int *threads,
                  std::vector<int> &per_rep) {
    if (!path) return false;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream ls(line);
        std::string k;
        int bld = 0, t = 0, n = 0;
        if (!(ls >> k >> bld >> t >> n) || k != key || n != nrep) continue;
        std::vector<int> v(nrep);
        bool ok = true;
        for (int i = 0; i < nrep && ok; ++i) ok = (bool)(ls >> v[i]) && v[i] >= 1;
        if (!ok) continue;
        *build = bld;
        *threads = t;
        per_rep = v;
        return true;
    }
    return false;
}

void cache_store(const char *path, const std::string &key, int build, int threads, const std::vector<int> &per_rep) {
    if (!path) return;
    std::vector<std::string> keep;
    {
        std::ifstream f(path);
        std::string line;
        while (std::getline(f, line))
            if (line.compare(0, key.size() + 1, key + " ") != 0) keep.push_back(line);
    }
    std::ofstream f(path, std::ios::trunc);
    for (const auto &l : keep) f << l << "\n";
    f << key << " " << build << " " << threads << " " << per_rep.size();
    for (int c : per_rep) f << " " << c;
    f << "\n";
}

int time_schedule(uppasd_gpu_mcbatch *b, int sweeps, float *ms, std::vector<long long> *rep_ns) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = enqueue_chunk(b, sweeps);  // warm-up of this schedule
    if (!rc) {
        cudaEventRecord(e0, b->stream);
        rc = enqueue_chunk(b, sweeps);
        cudaEventRecord(e1, b->stream);
    }
    if (!rc) rc = check_err(b);
    if (!rc) cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!rc && rep_ns) {
        rep_ns->resize(b->reps.size());
        cudaError_t e =
            cudaMemcpy(rep_ns->data(), b->p.rep_ns, b->reps.size() * sizeof(long long), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail("mcbatch tune", e);
    }
    return rc;
}

}  // namespace

extern "C" {

int uppasd_gpu_mcbatch_create(int32_t nrep, const int32_t *L, const double *temperature, const int32_t *heatbath,
                              const double *j_shells_mry, double mom, const double *bfield, uint64_t seed,
                              int32_t series_len, int32_t max_sweeps_per_launch, uppasd_gpu_mcbatch **out) {
    if (!out || nrep <= 0 || !L || !temperature || !j_shells_mry || !(mom > 0.0) || series_len < 0 ||
        max_sweeps_per_launch < 1 || max_sweeps_per_launch > 65536) {
        set_error("mcbatch_create: bad arguments");
        return UPPASD_GPU_EINVAL;
    }
    *out = nullptr;
    for (int i = 0; i < nrep; ++i) {
        if (L[i] < 4 || (L[i] & 1) || L[i] > 1024) {
            set_error("mcbatch_create: every L must be even with 4 <= L <= 1024");
            return UPPASD_GPU_EINVAL;
        }
        if (!(temperature[i] > 0.0)) {
            set_error("mcbatch_create: temperatures must be positive");
            return UPPASD_GPU_EINVAL;
        }
    }
    int dev = 0, coop = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess) {
        set_error("mcbatch_create: no CUDA device");
        return UPPASD_GPU_ENODEV;
    }
    if (!coop) {
        set_error("mcbatch_create: device lacks cooperative launch");
        return UPPASD_GPU_ENODEV;
    }
    uppasd_gpu_mcbatch *b = new (std::nothrow) uppasd_gpu_mcbatch();
    if (!b) return UPPASD_GPU_ENOMEM;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    b->own_stream = e == cudaSuccess;
    const double fc2 = 2.0 * uppasd::kMry / uppasd::kMub;
    long long pool = 0;
    for (int i = 0; i < nrep; ++i) {
        MBRep R{};
        R.L = L[i];
        R.Lh = L[i] / 2;
        R.mL = (unsigned)((0x100000000ull + (unsigned)R.L - 1) / (unsigned)R.L);
        R.mLh = (unsigned)((0x100000000ull + (unsigned)R.Lh - 1) / (unsigned)R.Lh);
        R.nhalf = (long long)L[i] * L[i] * L[i] / 2;
        R.off = pool;
        pool += 4 * R.nhalf;
        // reference coupling ncoup = J fc2 / m^2 acts on full moments: J fc2 / m on unit vectors
        R.c1 = (float)(j_shells_mry[0] * fc2 / mom);
        R.c2 = (float)(j_shells_mry[1] * fc2 / mom);
        for (int c = 0; c < 3; ++c) R.ext[c] = bfield ? (float)bfield[c] : 0.f;
        R.beta_mu = (float)(uppasd::kMub * mom / (uppasd::kKbolt * temperature[i]));
        R.delta = (float)((double)(2.0f / 25.0f) * pow(uppasd::kKbolt * temperature[i] / uppasd::kMub, 0.20));
        R.heatbath = heatbath ? (heatbath[i] ? 1 : 0) : 1;
        R.slot = i;
        b->temperature.push_back(temperature[i]);
        const double natom = 4.0 * (double)R.nhalf;  // 2 L^3
        R.e_scale = mom * uppasd::kMub / uppasd::kMry / natom;
        R.m_scale = mom / natom;
        b->reps.push_back(R);
        b->total_sites += 4 * R.nhalf;
    }
    b->pool_f4 = pool;
    auto al = [&](void **q, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(q, bytes);
        if (e == cudaSuccess) e = cudaMemset(*q, 0, bytes);
    };
    al((void **)&b->reps_d, nrep * sizeof(MBRep));
    al((void **)&b->measuring_d, sizeof(int));
    al((void **)&b->p.pool, pool * sizeof(float4));
    al((void **)&b->p.bar, (size_t)nrep * uppasd::kBarStride * sizeof(unsigned long long));
    al((void **)&b->p.err, sizeof(int));
    al((void **)&b->p.delta, (size_t)nrep * max_sweeps_per_launch * 4 * sizeof(double));
    al((void **)&b->p.base, (size_t)nrep * 4 * sizeof(double));
    al((void **)&b->p.acc, (size_t)nrep * 10 * sizeof(double));
    al((void **)&b->p.last, (size_t)nrep * 4 * sizeof(double));
    al((void **)&b->p.nsample, (size_t)nrep * sizeof(long long));
    al((void **)&b->p.sweep_ctr, sizeof(long long));
    al((void **)&b->p.rep_ns, (size_t)nrep * sizeof(long long));
    if (series_len > 0) al((void **)&b->p.series, (size_t)nrep * series_len * 2 * sizeof(double));
    al((void **)&b->rep_of_slot_d, (size_t)nrep * sizeof(int));
    al((void **)&b->slot_beta_d, (size_t)nrep * sizeof(double));
    al((void **)&b->pt_ctr_d, sizeof(long long));
    if (e == cudaSuccess) {
        std::vector<int> id(nrep);
        std::vector<double> beta(nrep);
        for (int i = 0; i < nrep; ++i) {
            id[i] = i;
            beta[i] = 1.0 / (uppasd::kKbolt * temperature[i]);
        }
        e = cudaMemcpy(b->rep_of_slot_d, id.data(), nrep * sizeof(int), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(b->slot_beta_d, beta.data(), nrep * sizeof(double), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        int rc = cuda_fail("mcbatch_create", e);
        mb_free(b);
        return rc;
    }
    // the device copy of the replica table is authoritative from here on (replica
    // exchange edits temperatures in place; install() reads it back)
    if (e == cudaSuccess) e = cudaMemcpy(b->reps_d, b->reps.data(), nrep * sizeof(MBRep), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        int rc = cuda_fail("mcbatch_create", e);
        mb_free(b);
        return rc;
    }
    b->p.reps = b->reps_d;
    b->p.nrep = nrep;
    b->p.max_spl = max_sweeps_per_launch;
    b->p.series_len = series_len;
    b->p.measuring = b->measuring_d;
    b->p.seed = seed;
    b->p.rep_of_slot = b->rep_of_slot_d;
    b->p.slot_beta = b->slot_beta_d;
    b->p.pt_ctr = b->pt_ctr_d;
    b->p.spin_limit = kDefaultSpinLimit;
    b->p.rep_id0 = 0;
    {
        const int rc = draw_initial_state(b);
        if (rc) {
            mb_free(b);
            return rc;
        }
    }
    // default schedule: the 3-CTAs-per-SM register build, 256 threads, all co-resident
    // CTAs, counts proportional to sites
    int occ = 0, nsm = 0;
    {
        int nh = 0;
        for (const MBRep &R : b->reps) nh += R.heatbath;
        b->kind = nh == nrep ? uppasd::kHeatBath : (nh == 0 ? uppasd::kMetropolis : uppasd::kMixed);
    }
    int rc = max_coresident(b->kind, 1, 256, &occ, &nsm);
    if (!rc) {
        std::vector<double> work;
        for (const MBRep &R : b->reps) work.push_back((double)R.nhalf);
        if (occ * nsm < nrep) {
            set_error("mcbatch_create: more replicas than co-resident CTAs");
            rc = UPPASD_GPU_EINVAL;
        } else {
            rc = install(b, 1, 256, proportional(work, occ * nsm));
        }
    }
    if (rc) {
        mb_free(b);
        return rc;
    }
    *out = b;
    return UPPASD_GPU_OK;
}

int uppasd_gpu_mcbatch_set_stream(uppasd_gpu_mcbatch *b, void *cuda_stream) {
    if (!b) {
        set_error("mcbatch_set_stream: null handle");
        return UPPASD_GPU_EINVAL;
    }
    cudaStreamSynchronize(b->stream);
    if (b->own_stream) cudaStreamDestroy(b->stream);
    b->own_stream = false;
    b->stream = (cudaStream_t)cuda_stream;
    if (!cuda_stream) {
        if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
            set_error("mcbatch_set_stream: stream creation failed");
            return UPPASD_GPU_ECUDA;
        }
        b->own_stream = true;
    }
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return UPPASD_GPU_OK;
}

int uppasd_gpu_mcbatch_set_schedule(uppasd_gpu_mcbatch *b, int32_t reg_build, int32_t threads,
                                    const int32_t *ctas_per_rep) {
    if (!b || threads < 32 || threads > uppasd::kMBMaxThreads || (threads & 31) || !ctas_per_rep) {
        set_error("mcbatch_set_schedule: threads must be a multiple of 32 in [32, 256], counts non-null");
        return UPPASD_GPU_EINVAL;
    }
    std::vector<int> v(ctas_per_rep, ctas_per_rep + b->reps.size());
    return install(b, reg_build, threads, v);
}

int uppasd_gpu_mcbatch_get_schedule(uppasd_gpu_mcbatch *b, int32_t *reg_build, int32_t *threads,
                                    int32_t *ctas_per_rep) {
    if (!b || !reg_build || !threads || !ctas_per_rep) {
        set_error("mcbatch_get_schedule: null argument");
        return UPPASD_GPU_EINVAL;
    }
    *reg_build = b->build;
    *threads = b->threads;
    for (size_t i = 0; i < b->reps.size(); ++i) ctas_per_rep[i] = b->cta_of_rep[i];
    return UPPASD_GPU_OK;
}

int uppasd_gpu_mcbatch_autotune(uppasd_gpu_mcbatch *b, int32_t sweeps_per_trial, const char *cache_path,
                                float *best_ms_per_sweep) {
    if (!b || sweeps_per_trial < 1 || sweeps_per_trial > b->p.max_spl) {
        set_error("mcbatch_autotune: bad arguments");
        return UPPASD_GPU_EINVAL;
    }
    int rc = set_measuring(b, 0);
    if (rc) return rc;
    const int nrep = (int)b->reps.size();
    const std::string key = tune_key(b);
    int build = 0, threads = 0;
    std::vector<int> cached;
    if (cache_lookup(cache_path, key, nrep, &build, &threads, cached) &&
        install(b, build, threads, cached) == UPPASD_GPU_OK) {
        float ms = 0.f;
        if ((rc = time_schedule(b, sweeps_per_trial, &ms, nullptr))) return rc;
        if (best_ms_per_sweep) *best_ms_per_sweep = ms / sweeps_per_trial;
        return UPPASD_GPU_OK;
    }
    float best = 1e30f;
    int best_build = b->build, best_threads = b->threads;
    std::vector<int> best_rep = b->cta_of_rep;
    std::vector<double> sites;
    for (const MBRep &R : b->reps) sites.push_back((double)R.nhalf);
    for (int bld = 0; bld < 3; ++bld) {
        for (int t : {64, 128, 256}) {
            int occ = 0, nsm = 0;
            if (max_coresident(b->kind, bld, t, &occ, &nsm)) continue;
            for (int per_sm = 1; per_sm <= occ; per_sm = per_sm < 4 ? per_sm + 1 : per_sm * 2) {
                const int total = per_sm * nsm;
                if (total < nrep) continue;
                std::vector<int> cur = proportional(sites, total);
                for (int it = 0; it < 4; ++it) {
                    if ((rc = install(b, bld, t, cur))) return rc;
                    float ms = 0.f;
                    std::vector<long long> ns;
                    if ((rc = time_schedule(b, sweeps_per_trial, &ms, &ns))) return rc;
                    if (ms < best) {
                        best = ms;
                        best_build = bld;
                        best_threads = t;
                        best_rep = cur;
                    }
                    // rebalance: a group's work ~ its time x its CTAs
                    std::vector<double> work(nrep);
                    for (int i = 0; i < nrep; ++i) work[i] = (double)std::max<long long>(ns[i], 1) * cur[i];
                    std::vector<int> next = proportional(work, total);
                    if (next == cur) break;
                    cur = next;
                }
            }
        }
    }
    if ((rc = install(b, best_build, best_threads, best_rep))) return rc;
    cache_store(cache_path, key, best_build, best_threads, best_rep);
    if (best_ms_per_sweep) *best_ms_per_sweep = best / sweeps_per_trial;
    return UPPASD_GPU_OK;
}

int uppasd_gpu_mcbatch_run(uppasd_gpu_mcbatch *b, int64_t nsweeps, int32_t sweeps_per_launch, int32_t measure) {
    if (!b || nsweeps < 0 || sweeps_per_launch < 1 || sweeps_per_launch > b->p.max_spl) {
        set_error("mcbatch_run: bad arguments (sweeps_per_launch must be in [1, max_sweeps_per_launch])");
        return UPPASD_GPU_EINVAL;
    }
    int rc = set_measuring(b, measure ? 1 : 0);
    if (rc) return rc;
    if ((rc = run_sweeps(b, nsweeps, sweeps_per_launch))) return rc;
    return check_err(b);
}

// Enqueue only (no synchronisation), e.g. for callers timing on their own stream.
int uppasd_gpu_mcbatch_enqueue(uppasd_gpu_mcbatch *b, int64_t nsweeps, int32_t sweeps_per_launch, int32_t measure) {
    if (!b || nsweeps < 0 || sweeps_per_launch < 1 || sweeps_per_launch > b->p.max_spl) {
        set_error("mcbatch_enqueue: bad arguments");
        return UPPASD_GPU_EINVAL;
    }
    int rc = set_measuring(b, measure ? 1 : 0);
    if (rc) return rc;
    return run_sweeps(b, nsweeps, sweeps_per_launch);
}

int uppasd_gpu_mcbatch_check(uppasd_gpu_mcbatch *b) {
    if (!b) {
        set_error("mcbatch_check: null handle");
        return UPPASD_GPU_EINVAL;
    }
    return check_err(b);
}

int uppasd_gpu_mcbatch_stats(uppasd_gpu_mcbatch *b, double *acc, int64_t *nsample, double *last) {
    if (!b) {
        set_error("mcbatch_stats: null handle");
        return UPPASD_GPU_EINVAL;
    }
    const size_t nrep = b->reps.size();
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e == cudaSuccess && acc) e = cudaMemcpy(acc, b->p.acc, nrep * 10 * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && nsample)
        e = cudaMemcpy(nsample, b->p.nsample, nrep * sizeof(long long), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && last) e = cudaMemcpy(last, b->p.last, nrep * 4 * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail("mcbatch_stats", e);
    return UPPASD_GPU_OK;
}

int uppasd_gpu_mcbatch_series(uppasd_gpu_mcbatch *b, double *series) {
    if (!b || !series || b->p.series_len <= 0) {
        set_error("mcbatch_series: no series buffer");
        return UPPASD_GPU_EINVAL;
    }
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e == cudaSuccess)
        e = cudaMemcpy(series, b->p.series, b->reps.size() * (size_t)b->p.series_len * 2 * sizeof(double),
                       cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail("mcbatch_series", e);
    return UPPASD_GPU_OK;
}

int uppasd_gpu_mcbatch_reset_stats(uppasd_gpu_mcbatch *b) {
    if (!b) {
        set_error("mcbatch_reset_stats: null handle");
        return UPPASD_GPU_EINVAL;
    }
    const size_t nrep = b->reps.size();
    cudaError_t e = cudaMemsetAsync(b->p.acc, 0, nrep * 10 * sizeof(double), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->p.nsample, 0, nrep * sizeof(long long), b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_fail("mcbatch_reset_stats", e);
    return UPPASD_GPU_OK;
}

// Spins of every replica in the reference layout: replica-major, each (3, 2 L^3)
// with site i = b + 2 (x + L (y + L z)).
int uppasd_gpu_mcbatch_get_spins(uppasd_gpu_mcbatch *b, double *emom) {
    if (!b || !emom) {
        set_error("mcbatch_get_spins: null argument");
        return UPPASD_GPU_EINVAL;
    }
    std::vector<float4> h((size_t)b->pool_f4);
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e == cudaSuccess) e = cudaMemcpy(h.data(), b->p.pool, h.size() * sizeof(float4), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail("mcbatch_get_spins", e);
    double *o = emom;
    for (const MBRep &R : b->reps) {
        const long long n = 4 * R.nhalf;
        for (long long i = 0; i < n; ++i) {
            const int bb = (int)(i & 1);
            const long long cell = i >> 1;
            const int x = (int)(cell % R.L), y = (int)((cell / R.L) % R.L), z = (int)(cell / ((long long)R.L * R.L));
            const int par = (x + y + z) & 1;
            const float4 v = h[(size_t)(R.off + (2 * bb + par) * R.nhalf + ((long long)z * R.L + y) * R.Lh + x / 2)];
            o[3 * i] = v.x;
            o[3 * i + 1] = v.y;
            o[3 * i + 2] = v.z;
        }
        o += 3 * n;
    }
    return UPPASD_GPU_OK;
}

int uppasd_gpu_mcbatch_put_spins(uppasd_gpu_mcbatch *b, const double *emom) {
    if (!b || !emom) {
        set_error("mcbatch_put_spins: null argument");
        return UPPASD_GPU_EINVAL;
    }
    std::vector<float4> h((size_t)b->pool_f4);
    const double *s = emom;
    for (const MBRep &R : b->reps) {
        const long long n = 4 * R.nhalf;
        for (long long i = 0; i < n; ++i) {
            const double nx = s[3 * i], ny = s[3 * i + 1], nz = s[3 * i + 2];
            const double l = sqrt(nx * nx + ny * ny + nz * nz);
            if (!(l > 0.5 && l < 2.0)) {
                set_error("mcbatch_put_spins: spins must be (near) unit vectors");
                return UPPASD_GPU_EINVAL;
            }
            const int bb = (int)(i & 1);
            const long long cell = i >> 1;
            const int x = (int)(cell % R.L), y = (int)((cell / R.L) % R.L), z = (int)(cell / ((long long)R.L * R.L));
            const int par = (x + y + z) & 1;
            h[(size_t)(R.off + (2 * bb + par) * R.nhalf + ((long long)z * R.L + y) * R.Lh + x / 2)] =
                make_float4((float)(nx / l), (float)(ny / l), (float)(nz / l), 0.f);
        }
        s += 3 * n;
    }
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e == cudaSuccess) e = cudaMemcpy(b->p.pool, h.data(), h.size() * sizeof(float4), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail("mcbatch_put_spins", e);
    return UPPASD_GPU_OK;
}

int uppasd_gpu_mcbatch_set_sweep(uppasd_gpu_mcbatch *b, int64_t sweep) {
    if (!b || sweep < 0) {
        set_error("mcbatch_set_sweep: bad arguments");
        return UPPASD_GPU_EINVAL;
    }
    long long v = sweep;
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e == cudaSuccess) e = cudaMemcpy(b->p.sweep_ctr, &v, sizeof(long long), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail("mcbatch_set_sweep", e);
    return UPPASD_GPU_OK;
}

// Replica exchange after every launch (every sweeps_per_launch sweeps) between
// temperatures adjacent in T among the replicas of one size L.
int uppasd_gpu_mcbatch_set_exchange(uppasd_gpu_mcbatch *b, int32_t enable) {
    if (!b) {
        set_error("mcbatch_set_exchange: null handle");
        return UPPASD_GPU_EINVAL;
    }
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_fail("mcbatch_set_exchange", e);
    if (enable && !b->pairs_d) {
        // ladders: per size, slots sorted by temperature; even pairs first, then odd pairs
        std::vector<int> order(b->reps.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
        std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
            return b->reps[a].L != b->reps[c].L ? b->reps[a].L < b->reps[c].L
                                                 : b->temperature[a] < b->temperature[c];
        });
        std::vector<int2> even, odd;
        for (size_t i = 0; i + 1 < order.size(); ++i) {
            if (b->reps[order[i]].L != b->reps[order[i + 1]].L) continue;
            // position within the ladder decides the parity
            size_t start = i;
            while (start > 0 && b->reps[order[start - 1]].L == b->reps[order[i]].L) --start;
            ((i - start) % 2 == 0 ? even : odd).push_back(make_int2(order[i], order[i + 1]));
        }
        b->pairs_h = even;
        b->pairs_h.insert(b->pairs_h.end(), odd.begin(), odd.end());
        if (b->pairs_h.empty()) {
            set_error("mcbatch_set_exchange: no two replicas share a size");
            return UPPASD_GPU_EINVAL;
        }
        const size_t np = b->pairs_h.size();
        e = cudaMalloc(&b->pairs_d, np * sizeof(int2));
        if (e == cudaSuccess) e = cudaMemcpy(b->pairs_d, b->pairs_h.data(), np * sizeof(int2), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMalloc(&b->pt_att_d, np * sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMemset(b->pt_att_d, 0, np * sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMalloc(&b->pt_acc_d, np * sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMemset(b->pt_acc_d, 0, np * sizeof(unsigned long long));
        if (e != cudaSuccess) return cuda_fail("mcbatch_set_exchange", e);
        b->p.pairs = b->pairs_d;
        b->p.npair[0] = (int)even.size();
        b->p.npair[1] = (int)odd.size();
        b->p.pt_att = b->pt_att_d;
        b->p.pt_acc = b->pt_acc_d;
    }
    b->exchange = enable != 0;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return UPPASD_GPU_OK;
}

// slot_of_rep (nrep): the temperature slot each replica holds; pairs (npairs x 2)
// of slots, attempts and accepts (npairs), any may be NULL; *npairs always set.
int uppasd_gpu_mcbatch_exchange_state(uppasd_gpu_mcbatch *b, int32_t *slot_of_rep, int32_t *npairs,
                                      int32_t *pairs, int64_t *attempts, int64_t *accepts) {
    if (!b || !npairs) {
        set_error("mcbatch_exchange_state: null argument");
        return UPPASD_GPU_EINVAL;
    }
    cudaError_t e = cudaStreamSynchronize(b->stream);
    std::vector<MBRep> reps(b->reps.size());
    if (e == cudaSuccess) e = cudaMemcpy(reps.data(), b->reps_d, reps.size() * sizeof(MBRep), cudaMemcpyDeviceToHost);
    const size_t np = b->pairs_h.size();
    if (e == cudaSuccess && np && attempts)
        e = cudaMemcpy(attempts, b->pt_att_d, np * sizeof(int64_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && np && accepts)
        e = cudaMemcpy(accepts, b->pt_acc_d, np * sizeof(int64_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail("mcbatch_exchange_state", e);
    *npairs = (int32_t)np;
    if (slot_of_rep)
        for (size_t i = 0; i < reps.size(); ++i) slot_of_rep[i] = reps[i].slot;
    if (pairs)
        for (size_t q = 0; q < np; ++q) {
            pairs[2 * q] = b->pairs_h[q].x;
            pairs[2 * q + 1] = b->pairs_h[q].y;
        }
    return UPPASD_GPU_OK;
}

int uppasd_gpu_mcbatch_set_replica_ids(uppasd_gpu_mcbatch *b, int32_t first_id) {
    if (!b || first_id < 0) {
        set_error("mcbatch_set_replica_ids: null handle or negative id");
        return UPPASD_GPU_EINVAL;
    }
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_fail("mcbatch_set_replica_ids", e);
    b->p.rep_id0 = first_id;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return draw_initial_state(b);
}

int uppasd_gpu_mcbatch_set_spin_limit(uppasd_gpu_mcbatch *b, int64_t limit) {
    if (!b || limit < 0) {
        set_error("mcbatch_set_spin_limit: null handle or negative limit");
        return UPPASD_GPU_EINVAL;
    }
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_fail("mcbatch_set_spin_limit", e);
    b->p.spin_limit = limit ? (long long)limit : kDefaultSpinLimit;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return UPPASD_GPU_OK;
}

int uppasd_gpu_mcbatch_destroy(uppasd_gpu_mcbatch *b) {
    if (!b) {
        set_error("mcbatch_destroy: null handle");
        return UPPASD_GPU_EINVAL;
    }
    mb_free(b);
    return UPPASD_GPU_OK;
}

}  // extern "C"
