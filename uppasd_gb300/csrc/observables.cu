// observables.cu -- per-ensemble reductions of the spin state on the device.
//
//   total moment and |M|/natom   Measurement/measurements.f90:211-235,
//                                Measurement/prn_averages.f90:114-119
//   energy per atom (mRy)        Hamiltonian/energy.f90:60-405: exchange and DM
//                                with factor 1/2, anisotropy with 1/2 of its field,
//                                Zeeman with factor 1 (update_ene, :559-571)
// Block partial sums use warp shuffles; one atomicAdd per block and quantity.
#include "common.cuh"
#include "field_fp64.cuh"
#include "sim.h"

namespace uppasd {

enum { kRedMx = 0, kRedMy, kRedMz, kRedXc, kRedDm, kRedAni, kRedExt, kRedDip, kRedCount = 8 };

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(256) obs_kernel(HamDev h, Vec3D m, double *red) {
    const int N = h.natom;
    const int k = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t off = (size_t)k * N;
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (i < N) {
        double mi[3] = {m.x[off + i], m.y[off + i], m.z[off + i]};
        v[0] = mi[0];
        v[1] = mi[1];
        v[2] = mi[2];
        const int ih = h.aham[i];
        double bx[3] = {0.0, 0.0, 0.0};
        if (h.do_jtensor) {
            tensor_exchange(h, m, i, ih, off, bx);  // the pair energy, energy.f90:244-247
        } else {
            for (int s = 0; s < h.nsize[i]; ++s) {
                int j = h.nlist[(size_t)s * N + i];
                double c = h.ncoup[(size_t)s * h.nham + ih];
                bx[0] = bx[0] + c * m.x[off + j];
                bx[1] = bx[1] + c * m.y[off + j];
                bx[2] = bx[2] + c * m.z[off + j];
            }
        }
        v[3] = -0.5 * (mi[0] * bx[0] + mi[1] * bx[1] + mi[2] * bx[2]);
        // with the tensor the reference evaluates no separate DM energy (energy.f90:219-247, :371-379)
        if (h.do_dm && !h.do_jtensor) {
            double bd[3] = {0.0, 0.0, 0.0};
            for (int s = 0; s < h.dmsize[i]; ++s) {
                int j = h.dmlist[(size_t)s * N + i];
                size_t d = (size_t)s * h.nham + ih;
                double m1 = m.x[off + j], m2 = m.y[off + j], m3 = m.z[off + j];
                bd[0] = bd[0] + h.dmz[d] * m2 - h.dmy[d] * m3;
                bd[1] = bd[1] + h.dmx[d] * m3 - h.dmz[d] * m1;
                bd[2] = bd[2] + h.dmy[d] * m1 - h.dmx[d] * m2;
            }
            v[4] = -0.5 * (mi[0] * bd[0] + mi[1] * bd[1] + mi[2] * bd[2]);
        }
        if (h.do_aniso) {
            double bs[3] = {0.0, 0.0, 0.0}, bq[3] = {0.0, 0.0, 0.0};
            aniso_field(h, i, mi[0], mi[1], mi[2], bs, bq);
            double ta[3] = {bs[0] + bq[0], bs[1] + bq[1], bs[2] + bq[2]};
            v[5] = -0.5 * (mi[0] * ta[0] + mi[1] * ta[1] + mi[2] * ta[2]);
        }
        double be[3] = {0.0 + h.ext.x[off + i], 0.0 + h.ext.y[off + i], 0.0 + h.ext.z[off + i]};
        v[6] = -1.0 * (mi[0] * be[0] + mi[1] * be[1] + mi[2] * be[2]);
        // dipolar energy with the field evaluated for m (energy.f90:286-291)
        if (h.do_dip) v[7] = -0.5 * (mi[0] * h.dip.x[off + i] + mi[1] * h.dip.y[off + i] + mi[2] * h.dip.z[off + i]);
    }
    __shared__ double part[8][8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        double w = warp_sum(v[q]);
        if (lane == 0) part[wid][q] = w;
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            double w = lane < nw ? part[lane][q] : 0.0;
            w = warp_sum(w);
            if (lane == 0) atomicAdd(&red[k * kRedCount + q], w);
        }
    }
}

int observables(Sim &s, double *mvec_h, double *mabs_h, double *energy_h, const Vec3D *src, double *terms_h) {
    const int N = s.ham.natom, M = s.ham.mensemble;
    const Vec3D &m = src ? *src : s.eM;
    if (s.ham.do_dip) {
        int rc = dipole_field(s, m);
        if (rc) return rc;
    }
    UPPASD_CUDA_TRY(cudaMemsetAsync(s.red, 0, sizeof(double) * kRedCount * M, s.stream));
    dim3 grid((N + 255) / 256, M);
    obs_kernel<<<grid, 256, 0, s.stream>>>(s.ham, m, s.red);
    UPPASD_CUDA_TRY(cudaGetLastError());
    double *h = new double[(size_t)kRedCount * M];
    cudaError_t err = cudaMemcpyAsync(h, s.red, sizeof(double) * kRedCount * M, cudaMemcpyDeviceToHost, s.stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s.stream);
    if (err != cudaSuccess) {
        delete[] h;
        set_error(std::string("observables: ") + cudaGetErrorString(err));
        return UPPASD_GPU_ECUDA;
    }
    const double fcinv = s.ham.mub / s.ham.mry;
    for (int k = 0; k < M; ++k) {
        const double *r = h + (size_t)k * kRedCount;
        if (mvec_h) {
            mvec_h[3 * k] = r[kRedMx];
            mvec_h[3 * k + 1] = r[kRedMy];
            mvec_h[3 * k + 2] = r[kRedMz];
        }
        if (mabs_h) mabs_h[k] = sqrt(r[kRedMx] * r[kRedMx] + r[kRedMy] * r[kRedMy] + r[kRedMz] * r[kRedMz]) / N;
        double xc = r[kRedXc] / N, dm = r[kRedDm] / N, an = r[kRedAni] / N, ex = r[kRedExt] / N;
        const double dp = r[kRedDip] / N;
        if (energy_h) energy_h[k] = (xc + dm + ex + an + dp) * fcinv;
        if (terms_h) {
            double *t = terms_h + 5 * (size_t)k;
            t[0] = (xc + dm + ex + an + dp) * fcinv;
            t[1] = xc * fcinv;
            t[2] = an * fcinv;
            t[3] = dm * fcinv;
            t[4] = ex * fcinv;
        }
    }
    delete[] h;
    return UPPASD_GPU_OK;
}

__global__ void __launch_bounds__(256) field_kernel(HamDev h, Vec3D m, double *beff) {
    const int N = h.natom;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)N * h.mensemble) return;
    const int k = (int)(t / N), i = (int)(t - (int64_t)k * N);
    double B[3];
    site_field(h, m, i, k, B);
    size_t o = 3 * ((size_t)i + (size_t)N * k);
    beff[o] = B[0];
    beff[o + 1] = B[1];
    beff[o + 2] = B[2];
}

int field_to_host(Sim &s, double *beff_h) {
    const size_t n = (size_t)s.ham.natom * s.ham.mensemble;
    double *d = stage_buffer(s);
    if (!d) return UPPASD_GPU_ENOMEM;
    if (s.ham.do_dip) {
        int rc = dipole_field(s, s.eM);
        if (rc) return rc;
    }
    field_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s.stream>>>(s.ham, s.eM, d);
    cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaMemcpyAsync(beff_h, d, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, s.stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s.stream);
    if (err != cudaSuccess) {
        set_error(std::string("field_to_host: ") + cudaGetErrorString(err));
        return UPPASD_GPU_ECUDA;
    }
    return UPPASD_GPU_OK;
}

}  // namespace uppasd
