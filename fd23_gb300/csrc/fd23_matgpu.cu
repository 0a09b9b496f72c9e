// Material builder on the GPU (FP32 and FP64 storage): the arithmetic of the
// host builders in fd23_host.cpp (PD/material/material.cpp:101-311 for P-SV,
// SH/material/material.cpp:68-172 for SH), cell by cell in FP64 with the
// same operation order and no contraction, so the stored material is bit for
// bit the host builder's rounded to the storage type.  fd23_set_model uses
// it so that a shot's set-up uploads vp, vs, density once instead of
// building five arrays on one host core.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "fd23_device.cuh"
#include "fd23_solver.h"

namespace fd23 {

namespace {

__device__ __forceinline__ double dmax(double a, double b) { return a < b ? b : a; }  // std::max(a, b)

// pass 1: MU and LAM with the fluid rule of the 5-cell band at the left,
// right and bottom edges (PD/material/material.cpp:166-200)
__global__ void psv_mu_lam(int nx, int nz, const double *vp, const double *vs, const double *den, double *mu,
                           double *lam)
{
    const long long n = (long long)nx * nz;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(k / nx), ix = (int)(k % nx);
        double m = vs[k] * vs[k] * den[k];
        double l = vp[k] * vp[k] * den[k] - 2.0 * m;
        const int band = 5;
        const bool edge = ix < band || ix >= nx - band || iz >= nz - band;
        if (edge && vs[k] / vp[k] < 0.01) {
            m = vp[k] * vp[k] / 3.0 * den[k];
            l = vp[k] * vp[k] * den[k] - 2.0 * m;
        }
        mu[k] = m;
        lam[k] = l;
    }
}

template <class S>
__device__ __forceinline__ S store(double v)
{
    return (S)v;
}

// pass 2: BU, BW, MUA (harmonic average of the 4 MU around the node), the
// free-surface row, the dt/h factor; written to the padded storage arrays
template <class S>
__global__ void psv_rest(int nx, int nz, const double *den, const double *mu, const double *lam, double fac,
                         long long origin, int pitch, S *LAM, S *MU, S *MUA, S *BU, S *BW)
{
    const long long n = (long long)nx * nz;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(k / nx), ix = (int)(k % nx);
        double l = lam[k], m = mu[k], bu = 0.0, bw = 0.0, mua = 0.0;
        if (iz >= 1) {
            const long long kr = (k + 1 < n) ? k + 1 : k;
            bu = 2.0 / (den[k] + den[kr]);
            const long long kb = (k + nx < n) ? k - nx : k;
            bw = 2.0 / (den[k] + den[kb]);
            if (ix + 1 < nx && iz + 1 < nz) {
                const double m1 = mu[k], m2 = mu[k + 1], m3 = mu[k - nx], m4 = mu[k + 1 - nx];
                const double d = dmax(m2 * m3 * m4 + m1 * m3 * m4 + m1 * m2 * m4 + m2 * m3 * m4, 1e-10);
                mua = 4.0 * m1 * m2 * m3 * m4 / d;
            } else {
                mua = mu[k];
            }
        } else if (ix >= 1 && ix < nx - 1) {
            bu = 4.0 / (den[ix] + den[ix + 1]);
            l = 0.0;
            m = 0.5 * m;
        }
        const long long o = origin + (long long)iz * pitch + ix;
        LAM[o] = store<S>(l * fac);
        MU[o] = store<S>(m * fac);
        MUA[o] = store<S>(mua * fac);
        BU[o] = store<S>(bu * fac);
        BW[o] = store<S>(bw * fac);
    }
}

// SH: MUX, MUZ (harmonic means with the next cell and the cell above), BV
template <class S>
__global__ void sh_all(int nx, int nz, const double *vs, const double *den, double fac, long long origin, int pitch,
                       S *MUX, S *MUZ, S *BV)
{
    const long long n = (long long)nx * nz;
    auto shear = [&](long long k) { return vs[k] * vs[k] * den[k]; };
    auto harm = [](double a, double b) { return 2.0 * a * b / dmax(a + b, 1e-10); };
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(k / nx), ix = (int)(k % nx);
        const double m1 = shear(k);
        const double mux = harm(m1, (k + 1 < n) ? shear(k + 1) : m1);
        const double muz = harm(m1, (k - nx >= 0) ? shear(k - nx) : m1);
        const double bv = 1.0 / den[k];
        const long long o = origin + (long long)iz * pitch + ix;
        MUX[o] = store<S>(mux * fac);
        MUZ[o] = store<S>(muz * fac);
        BV[o] = store<S>(bv * fac);
    }
}

template <class S>
int build_on_device(fd23_solver *s, const double *vp, const double *vs, const double *den)
{
    const int nx = s->d.nx, nz = s->d.nz;
    const size_t n = (size_t)nx * nz, bytes = n * sizeof(double);
    const int nin = s->d.wave == FD23_PSV ? 3 : 2;
    double *buf = nullptr;  // inputs, then MU and LAM (P-SV)
    int rc = dev_alloc((void **)&buf, (nin + 2) * bytes);
    if (rc) return rc;
    double *dvp = buf, *dvs = buf + (nin == 3 ? n : 0), *dden = buf + (nin - 1) * n;
    double *dmu = buf + nin * n, *dlam = dmu + n;
    cudaError_t e = cudaSuccess;
    if (nin == 3) e = cudaMemcpyAsync(dvp, vp, bytes, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dvs, vs, bytes, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dden, den, bytes, cudaMemcpyHostToDevice, s->stream);
    const double fac = s->d.dt / s->d.h;  // as the host builders: dt / h, then value * fac
    const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 32);
    if (e == cudaSuccess) {
        S *const *mm = reinterpret_cast<S *const *>(s->mat);
        if (s->d.wave == FD23_PSV) {
            psv_mu_lam<<<blocks, 256, 0, s->stream>>>(nx, nz, dvp, dvs, dden, dmu, dlam);
            psv_rest<S><<<blocks, 256, 0, s->stream>>>(nx, nz, dden, dmu, dlam, fac, s->L.origin, s->L.pitch, mm[0],
                                                       mm[1], mm[2], mm[3], mm[4]);
        } else {
            sh_all<S><<<blocks, 256, 0, s->stream>>>(nx, nz, dvs, dden, fac, s->L.origin, s->L.pitch, mm[0], mm[1],
                                                     mm[2]);
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(buf);
    return e == cudaSuccess ? FD23_OK : FD23_ERR_CUDA;
}

}  // namespace

int build_material_device(fd23_solver *s, const double *vp, const double *vs, const double *den)
{
    if (s->d.prec == FD23_F64) return build_on_device<double>(s, vp, vs, den);
    if (s->d.prec == FD23_F32) return build_on_device<float>(s, vp, vs, den);
    return FD23_ERR_UNSUPPORTED;  // the 16-bit forms scale their material first (host path)
}

}  // namespace fd23
