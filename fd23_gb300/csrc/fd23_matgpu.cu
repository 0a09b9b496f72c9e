// Material builder on the GPU (FP32 and FP64 storage): the arithmetic of the
// host builders in fd23_host.cpp (PD/material/material.cpp:101-311 for P-SV,
// SH/material/material.cpp:68-172 for SH), cell by cell in FP64 with the
// same operation order and no contraction, so the stored material is bit for
// bit the host builder's rounded to the storage type.  fd23_set_model uses
// it so that a shot's set-up uploads vp, vs, density once instead of
// building five arrays on one host core.  The 16-bit forms add their
// power-of-two scale kappa (chosen from the maxima of the two material
// groups, the first time) and the host conversion's rounding: the scaled
// double to float, then to 16 bits, each to nearest even.
#include <cmath>
#include <cstring>
#include <type_traits>

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

// What the material kernels do with each dt/h-scaled value x of array m
// (the first nms arrays feed the stress update, the rest the velocity update):
//   kStore:  storage element (S)x, FP32 / FP64 storage;
//   kMax:    the largest |x| of each group, for the 16-bit forms' power-of-two
//            scale kappa (fd23_set_material's choice);
//   kScaled: 16-bit storage element of x * f (f = kappa or 1/kappa, exact),
//            rounded to float and then to 16 bits, as the host conversion does.
enum { kStore = 0, kMax = 1, kScaled = 2 };

template <class S>
__device__ __forceinline__ S store(double v)
{
    return (S)v;
}
template <>
__device__ __forceinline__ __half store<__half>(double v)
{
    return __float2half_rn((float)v);
}
template <>
__device__ __forceinline__ __nv_bfloat16 store<__nv_bfloat16>(double v)
{
    return __float2bfloat16_rn((float)v);
}

struct MatOut {
    long long origin;
    int pitch;
    double fs, fv;                 // kScaled factors of the stress / velocity group
    unsigned long long *maxbits;   // kMax: [2] bit patterns of the group maxima
};

// Hybrid-box homogenisation applied while the material is stored (P-SV,
// kStore): the cells of the box whose dt/h-scaled coefficients differ from
// the source material's by more than 1e-4 (relative) take the source
// material, and every box cell's final values go to bmat ([5][bz][bx],
// FP64), as box_material does on the host (PD/material/material.cpp:39-97).
struct BoxHomog {
    int on, x0, z0, bx, bz;
    double lam, mu, b;     // source material, dt/h scaled
    double *bmat;
    int *replaced;
};

template <class S, int MODE>
struct MatSink {
    const MatOut &o;
    double ms = 0.0, mv = 0.0;
    __device__ MatSink(const MatOut &out) : o(out) {}
    __device__ __forceinline__ void put(S *a, long long k, int nx, bool stress, double x)
    {
        if constexpr (MODE == kMax) {
            const double ax = fabs(x);
            if (stress) ms = ax > ms ? ax : ms;
            else mv = ax > mv ? ax : mv;
        } else {
            const int iz = (int)(k / nx), ix = (int)(k % nx);
            const long long i = o.origin + (long long)iz * o.pitch + ix;
            a[i] = MODE == kScaled ? store<S>(x * (stress ? o.fs : o.fv)) : store<S>(x);
        }
    }
    // block-wide maxima into maxbits (non-negative doubles order as their bits)
    __device__ __forceinline__ void finish()
    {
        if constexpr (MODE == kMax) {
            __shared__ double red[2][32];
            double a = ms, b = mv;
            for (int d = 16; d > 0; d >>= 1) {
                a = fmax(a, __shfl_xor_sync(0xffffffffu, a, d));
                b = fmax(b, __shfl_xor_sync(0xffffffffu, b, d));
            }
            const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
            if (lane == 0) {
                red[0][w] = a;
                red[1][w] = b;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                for (int i = 1; i < (int)(blockDim.x >> 5); ++i) {
                    a = fmax(a, red[0][i]);
                    b = fmax(b, red[1][i]);
                }
                atomicMax(o.maxbits, (unsigned long long)__double_as_longlong(a));
                atomicMax(o.maxbits + 1, (unsigned long long)__double_as_longlong(b));
            }
        }
    }
};

// pass 2: BU, BW, MUA (harmonic average of the 4 MU around the node), the
// free-surface row, the dt/h factor; written to the padded storage arrays
template <class S, int MODE = kStore>
__global__ void psv_rest(int nx, int nz, const double *den, const double *mu, const double *lam, double fac,
                         MatOut out, S *LAM, S *MU, S *MUA, S *BU, S *BW, BoxHomog hb)
{
    MatSink<S, MODE> sink(out);
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
        double v[5] = {l * fac, m * fac, mua * fac, bu * fac, bw * fac};
        if (hb.on && ix >= hb.x0 && ix < hb.x0 + hb.bx && iz >= hb.z0 && iz < hb.z0 + hb.bz) {
            const double eps = 1e-4;
            if (fabs(hb.b - v[3]) > hb.b * eps || fabs(hb.b - v[4]) > hb.b * eps || fabs(hb.mu - v[1]) > hb.mu * eps ||
                fabs(hb.mu - v[2]) > hb.mu * eps || fabs(hb.lam - v[0]) > hb.lam * eps) {
                v[0] = hb.lam;
                v[1] = v[2] = hb.mu;
                v[3] = v[4] = hb.b;
                atomicAdd(hb.replaced, 1);
            }
            const long long nb = (long long)hb.bx * hb.bz, q = (long long)(iz - hb.z0) * hb.bx + (ix - hb.x0);
#pragma unroll
            for (int f = 0; f < 5; ++f) hb.bmat[f * nb + q] = v[f];
        }
        sink.put(LAM, k, nx, true, v[0]);
        sink.put(MU, k, nx, true, v[1]);
        sink.put(MUA, k, nx, true, v[2]);
        sink.put(BU, k, nx, false, v[3]);
        sink.put(BW, k, nx, false, v[4]);
    }
    sink.finish();
}

// SH: MUX, MUZ (harmonic means with the next cell and the cell above), BV
template <class S, int MODE = kStore>
__global__ void sh_all(int nx, int nz, const double *vs, const double *den, double fac, MatOut out, S *MUX, S *MUZ,
                       S *BV)
{
    MatSink<S, MODE> sink(out);
    const long long n = (long long)nx * nz;
    auto shear = [&](long long k) { return vs[k] * vs[k] * den[k]; };
    auto harm = [](double a, double b) { return 2.0 * a * b / dmax(a + b, 1e-10); };
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const double m1 = shear(k);
        const double mux = harm(m1, (k + 1 < n) ? shear(k + 1) : m1);
        const double muz = harm(m1, (k - nx >= 0) ? shear(k - nx) : m1);
        const double bv = 1.0 / den[k];
        sink.put(MUX, k, nx, true, mux * fac);
        sink.put(MUZ, k, nx, true, muz * fac);
        sink.put(BV, k, nx, false, bv * fac);
    }
    sink.finish();
}

template <class S, bool SCALED>
int build_on_device(fd23_solver *s, const double *vp, const double *vs, const double *den, const BoxHomog &hb)
{
    const int nx = s->d.nx, nz = s->d.nz;
    const size_t n = (size_t)nx * nz, bytes = n * sizeof(double);
    const int nin = s->d.wave == FD23_PSV ? 3 : 2;
    double *buf = nullptr;  // inputs, then MU and LAM (P-SV)
    int rc = dev_alloc((void **)&buf, (nin + 2) * bytes + 2 * sizeof(unsigned long long));
    if (rc) return rc;
    double *dvp = buf, *dvs = buf + (nin == 3 ? n : 0), *dden = buf + (nin - 1) * n;
    double *dmu = buf + nin * n, *dlam = dmu + n;
    cudaError_t e = cudaSuccess;
    if (nin == 3) e = cudaMemcpyAsync(dvp, vp, bytes, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dvs, vs, bytes, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dden, den, bytes, cudaMemcpyHostToDevice, s->stream);
    const double fac = s->d.dt / s->d.h;  // as the host builders: dt / h, then value * fac
    const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 32);
    S *const *mm = reinterpret_cast<S *const *>(s->mat);
    MatOut out{s->L.origin, s->L.pitch, 1.0, 1.0, reinterpret_cast<unsigned long long *>(dmu)};
    auto launch = [&](auto mode) {
        constexpr int M = decltype(mode)::value;
        if (s->d.wave == FD23_PSV)
            psv_rest<S, M><<<blocks, 256, 0, s->stream>>>(nx, nz, dden, dmu, dlam, fac, out, mm[0], mm[1], mm[2],
                                                          mm[3], mm[4], M == kStore ? hb : BoxHomog{});
        else
            sh_all<S, M><<<blocks, 256, 0, s->stream>>>(nx, nz, dvs, dden, fac, out, mm[0], mm[1], mm[2]);
    };
    if (e == cudaSuccess && s->d.wave == FD23_PSV) {
        psv_mu_lam<<<blocks, 256, 0, s->stream>>>(nx, nz, dvp, dvs, dden, dmu, dlam);
        e = cudaGetLastError();
    }
    if constexpr (SCALED) {
        // kappa from the largest stress-update and velocity-update values, the
        // first time (fd23_set_material's rule); the maxima go to a scratch
        // pair after the inputs and MU, LAM
        unsigned long long *dmax = reinterpret_cast<unsigned long long *>(dlam + n);
        out.maxbits = dmax;
        if (e == cudaSuccess && !s->kappa_set) {
            e = cudaMemsetAsync(dmax, 0, 2 * sizeof(unsigned long long), s->stream);
            if (e == cudaSuccess) {
                launch(std::integral_constant<int, kMax>());
                e = cudaGetLastError();
            }
            unsigned long long hb[2] = {0, 0};
            if (e == cudaSuccess) e = cudaMemcpyAsync(hb, dmax, sizeof(hb), cudaMemcpyDeviceToHost, s->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
            if (e == cudaSuccess) {
                double ms, mv;
                std::memcpy(&ms, &hb[0], 8);
                std::memcpy(&mv, &hb[1], 8);
                s->kappa = (ms > 0 && mv > 0) ? pow2_round(std::sqrt(mv / ms)) : 1.0;
                s->kappa_set = true;
                const int rc = upload_source_amps(s);
                if (rc) {
                    cudaFree(buf);
                    return rc;
                }
            }
        }
        out.fs = s->kappa;
        out.fv = 1.0 / s->kappa;
        if (e == cudaSuccess) {
            launch(std::integral_constant<int, kScaled>());
            e = cudaGetLastError();
        }
    } else if (e == cudaSuccess) {
        launch(std::integral_constant<int, kStore>());
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(buf);
    return e == cudaSuccess ? FD23_OK : FD23_ERR_CUDA;
}

}  // namespace

int build_material_device(fd23_solver *s, const double *vp, const double *vs, const double *den)
{
    const BoxHomog none{};
    switch (s->d.prec) {
        case FD23_F64: return build_on_device<double, false>(s, vp, vs, den, none);
        case FD23_F32: return build_on_device<float, false>(s, vp, vs, den, none);
        case FD23_F16: return build_on_device<__half, true>(s, vp, vs, den, none);
        default: return build_on_device<__nv_bfloat16, true>(s, vp, vs, den, none);
    }
}

namespace {
template <class C>
__global__ void to_compute_kernel(long long n, const double *in, C *out)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        out[k] = (C)in[k];
}
}  // namespace

int build_material_box_device(fd23_solver *s, const double *vp, const double *vs, const double *den, int x0,
                              int z0, int bx, int bz, double src_vp, double src_vs, double src_den, int *replaced,
                              double *bmat_out)
{
    // the source material as the host's box_material computes it
    const double dt = s->d.dt, h = s->d.h;
    const double mu0 = src_vs * src_vs * src_den;
    BoxHomog hb{1, x0, z0, bx, bz, (src_vp * src_vp * src_den - 2.0 * mu0) * dt / h, mu0 * dt / h,
                1.0 / src_den * dt / h, nullptr, nullptr};
    const size_t nb = (size_t)bx * bz;
    void *scratch = nullptr;
    int rc = dev_alloc(&scratch, 5 * nb * sizeof(double) + sizeof(int));
    if (rc) return rc;
    hb.bmat = static_cast<double *>(scratch);
    hb.replaced = reinterpret_cast<int *>(hb.bmat + 5 * nb);
    cudaError_t e = cudaMemsetAsync(hb.replaced, 0, sizeof(int), s->stream);
    if (e == cudaSuccess) {
        rc = s->d.prec == FD23_F64 ? build_on_device<double, false>(s, vp, vs, den, hb)
                                   : build_on_device<float, false>(s, vp, vs, den, hb);
    } else {
        rc = FD23_ERR_CUDA;
    }
    // the box material in the compute type (the residual field's material)
    for (int m = 0; m < 5 && rc == FD23_OK; ++m) {
        const unsigned blocks = (unsigned)std::min<size_t>((nb + 255) / 256, 1024);
        if (s->d.prec == FD23_F64)
            to_compute_kernel<double><<<blocks, 256, 0, s->stream>>>((long long)nb, hb.bmat + m * nb,
                                                                     static_cast<double *>(s->box_mat[m]));
        else
            to_compute_kernel<float><<<blocks, 256, 0, s->stream>>>((long long)nb, hb.bmat + m * nb,
                                                                    static_cast<float *>(s->box_mat[m]));
        if (cudaGetLastError() != cudaSuccess) rc = FD23_ERR_CUDA;
    }
    int nrep = 0;
    if (rc == FD23_OK && bmat_out &&
        cudaMemcpyAsync(bmat_out, hb.bmat, 5 * nb * sizeof(double), cudaMemcpyDeviceToHost, s->stream) != cudaSuccess)
        rc = FD23_ERR_CUDA;
    if (rc == FD23_OK && (cudaMemcpyAsync(&nrep, hb.replaced, sizeof(int), cudaMemcpyDeviceToHost, s->stream) !=
                              cudaSuccess ||
                          cudaStreamSynchronize(s->stream) != cudaSuccess))
        rc = FD23_ERR_CUDA;
    cudaFree(scratch);
    if (rc == FD23_OK && replaced) *replaced = nrep;
    return rc;
}

}  // namespace fd23
