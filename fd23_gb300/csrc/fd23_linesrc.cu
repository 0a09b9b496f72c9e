// Box-source generator on the GPU: the reference's ntde_line program
// (PD/source/source_line.cpp:307-410) -- displacement planes of a line
// moment source in a homogeneous full space, the incident field of the
// hybrid box -- and its use as the box's incident field without a file.
//
// Three FP64 kernels:
//   line_points    one thread per plane point (component, cell): distance,
//                  arrival steps, integrated first samples and the five
//                  coefficients k[] of the closed form
//                    v(t) = t^3 (Ta - Tb) k0 + t (Ta k1 + Tb k2) + (Ta k3 + Tb k4) / t
//                  (the Mathematica expressions of compute_pQpW_mathematica,
//                  :196-305, gathered per power of t);
//   line_green     one thread per (point, sample) of a time window;
//   line_convolve  the causal convolution with the wavelet in the reference
//                  kernel's order (cu_con, PD/source/cu_source.cu:2-42: taps
//                  padded to a multiple of 32, last tap first, one fused
//                  multiply-add each), 32 points x 32 frames per CTA, turned
//                  through shared memory so that frames are written point-
//                  contiguous, the reference file's layout.
// The box path adds line_incident (BOX::setboxsource, PD/box/box.cpp:120-196,
// on the ring cells) and generates only the plane points the ring stencils
// read.  All arithmetic is the host builder's sequence (no contraction:
// -fmad=false), so planes and incident fields equal the host path's bit for
// bit.  The work is FP64 and bound by the FP64 pipe, which GB300 keeps small.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fd23_device.cuh"
#include "fd23_solver.h"

namespace fd23 {

namespace {

constexpr double kPiRef = 3.14159265358979;  // the reference's PI, PD/param/const.h:26
constexpr int kMaxTaps = 8192;
constexpr size_t kChunkBytes = size_t(1) << 30;  // device working set of one frame chunk
constexpr int kMaxChunkFrames = 8192;            // also bounds the incident grid's y extent

struct LinePoint {
    double R, k[5];
    double ua, ub;  // R/vp/dt, R/vs/dt
    double fa, fb;  // integrated first samples
    int na, nb;     // arrival steps floor(ua), floor(ub)
};

struct LineGeom {
    int px, pz, ox, oz;
    double h, dt, vp, vs, den, a0, a1, a2, sx, sz;
};

// k[] of one point (r, z metres from the source, z down), component 0 = U,
// 1 = W.  Rows: the three radiation terms; columns: t^3 (Ta - Tb), t Ta,
// t Tb, Ta / t, Tb / t.
__device__ void line_kcoef(double r, double z, int comp, const LineGeom &g, double *k)
{
    const double r2 = r * r, z2 = z * z, rz = r * z;
    const double r4 = r2 * r2, z4 = z2 * z2, r6 = r4 * r2, z6 = z4 * z2, z8 = z4 * z4;
    const double R2 = r2 + z2, R4 = R2 * R2;
    const double dif = r2 - z2;
    const double e4 = r4 - 6.0 * r2 * z2 + z4;
    const double e6 = r6 - 5.0 * r4 * z2 - 5.0 * r2 * z4 + z6;
    const double f4 = 3.0 * r4 - 2.0 * r2 * z2 - 5.0 * z4;
    double p[3][5];
    if (comp == 0) {
        p[0][0] = e4;
        p[0][1] = 2.0 * (3.0 * r4 * z2 + 2.0 * r2 * z4 - z6);
        p[0][2] = e6;
        p[0][3] = R4 * z4;
        p[0][4] = r2 * R4 * z2;
        p[1][0] = -8.0 * rz * dif;
        p[1][1] = 2.0 * rz * f4;
        p[1][2] = 8.0 * rz * (z4 - r4);
        p[1][3] = 2.0 * rz * R4 * z2;
        p[1][4] = rz * R4 * dif;
        p[2][0] = -3.0 * e4;
        p[2][1] = 2.0 * (r6 - 8.0 * r4 * z2 - 7.0 * r2 * z4 + 2.0 * z6);
        p[2][2] = -3.0 * e6;
        p[2][3] = 2.0 * r6 * z2 + 3.0 * r4 * z4 - z8;
        p[2][4] = -3.0 * r2 * R4 * z2;
    } else {
        p[0][0] = 4.0 * rz * dif;
        p[0][1] = -rz * f4;
        p[0][2] = rz * f4;
        p[0][3] = -rz * R4 * z2;
        p[0][4] = rz * R4 * z2;
        p[1][0] = 2.0 * e4;
        p[1][1] = -2.0 * e6;
        p[1][2] = r6 - 11.0 * r4 * z2 - 9.0 * r2 * z4 + 3.0 * z6;
        p[1][3] = -2.0 * r2 * R4 * z2;
        p[1][4] = R4 * dif * z2;
        p[2][0] = -12.0 * rz * dif;
        p[2][1] = rz * (13.0 * r4 + 2.0 * r2 * z2 - 11.0 * z4);
        p[2][2] = -3.0 * rz * f4;
        p[2][3] = rz * (z6 - 2.0 * r6 - 3.0 * r4 * z2);
        p[2][4] = -3.0 * rz * R4 * z2;
    }
    const double ivp2 = 1.0 / (g.vp * g.vp), ivs2 = 1.0 / (g.vs * g.vs);
    const double G = sqrt(2.0) / (4.0 * kPiRef * kPiRef * g.den);
    const double S = G / (R4 * R4);
    const double w[5] = {S, S * ivp2, S * ivs2, S * (ivp2 * ivp2), S * (ivs2 * ivs2)};
    for (int j = 0; j < 5; j++) k[j] = (g.a0 * p[0][j] + g.a1 * p[1][j] + g.a2 * p[2][j]) * w[j];
}

// point index pt = comp * px * pz + q * px + p (list == nullptr), or the
// pt of entry i of the list
__global__ void line_points(LineGeom g, const int *list, int npts, LinePoint *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npts) return;
    const int plane = g.px * g.pz;
    const int pt = list ? list[i] : i;
    const int comp = pt / plane, c = pt - comp * plane;
    const int p = c % g.px, q = c / g.px;
    const double x = comp == 0 ? ((g.ox + p) + 0.5) - g.sx : (g.ox + p) - g.sx;
    const double zz = comp == 0 ? (g.oz + q) - g.sz : ((g.oz + q) - 0.5) - g.sz;
    const double r = x * g.h, z = zz * g.h;
    LinePoint o;
    line_kcoef(r, z, comp, g, o.k);
    o.R = sqrt(r * r + z * z);
    o.ua = o.R / g.vp / g.dt;
    o.ub = o.R / g.vs / g.dt;
    o.na = (int)floor(o.ua);
    o.nb = (int)floor(o.ub);
    const double ba = ((double)(o.na + 1) - o.ua) + 0.5, bb = ((double)(o.nb + 1) - o.ub) + 0.5;
    o.fa = sqrt(ba * (2.0 * o.ua + ba));
    o.fb = sqrt(bb * (2.0 * o.ub + bb));
    out[i] = o;
}

// wave factor at sample i: 0 up to the arrival step n, the integrated
// first sample at n + 1, then 1/sqrt(1 - (R/(t v))^2)
__device__ __forceinline__ double line_wave(double R, double v, double t, int i, int n, double first)
{
    if (i <= n) return 0.0;
    if (i == n + 1) return first;
    const double q = R / (t * v);
    return 1.0 / sqrt(1.0 - q * q);
}

// g[pt][w] = v at sample i0 + w (0 for i < 0 and before the P arrival step)
__global__ void line_green(LineGeom g, const LinePoint *pts, int npts, int i0, int nw, double *out)
{
    const long long n = (long long)npts * nw;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int pi = (int)(e / nw), w = (int)(e - (long long)pi * nw);
        const int i = i0 + w;
        const LinePoint &P = pts[pi];
        double v = 0.0;
        if (i >= 0 && i >= P.na) {
            const double t = i * g.dt;
            const double ta = line_wave(P.R, g.vp, t, i, P.na, P.fa);
            const double tb = line_wave(P.R, g.vs, t, i, P.nb, P.fb);
            const double t3 = (t * t) * t;
            v = (t3 * (ta - tb)) * P.k[0];
            v = v + t * (ta * P.k[1] + tb * P.k[2]);
            v = v + (ta * P.k[3] + tb * P.k[4]) / t;
        }
        out[e] = v;
    }
}

// frames[f][pt] = sum over taps j = ntap-1 .. 0 of fma(tap[j], g[pt][f + ntap-1 - j])
// (g rows hold samples from frame 0 - (ntap-1)); 256 threads: warp w holds
// points pt0 + w + 8m (m < 4), lane = frame f0 + lane
constexpr int kConvPts = 32, kConvFrames = 32;
__global__ void __launch_bounds__(256) line_convolve(const double *g, int npts, int nw, const double *tap, int ntap,
                                                     int nf, double *frames)
{
    __shared__ double tile[kConvPts][kConvFrames + 1];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int pt0 = blockIdx.x * kConvPts, f0 = blockIdx.y * kConvFrames;
    const int f = f0 + lane;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const double *row[4];
    bool live[4];
    for (int m = 0; m < 4; m++) {
        const int pt = pt0 + wp + 8 * m;
        live[m] = pt < npts && f < nf;
        row[m] = g + (size_t)(pt < npts ? pt : 0) * nw + (f < nf ? f : 0) + (ntap - 1);
    }
    for (int j = ntap - 1; j >= 0; j--) {
        const double c = __ldg(tap + j);
        for (int m = 0; m < 4; m++)
            if (live[m]) acc[m] = fma(c, __ldg(row[m] - j), acc[m]);
    }
    for (int m = 0; m < 4; m++) tile[wp + 8 * m][lane] = acc[m];
    __syncthreads();
    for (int m = 0; m < 4; m++) {
        const int fr = f0 + wp + 8 * m, pt = pt0 + lane;
        if (fr < nf && pt < npts) frames[(size_t)fr * npts + pt] = tile[lane][wp + 8 * m];
    }
}

// BOX::setboxsource on the ring cells: steps s of the chunk read frames s
// (old) and s + 1 (new); slot[comp][q][p] = the point of plane cell (p, q)
// in the frames (every stencil cell has one by construction; -1 elsewhere)
template <class C>
__global__ void line_incident(int bx, int bz, const int2 *cells, int nring, const double *rlam, const double *rmu,
                              const double *rmua, const int *slot, const double *frames, int npts, int nsteps,
                              double dt, C *inc, int *err)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (q >= nring || s >= nsteps) return;
    const int pw = bx + 8, plane = pw * (bz + 8);
    const int tx = cells[q].x + 4, ty = cells[q].y + 4;
    const double *fo = frames + (size_t)s * npts, *fn = fo + npts;
    bool bad = false;
    auto at = [&](const double *fr, int comp, int i, int j) {
        const int sl = slot[comp * plane + j * pw + i];
        if (sl < 0) {
            bad = true;
            return 0.0;
        }
        return fr[sl];
    };
    const int oz = abs(ty - 3 - (bz + 1) / 2) - 1, ox = abs(tx - 3 - (bx + 1) / 2) - 1;
    const int ord = max(0, min(4, max(oz, ox)));
    const double c0 = kCoefD[ord][0], c1 = kCoefD[ord][1], c2 = kCoefD[ord][2], c3 = kCoefD[ord][3];
    auto diff = [&](int comp, int di, int dj, int p) {
        auto d = [&](int k) {
            return at(fn, comp, tx + (k + p) * di, ty + (k + p) * dj) -
                   at(fn, comp, tx - (k + 1 - p) * di, ty - (k + 1 - p) * dj);
        };
        return c0 * d(0) - c1 * d(1) + c2 * d(2) - c3 * d(3);
    };
    const double ux = diff(0, 1, 0, 0), uz = diff(0, 0, 1, 0);
    const double wx = diff(1, 1, 0, 1), wz = diff(1, 0, 1, 1);
    const double lam = rlam[q], mu = rmu[q], mua = rmua[q];
    const double gam = lam + 2.0 * mu;
    const double U = (at(fn, 0, tx, ty) - at(fo, 0, tx, ty)) / dt;
    const double W = (at(fn, 1, tx, ty) - at(fo, 1, tx, ty)) / dt;
    C *o = inc + (size_t)s * 5 * nring;
    o[q] = (C)U;
    o[(size_t)nring + q] = (C)W;
    o[2 * (size_t)nring + q] = (C)((gam * ux + lam * wz) / dt);
    o[3 * (size_t)nring + q] = (C)((mua * (wx + uz)) / dt);
    o[4 * (size_t)nring + q] = (C)((lam * ux + gam * wz) / dt);
    if (bad) atomicExch(err, 1);
}

LineGeom geom_of(const fd23_line_desc *d)
{
    LineGeom g;
    g.px = d->px;
    g.pz = d->pz;
    g.ox = d->ox;
    g.oz = d->oz;
    g.h = d->h;
    g.dt = d->dt;
    g.vp = d->vp;
    g.vs = d->vs;
    g.den = d->den;
    g.a0 = d->a[0];
    g.a1 = d->a[1];
    g.a2 = d->a[2];
    g.sx = d->sx;
    g.sz = d->sz;
    return g;
}

bool desc_ok(const fd23_line_desc *d, const double *src, int lsrc)
{
    return d && src && lsrc >= 1 && lsrc <= kMaxTaps && d->px > 0 && d->pz > 0 &&
           (long long)d->px * d->pz <= (1 << 28) && d->h > 0 && d->dt > 0 && d->vp > 0 && d->vs > 0 && d->den > 0 &&
           std::isfinite(d->sx) && std::isfinite(d->sz);
}

int ntaps(int lsrc) { return ((lsrc + 31) / 32) * 32; }

// Frames [f0, f0 + nf) of the points into dframes (device, [nf][npts]);
// scratch: pts (npts), g (npts * (nf + ntap - 1)), dtap (ntap).
int frames_chunk(const LineGeom &g, const LinePoint *pts, int npts, const double *dtap, int ntap, int f0, int nf,
                 double *dg, double *dframes, cudaStream_t st)
{
    const int nw = nf + ntap - 1;
    const long long ne = (long long)npts * nw;
    const unsigned blocks = (unsigned)std::min<long long>((ne + 255) / 256, 152LL * 16);
    line_green<<<blocks, 256, 0, st>>>(g, pts, npts, f0 - (ntap - 1), nw, dg);
    const dim3 grid((npts + kConvPts - 1) / kConvPts, (nf + kConvFrames - 1) / kConvFrames);
    line_convolve<<<grid, 256, 0, st>>>(dg, npts, nw, dtap, ntap, nf, dframes);
    CK(cudaGetLastError());
    return FD23_OK;
}

// frames per chunk so that g + frames stay within the chunk budget
int chunk_frames(int npts, int ntap, int want)
{
    const long long per = 16LL * npts;  // g and frames, per frame
    long long nf = (long long)(kChunkBytes / (size_t)per) - ntap;
    nf = std::max<long long>(nf, 32);
    return (int)std::min<long long>(std::min<long long>(nf, kMaxChunkFrames), want);
}

struct DevBufs {
    std::vector<void *> p;
    ~DevBufs()
    {
        for (void *q : p) cudaFree(q);
    }
    template <class T>
    int get(T **out, size_t bytes)
    {
        void *q = nullptr;
        const int rc = dev_alloc(&q, bytes ? bytes : 8);
        if (rc) return rc;
        p.push_back(q);
        *out = (T *)q;
        return FD23_OK;
    }
};

int upload_taps(DevBufs &B, const double *src, int lsrc, double **dtap, cudaStream_t st)
{
    const int nt = ntaps(lsrc);
    std::vector<double> tap(nt, 0.0);
    std::copy(src, src + lsrc, tap.begin());
    int rc = B.get(dtap, nt * sizeof(double));
    if (rc) return rc;
    CK(cudaMemcpyAsync(*dtap, tap.data(), nt * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));  // tap is a stack vector
    return FD23_OK;
}

template <class C>
int box_line_source(fd23_solver *s, const fd23_line_desc *d, const double *src, int lsrc, const double *bmat,
                    int it0, int nsteps)
{
    const int bx = s->box_bx, bz = s->box_bz, nring = s->box_nring;
    const int px = bx + 8, pz = bz + 8, plane = px * pz;
    // plane points the ring stencils read: U at (tx-4 .. tx+3, ty) and
    // (tx, ty-4 .. ty+3), W at (tx-3 .. tx+4, ty) and (tx, ty-3 .. ty+4)
    std::vector<int> slot(2 * (size_t)plane, -1);
    std::vector<int2> cells(nring);
    std::vector<double> rm(3 * (size_t)nring);
    const size_t nb = (size_t)bx * bz;
    for (int j = 0; j < bz; ++j)
        for (int i = 0; i < bx; ++i) {
            const int q = box_ring_index(i, j, bx, bz);
            if (q < 0) continue;
            cells[q] = make_int2(i, j);
            const size_t b = (size_t)j * bx + i;
            rm[q] = bmat[b];
            rm[(size_t)nring + q] = bmat[nb + b];
            rm[2 * (size_t)nring + q] = bmat[2 * nb + b];
            const int tx = i + 4, ty = j + 4;
            for (int k = -4; k <= 4; ++k) {
                if (k <= 3) {
                    slot[(size_t)ty * px + tx + k] = 0;
                    slot[(size_t)(ty + k) * px + tx] = 0;
                }
                if (k >= -3) {
                    slot[plane + (size_t)ty * px + tx + k] = 0;
                    slot[plane + (size_t)(ty + k) * px + tx] = 0;
                }
            }
        }
    std::vector<int> list;
    for (int pt = 0; pt < 2 * plane; ++pt)
        if (slot[pt] == 0) {
            slot[pt] = (int)list.size();
            list.push_back(pt);
        }
    const int npts = (int)list.size();
    const int ntap = ntaps(lsrc);
    cudaStream_t st = s->stream;
    const LineGeom g = geom_of(d);
    DevBufs B;
    int rc;
    int *dlist, *dslot, *derr;
    double *drm, *dtap, *dg, *dfr;
    LinePoint *dpts;
    const int nfc = chunk_frames(npts, ntap, nsteps + 1);
    if ((rc = B.get(&dlist, list.size() * sizeof(int))) || (rc = B.get(&dslot, slot.size() * sizeof(int))) ||
        (rc = B.get(&derr, sizeof(int))) || (rc = B.get(&drm, rm.size() * sizeof(double))) ||
        (rc = B.get(&dpts, (size_t)npts * sizeof(LinePoint))) ||
        (rc = B.get(&dg, (size_t)npts * (nfc + ntap - 1) * sizeof(double))) ||
        (rc = B.get(&dfr, (size_t)npts * nfc * sizeof(double))) || (rc = upload_taps(B, src, lsrc, &dtap, st)))
        return rc;
    CK(cudaMemcpyAsync(dlist, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dslot, slot.data(), slot.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(drm, rm.data(), rm.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(derr, 0, sizeof(int), st));
    line_points<<<(npts + 127) / 128, 128, 0, st>>>(g, dlist, npts, dpts);
    // the incident buffer, as fd23_set_box_incident sizes it
    const size_t bytes = (size_t)nsteps * 5 * nring * sizeof(C);
    if (bytes > s->box_inc_bytes) {
        CK(cudaStreamSynchronize(st));
        cudaFree(s->box_inc);
        s->box_inc = nullptr;
        s->box_inc_bytes = 0;
        s->box_inc_n = 0;
        if ((rc = dev_alloc(&s->box_inc, bytes))) return rc;
        s->box_inc_bytes = bytes;
    }
    // chunks of steps: nfc frames give nfc - 1 steps
    for (int s0 = 0; s0 < nsteps;) {
        const int ns = std::min(nsteps - s0, nfc - 1);
        if ((rc = frames_chunk(g, dpts, npts, dtap, ntap, it0 + s0, ns + 1, dg, dfr, st))) return rc;
        const dim3 grid((nring + 127) / 128, ns);
        line_incident<C><<<grid, 128, 0, st>>>(bx, bz, s->box_cells, nring, drm, drm + nring, drm + 2 * nring, dslot,
                                               dfr, npts, ns, d->dt,
                                               (C *)s->box_inc + (size_t)s0 * 5 * nring, derr);
        CK(cudaGetLastError());
        s0 += ns;
    }
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (herr) return FD23_ERR_CUDA;  // a stencil cell without a point (not reachable by construction)
    s->box_inc_it0 = it0;
    s->box_inc_n = nsteps;
    return FD23_OK;
}

}  // namespace

}  // namespace fd23

using namespace fd23;

extern "C" {

int fd23_line_source_coefs(double strike, double dip, double rake, double azimuth, double a[3])
{
    if (!a) return FD23_ERR_ARG;
    const double d = dip * kPiRef / 180.0, l = rake * kPiRef / 180.0, th = (azimuth - strike) * kPiRef / 180.0;
    a[0] = std::sin(2.0 * th) * std::cos(l) * std::sin(d) + 0.5 * std::cos(2.0 * th) * std::sin(l) * std::sin(2.0 * d);
    a[1] = std::cos(th) * std::cos(l) * std::cos(d) - std::sin(th) * std::sin(l) * std::cos(2.0 * d);
    a[2] = 0.5 * std::sin(l) * std::sin(2.0 * d);
    return FD23_OK;
}

int fd23_line_plane_origin(int bw) { return (bw + 1) / 2 + 4 + 1 - (bw + 8); }

int fd23_line_source_planes(int device, const fd23_line_desc *d, const double *src, int lsrc, int it0, int nframes,
                            double *out)
{
    if (!desc_ok(d, src, lsrc) || it0 < 0 || nframes < 0 || (nframes > 0 && !out)) return FD23_ERR_ARG;
    if (nframes == 0) return FD23_OK;
    CK(cudaSetDevice(device));
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } guard{st};
    const int npts = 2 * d->px * d->pz, ntap = ntaps(lsrc);
    const int nfc = chunk_frames(npts, ntap, nframes);
    const LineGeom g = geom_of(d);
    DevBufs B;
    int rc;
    double *dtap, *dg, *dfr;
    LinePoint *dpts;
    if ((rc = B.get(&dpts, (size_t)npts * sizeof(LinePoint))) ||
        (rc = B.get(&dg, (size_t)npts * (nfc + ntap - 1) * sizeof(double))) ||
        (rc = B.get(&dfr, (size_t)npts * nfc * sizeof(double))) || (rc = upload_taps(B, src, lsrc, &dtap, st)))
        return rc;
    line_points<<<(npts + 127) / 128, 128, 0, st>>>(g, nullptr, npts, dpts);
    for (int f0 = 0; f0 < nframes; f0 += nfc) {
        const int nf = std::min(nfc, nframes - f0);
        if ((rc = frames_chunk(g, dpts, npts, dtap, ntap, it0 + f0, nf, dg, dfr, st))) return rc;
        CK(cudaMemcpyAsync(out + (size_t)f0 * npts, dfr, (size_t)nf * npts * sizeof(double), cudaMemcpyDeviceToHost,
                           st));
    }
    CK(cudaStreamSynchronize(st));
    return FD23_OK;
}

int fd23_set_box_line_source(fd23_solver *s, const fd23_line_desc *d, const double *src, int lsrc,
                             const double *bmat, int it0, int nsteps)
{
    if (!s || !desc_ok(d, src, lsrc) || !bmat || it0 < 0 || nsteps < 0) return FD23_ERR_ARG;
    if (!s->box_on) return FD23_ERR_ORDER;
    if (d->px != s->box_bx + 8 || d->pz != s->box_bz + 8) return FD23_ERR_ARG;
    CK(cudaSetDevice(s->d.device));
    if (nsteps == 0) {
        s->box_inc_it0 = it0;
        s->box_inc_n = 0;
        return FD23_OK;
    }
    return s->d.prec == FD23_F64 ? box_line_source<double>(s, d, src, lsrc, bmat, it0, nsteps)
                                 : box_line_source<float>(s, d, src, lsrc, bmat, it0, nsteps);
}

}  // extern "C"
