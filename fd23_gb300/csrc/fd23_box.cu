// Hybrid-box kernels (P-SV): the ring exchanges between the grid field g and
// the residual field r, and the residual-field updates.
//
// Reference: ring exchanges PD/box/cu_box.cu:48-79 (ker_subsource,
// ker_addsource), residual updates PD/fd/cu_fd.cu:93-207 (one 32x32 block,
// boxes up to 32 cells) and PD/fd/fd.cpp:63-91, 208-234 (host, interior cells
// 4 .. n-5).  Here a box is any rectangle of at least 16 x 16 cells; the
// residual updates cover cells 4 .. n-5 of the box (the outer 4 are the sub
// ring, rewritten from g before every read), with one thread per cell.
// Every box kernel launches as a programmatic dependent of the kernel before
// it, so its launch latency hides under that kernel's tail.  Boxes whose
// interior and rings fit eight passes of a 1024-thread CTA (the reference's
// own boxes, up to 32 cells, among them) run each half of the box step as
// one CTA: two small launches per step instead of four.
//
// Stress exchange around the fused sweep: the residual stress update writes
// g = r + s into the old-stress slot of every add-ring cell, and the sweep
// keeps that value there instead of updating it (it is what the exchange
// after the stress update and the point source would store); after the sweep
// a ring kernel forms r = g - s on the sub ring.  The two-pass sweep runs the
// full stress exchange between its passes instead.
#include "fd23_device.cuh"
#include "fd23_kernels.h"

namespace fd23 {

namespace {

template <class C>
__device__ __forceinline__ C dminus_r(const C *p, long long s)
{
    return comb<C>(Coef4<C>::c0, Coef4<C>::c1, Coef4<C>::c2, Coef4<C>::c3, p[0] - p[-s], p[s] - p[-2 * s],
                   p[2 * s] - p[-3 * s], p[3 * s] - p[-4 * s]);
}
template <class C>
__device__ __forceinline__ C dplus_r(const C *p, long long s)
{
    return comb<C>(Coef4<C>::c0, Coef4<C>::c1, Coef4<C>::c2, Coef4<C>::c3, p[s] - p[0], p[2 * s] - p[-s],
                   p[3 * s] - p[-2 * s], p[4 * s] - p[-3 * s]);
}

// ring exchange of fields F0 .. F1-1 on buffer set `par`, ring positions
// [0, qend) (qend = nsub: the sub ring only)
// (inc: the step's incident field, [5][nring])
template <class S, class C, int F0, int F1>
__device__ __forceinline__ void ring_cell(const Shot<S, C> &s, int par, int q, const C *inc)
{
    const Box<C> &b = s.box;
    const int2 c = b.cells[q];
    const long long g = s.origin + (long long)(b.z0 + c.y) * s.pitch + (b.x0 + c.x);
    const long long r = (long long)c.y * b.bx + c.x;
    const bool add = q >= b.nsub;
#pragma unroll
    for (int f = F0; f < F1; ++f) {
        S *G = par ? s.f[1][f] : s.f[0][f];
        const C sv = inc[(long long)f * b.nring + q];
        if (add) G[g] = to_s<S>(b.r[f][r] + sv);
        else b.r[f][r] = to_c<C>(G[g]) - sv;
    }
}

// Every box kernel may run as a programmatic dependent of the kernel before
// it: it waits for that kernel (griddepcontrol.wait) before touching memory
// and lets its own successor launch at once (the successor waits in turn).
// Launched without the attribute, both instructions are no-ops.
__device__ __forceinline__ void pdl_enter()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <class S, class C, int F0, int F1>
__global__ void __launch_bounds__(256) box_ring_kernel(Shot<S, C> s, int par, int qend)
{
    pdl_enter();
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < qend; q += gridDim.x * blockDim.x)
        ring_cell<S, C, F0, F1>(s, par, q, s.box.inc);
}

// residual stress update of box cell (ix, iz), 4 <= ix, iz < n-4; the
// accumulation order is that of the main update (x terms, then z terms).
// On add-ring cells it also stores g = r + s into the grid stresses of
// buffer set `par` (the fused sweep's old-stress slot); add_g = 0 skips that.
template <class S, class C>
__device__ __forceinline__ void stress_r_cell(const Shot<S, C> &s, int par, int add_g, int ix, int iz, const C *inc)
{
    const Box<C> &b = s.box;
    const long long o = (long long)iz * b.bx + ix, P = b.bx;
    const C ux = dminus_r<C>(b.r[0] + o, 1), uz = dminus_r<C>(b.r[0] + o, P);
    const C wx = dplus_r<C>(b.r[1] + o, 1), wz = dplus_r<C>(b.r[1] + o, P);
    const C lam = b.rmat[0][o], mua = b.rmat[2][o];
    const C gam = lam + (C)2 * b.rmat[1][o];
    C txx = b.r[2][o], txz = b.r[3][o], tzz = b.r[4][o];
    txx = fmaC<C>(gam, ux, txx);
    tzz = fmaC<C>(lam, ux, tzz);
    txz = fmaC<C>(mua, wx, txz);
    txx = fmaC<C>(lam, wz, txx);
    tzz = fmaC<C>(gam, wz, tzz);
    txz = fmaC<C>(mua, uz, txz);
    b.r[2][o] = txx;
    b.r[3][o] = txz;
    b.r[4][o] = tzz;
    if (add_g) {
        const int q = box_ring_index(ix, iz, b.bx, b.bz);
        if (q >= b.nsub) {
            const long long g = s.origin + (long long)(b.z0 + iz) * s.pitch + (b.x0 + ix);
            const C t[3] = {txx, txz, tzz};
#pragma unroll
            for (int f = 0; f < 3; ++f) {
                S *G = par ? s.f[1][2 + f] : s.f[0][2 + f];
                G[g] = to_s<S>(t[f] + inc[(long long)(2 + f) * b.nring + q]);
            }
        }
    }
}

template <class S, class C>
__global__ void __launch_bounds__(256) box_stress_r(Shot<S, C> s, int par, int add_g)
{
    pdl_enter();
    const int ix = 4 + blockIdx.x * 32 + threadIdx.x, iz = 4 + blockIdx.y * 8 + threadIdx.y;
    if (ix >= s.box.bx - 4 || iz >= s.box.bz - 4) return;
    stress_r_cell<S, C>(s, par, add_g, ix, iz, s.box.inc);
}

// receivers of this step's output (buffer set `par`, before the next ring
// exchange rewrites the add ring): thread t of nthr
template <class S, class C>
__device__ __forceinline__ void box_receivers(const Shot<S, C> &s, int par, int rec_index, int t0, int nthr)
{
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        const S *F = par ? s.f[1][c] : s.f[0][c];
        for (int i = t0; i < s.nrec[c]; i += nthr)
            s.seis[c][(long long)rec_index * s.nrec[c] + i] = to_c<C>(F[s.rec[c][i]]);
    }
}

// residual velocity update of box cell (ix, iz)
template <class S, class C>
__device__ __forceinline__ void velocity_r_cell(const Shot<S, C> &s, int ix, int iz)
{
    const Box<C> &b = s.box;
    const long long o = (long long)iz * b.bx + ix, P = b.bx;
    const C dxTxx = dplus_r<C>(b.r[2] + o, 1), dzTzz = dminus_r<C>(b.r[4] + o, P);
    const C dxTxz = dminus_r<C>(b.r[3] + o, 1), dzTxz = dplus_r<C>(b.r[3] + o, P);
    const C bu = b.rmat[3][o], bw = b.rmat[4][o];
    C u = b.r[0][o], w = b.r[1][o];
    u = fmaC<C>(bu, dxTxx, u);
    w = fmaC<C>(bw, dxTxz, w);
    u = fmaC<C>(bu, dzTxz, u);
    w = fmaC<C>(bw, dzTzz, w);
    b.r[0][o] = u;
    b.r[1][o] = w;
}

template <class S, class C>
__global__ void __launch_bounds__(256) box_velocity_r(Shot<S, C> s, int par, int rec_index)
{
    pdl_enter();
    if (rec_index >= 0) {
        const int nthr = gridDim.x * gridDim.y * blockDim.x * blockDim.y;
        const int t0 = (blockIdx.y * gridDim.x + blockIdx.x) * (blockDim.x * blockDim.y) +
                       threadIdx.y * blockDim.x + threadIdx.x;
        box_receivers<S, C>(s, par, rec_index, t0, nthr);
    }
    const int ix = 4 + blockIdx.x * 32 + threadIdx.x, iz = 4 + blockIdx.y * 8 + threadIdx.y;
    if (ix >= s.box.bx - 4 || iz >= s.box.bz - 4) return;
    velocity_r_cell<S, C>(s, ix, iz);
}

// Small boxes: each half of the box step in one CTA, the ring exchange and
// the residual update it feeds separated by a barrier instead of a kernel
// boundary, launched as programmatic dependents so their launch overlaps
// the sweep.  Each waits for its predecessor (griddepcontrol.wait) before
// it touches memory and lets its successor launch at once (the successor
// waits for this grid's completion in turn).
constexpr int kSmallThreads = 1024;

// before the sweep: ring U, W (sub: r = g - s, add: g = r + s), then the
// residual stress update (+ g = r + s on the add ring for the fused sweep)
template <class S, class C>
__device__ __forceinline__ void small_pre_body(const Shot<S, C> &s, int par, int add_g, const C *inc)
{
    const Box<C> &b = s.box;
    const int t = threadIdx.x;
    for (int q = t; q < b.nring; q += kSmallThreads) ring_cell<S, C, 0, 2>(s, par, q, inc);
    __syncthreads();
    const int w = b.bx - 8, n = w * (b.bz - 8);
    for (int k = t; k < n; k += kSmallThreads) stress_r_cell<S, C>(s, par, add_g, 4 + k % w, 4 + k / w, inc);
}

template <class S, class C>
__global__ void __launch_bounds__(kSmallThreads, 1) box_small_pre(Shot<S, C> s, int par, int add_g)
{
    pdl_enter();
    small_pre_body<S, C>(s, par, add_g, s.box.inc);
}

// after the sweep: sub-ring stresses r = g - s (fused sweep only; the
// two-pass sweep did the whole exchange), then this step's receivers and
// the residual velocity update
template <class S, class C>
__device__ __forceinline__ void small_post_body(const Shot<S, C> &s, int par, int sub_t, int rec_index)
{
    const Box<C> &b = s.box;
    const int t = threadIdx.x;
    if (sub_t) {
        for (int q = t; q < b.nsub; q += kSmallThreads) ring_cell<S, C, 2, 5>(s, par, q, b.inc);
        __syncthreads();
    }
    if (rec_index >= 0) box_receivers<S, C>(s, par, rec_index, t, kSmallThreads);
    const int w = b.bx - 8, n = w * (b.bz - 8);
    for (int k = t; k < n; k += kSmallThreads) velocity_r_cell<S, C>(s, 4 + k % w, 4 + k / w);
}

template <class S, class C>
__global__ void __launch_bounds__(kSmallThreads, 1) box_small_post(Shot<S, C> s, int par, int sub_t, int rec_index)
{
    pdl_enter();
    small_post_body<S, C>(s, par, sub_t, rec_index);
}

// Between two steps of the fused sweep: the end of one step and the start of
// the next in one CTA, a barrier in place of a kernel boundary.  No sweep
// runs between them, so both work on buffer set `par`; the next step's
// incident field is inc_next.
template <class S, class C>
__global__ void __launch_bounds__(kSmallThreads, 1)
    box_small_mid(Shot<S, C> s, int par, int rec_index, const C *inc_next)
{
    pdl_enter();
    small_post_body<S, C>(s, par, 1, rec_index);
    __syncthreads();
    small_pre_body<S, C>(s, par, 1, inc_next);
}

// boxes whose interior and rings each fit a few passes of one CTA
template <class C>
inline bool small_box(const Box<C> &b)
{
    return (long long)(b.bx - 8) * (b.bz - 8) <= 8 * kSmallThreads && b.nring <= 8 * kSmallThreads;
}

template <class K, class... Args>
int launch_pdl(K kernel, dim3 grid, dim3 block, cudaStream_t st, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...) == cudaSuccess ? FD23_OK : FD23_ERR_CUDA;
}

inline dim3 interior_grid(int bx, int bz) { return dim3((unsigned)((bx - 8 + 31) / 32), (unsigned)((bz - 8 + 7) / 8)); }
inline unsigned ring_blocks(int nring) { return (unsigned)((nring + 255) / 256); }

}  // namespace

template <class S, class C>
int launch_box_ring(const Shot<S, C> &s, int par, int which, cudaStream_t st)
{
    const int n = s.box.nring;
    if (which == 0) return launch_pdl(box_ring_kernel<S, C, 0, 2>, dim3(ring_blocks(n)), dim3(256), st, s, par, n);
    return launch_pdl(box_ring_kernel<S, C, 2, 5>, dim3(ring_blocks(n)), dim3(256), st, s, par, n);
}

template <class S, class C>
int launch_box_pre(const Shot<S, C> &s, int par, int fused, cudaStream_t st)
{
    if (fused && small_box(s.box))
        return launch_pdl(box_small_pre<S, C>, dim3(1), dim3(kSmallThreads), st, s, par, fused);
    const int rc = launch_box_ring<S, C>(s, par, 0, st);
    if (rc) return rc;
    return launch_pdl(box_stress_r<S, C>, interior_grid(s.box.bx, s.box.bz), dim3(32, 8), st, s, par, fused);
}

template <class S, class C>
int launch_box_post(const Shot<S, C> &s, int par, int fused, int rec_index, cudaStream_t st)
{
    if (fused && small_box(s.box))
        return launch_pdl(box_small_post<S, C>, dim3(1), dim3(kSmallThreads), st, s, par, fused, rec_index);
    if (fused) {  // sub-ring stresses r = g - s (the two-pass sweep did the whole exchange)
        const int rc = launch_pdl(box_ring_kernel<S, C, 2, 5>, dim3(ring_blocks(s.box.nsub)), dim3(256), st, s, par,
                                  s.box.nsub);
        if (rc) return rc;
    }
    return launch_pdl(box_velocity_r<S, C>, interior_grid(s.box.bx, s.box.bz), dim3(32, 8), st, s, par, rec_index);
}

template <class S, class C>
int launch_box_mid(const Shot<S, C> &s, int par, int rec_index, cudaStream_t st)
{
    if (!small_box(s.box)) return FD23_ERR_UNSUPPORTED;
    const C *inc_next = s.box.inc + (size_t)5 * s.box.nring;
    return launch_pdl(box_small_mid<S, C>, dim3(1), dim3(kSmallThreads), st, s, par, rec_index, inc_next);
}

#define FD23_INST(S, C)                                                                  \
    template int launch_box_ring<S, C>(const Shot<S, C> &, int, int, cudaStream_t);     \
    template int launch_box_pre<S, C>(const Shot<S, C> &, int, int, cudaStream_t);      \
    template int launch_box_post<S, C>(const Shot<S, C> &, int, int, int, cudaStream_t); \
    template int launch_box_mid<S, C>(const Shot<S, C> &, int, int, cudaStream_t);
FD23_INST(float, float)
FD23_INST(double, double)
FD23_INST(__nv_bfloat16, float)
FD23_INST(__half, float)
#undef FD23_INST

}  // namespace fd23
