// Two-pass sweep: one thread per cell, a stress launch then a velocity launch
// per time step, updating the fields in place (as the reference does; the
// stress pass reads only velocities and writes only stresses, and vice
// versa, so in-place updates are race free).  This is the simple GPU form of
// the reference kernels (PD/fd/cu_fd.cu:209-501, SH/fd/cu_fd.cu:77-288) on the
// padded layout, for any nx, nz.  The fused single-pass sweep
// (fd23_fused.cuh, instantiated by fd23_fused*.cu) is the fast path; this one is the cross-check and the
// fallback for forms the fused sweep does not cover.
#include <algorithm>

#include "fd23_device.cuh"
#include "fd23_kernels.h"

namespace fd23 {

namespace {

// backward (D-minus) and forward (D-plus) differences along a stride
template <class S, class C>
__device__ __forceinline__ C dminus(const S *p, long long s, C c0, C c1, C c2, C c3)
{
    auto v = [&](int j) { return to_c<C>(p[j * s]); };
    return comb<C>(c0, c1, c2, c3, v(0) - v(-1), v(1) - v(-2), v(2) - v(-3), v(3) - v(-4));
}
template <class S, class C>
__device__ __forceinline__ C dplus(const S *p, long long s, C c0, C c1, C c2, C c3)
{
    auto v = [&](int j) { return to_c<C>(p[j * s]); };
    return comb<C>(c0, c1, c2, c3, v(1) - v(0), v(2) - v(-1), v(3) - v(-2), v(4) - v(-3));
}

// material array m at padded offset o, through the material table when the
// shot has one (lossless: the table holds the stored values)
template <class S, class C>
__device__ __forceinline__ C matv(const Shot<S, C> &s, int m, long long o)
{
    return s.midx ? to_c<C>(s.mtab[m * kTabEntries + s.midx[o]]) : to_c<C>(s.mat[m][o]);
}

template <class C>
__device__ __forceinline__ long long psi_x_index(int ix, int iz, int nx, int npml)
{
    // PD/fd/cu_fd.cu:305,315
    return ix < npml ? (long long)ix + (long long)iz * 2 * npml
                     : (long long)npml + nx - 1 - ix + (long long)iz * 2 * npml;
}
__device__ __forceinline__ long long psi_z_index(int ix, int iz, int nx, int nz, int npml, bool top)
{
    // PD/fd/cu_fd.cu:330,339
    return top ? (long long)iz * nx + ix : (long long)(npml + nz - 1 - iz) * nx + ix;
}

// ----------------------------- P-SV ---------------------------------------
template <class S, class C>
__device__ __forceinline__ void psv_stress_cell(const Shot<S, C> &s, int it, int ix, int iz)
{
    if (!punch_active(s.punch, ix, iz, it)) return;  // outside the tile's step window
    const long long o = s.origin + (long long)iz * s.pitch + ix, P = s.pitch;
    const S *U = s.f[0][0], *W = s.f[0][1];
    S *Txx = s.f[0][2], *Txz = s.f[0][3], *Tzz = s.f[0][4];
    const int ord = stencil_order(ix, iz, s.nx, s.nz);
    const C c0 = Coef<C>::get(ord, 0), c1 = Coef<C>::get(ord, 1), c2 = Coef<C>::get(ord, 2),
            c3 = Coef<C>::get(ord, 3);
    const C ux = dminus<S, C>(U + o, 1, c0, c1, c2, c3);
    const C uz = dminus<S, C>(U + o, P, c0, c1, c2, c3);
    const C wx = dplus<S, C>(W + o, 1, c0, c1, c2, c3);
    const C wz = dplus<S, C>(W + o, P, c0, c1, c2, c3);
    const C lam = matv<S, C>(s, 0, o), mu = matv<S, C>(s, 1, o), mua = matv<S, C>(s, 2, o);
    const C gam = lam + (C)2 * mu;
    C txx = to_c<C>(Txx[o]), tzz = to_c<C>(Tzz[o]), txz = to_c<C>(Txz[o]);
    const int nx = s.nx, nz = s.nz, npml = s.npml, B = s.cpml_blk;
    const C *b = s.cpml, *c = s.cpml + B, *k = s.cpml + 2 * B;
    // x chain, PD/fd/cu_fd.cu:303-326 (components: 0 Txx_x 1 Txz_x 2 U_x 3 W_x)
    if (ix < npml || ix >= nx - npml) {
        const long long p = psi_x_index<C>(ix, iz, nx, npml);
        C *pU = s.psi[0][2], *pW = s.psi[0][3];
        const C ps = fmaC<C>(b[2 * nx + ix], pU[p], c[2 * nx + ix] * ux);
        pU[p] = ps;
        const C t = fmaC<C>(ux, k[2 * nx + ix], ps);
        txx = fmaC<C>(gam, t, txx);
        tzz = fmaC<C>(lam, t, tzz);
        const C pw = fmaC<C>(b[3 * nx + ix], pW[p], c[3 * nx + ix] * wx);
        pW[p] = pw;
        txz = fmaC<C>(mua, fmaC<C>(wx, k[3 * nx + ix], pw), txz);
    } else if (iz != 0) {
        txx = fmaC<C>(gam, ux, txx);
        tzz = fmaC<C>(lam, ux, tzz);
        txz = fmaC<C>(mua, wx, txz);
    }
    // z chain, :328-355 (components after 4*nx: 0 Tzz_z 1 Txz_z 2 U_z 3 W_z)
    const bool top = iz < npml && s.topabsorb;
    if (top || iz >= nz - npml) {
        const long long p = psi_z_index(ix, iz, nx, nz, npml, top);
        C *pU = s.psi[0][6], *pW = s.psi[0][7];
        const int zb = 4 * nx;
        const C pw = fmaC<C>(b[zb + 3 * nz + iz], pW[p], c[zb + 3 * nz + iz] * wz);
        pW[p] = pw;
        const C t = fmaC<C>(wz, k[zb + 3 * nz + iz], pw);
        txx = fmaC<C>(lam, t, txx);
        tzz = fmaC<C>(gam, t, tzz);
        const C pu = fmaC<C>(b[zb + 2 * nz + iz], pU[p], c[zb + 2 * nz + iz] * uz);
        pU[p] = pu;
        txz = fmaC<C>(mua, fmaC<C>(uz, k[zb + 2 * nz + iz], pu), txz);
    } else if (iz == 0) {
        txx = fmaC<C>((C)2 * mu, ux, txx);
        tzz = (C)0;
        txz = (C)0;
    } else {
        txx = fmaC<C>(lam, wz, txx);
        tzz = fmaC<C>(gam, wz, tzz);
        txz = fmaC<C>(mua, uz, txz);
    }
    Txx[o] = to_s<S>(txx);
    Tzz[o] = to_s<S>(tzz);
    Txz[o] = to_s<S>(txz);
}

template <class S, class C>
__device__ __forceinline__ void psv_velocity_cell(const Shot<S, C> &s, int it, int ix, int iz)
{
    if (!punch_active(s.punch, ix, iz, it)) return;  // outside the tile's step window
    const long long o = s.origin + (long long)iz * s.pitch + ix, P = s.pitch;
    S *U = s.f[0][0], *W = s.f[0][1];
    const S *Txx = s.f[0][2], *Txz = s.f[0][3], *Tzz = s.f[0][4];
    const int ord = stencil_order(ix, iz, s.nx, s.nz);
    const C c0 = Coef<C>::get(ord, 0), c1 = Coef<C>::get(ord, 1), c2 = Coef<C>::get(ord, 2),
            c3 = Coef<C>::get(ord, 3);
    const C dxTxx = dplus<S, C>(Txx + o, 1, c0, c1, c2, c3);
    const C dzTzz = dminus<S, C>(Tzz + o, P, c0, c1, c2, c3);
    const C dxTxz = dminus<S, C>(Txz + o, 1, c0, c1, c2, c3);
    const C dzTxz = dplus<S, C>(Txz + o, P, c0, c1, c2, c3);
    const C bu = matv<S, C>(s, 3, o), bw = matv<S, C>(s, 4, o);
    C u = to_c<C>(U[o]), w = to_c<C>(W[o]);
    const int nx = s.nx, nz = s.nz, npml = s.npml, B = s.cpml_blk;
    const C *b = s.cpml, *c = s.cpml + B, *k = s.cpml + 2 * B;
    // x chain, PD/fd/cu_fd.cu:455-474
    if (ix < npml || ix >= nx - npml) {
        const long long p = psi_x_index<C>(ix, iz, nx, npml);
        C *pXX = s.psi[0][0], *pXZ = s.psi[0][1];
        const C a = fmaC<C>(b[ix], pXX[p], c[ix] * dxTxx);
        pXX[p] = a;
        u = fmaC<C>(bu, fmaC<C>(dxTxx, k[ix], a), u);
        const C q = fmaC<C>(b[nx + ix], pXZ[p], c[nx + ix] * dxTxz);
        pXZ[p] = q;
        w = fmaC<C>(bw, fmaC<C>(dxTxz, k[nx + ix], q), w);
    } else if (iz != 0) {
        u = fmaC<C>(bu, dxTxx, u);
        w = fmaC<C>(bw, dxTxz, w);
    }
    // z chain, :476-499
    const bool top = iz < npml && s.topabsorb;
    if (top || iz >= nz - npml) {
        const long long p = psi_z_index(ix, iz, nx, nz, npml, top);
        C *pZZ = s.psi[0][4], *pXZ = s.psi[0][5];
        const int zb = 4 * nx;
        const C a = fmaC<C>(b[zb + nz + iz], pXZ[p], c[zb + nz + iz] * dzTxz);
        const C q = fmaC<C>(b[zb + iz], pZZ[p], c[zb + iz] * dzTzz);
        pXZ[p] = a;
        pZZ[p] = q;
        u = fmaC<C>(bu, fmaC<C>(dzTxz, k[zb + nz + iz], a), u);
        w = fmaC<C>(bw, fmaC<C>(dzTzz, k[zb + iz], q), w);
    } else if (iz == 0) {
        u = fmaC<C>(bu, dxTxx + dzTxz, u);
        w = (C)0;
    } else {
        u = fmaC<C>(bu, dzTxz, u);
        w = fmaC<C>(bw, dzTzz, w);
    }
    U[o] = to_s<S>(u);
    W[o] = to_s<S>(w);
}

// ------------------------------ SH ----------------------------------------
template <class S, class C>
__device__ __forceinline__ void sh_stress_cell(const Shot<S, C> &s, int it, int ix, int iz)
{
    if (!punch_active(s.punch, ix, iz, it)) return;  // outside the tile's step window
    // cells skipped by the reference, SH/fd/cu_fd.cu:140
    if (ix == 0 || ix >= s.nx - 1 || iz >= s.nz - 1) return;
    const long long o = s.origin + (long long)iz * s.pitch + ix, P = s.pitch;
    const S *V = s.f[0][0];
    S *Tx = s.f[0][1], *Tz = s.f[0][2];
    const int ord = stencil_order(ix, iz, s.nx, s.nz);
    const C c0 = Coef<C>::get(ord, 0), c1 = Coef<C>::get(ord, 1), c2 = Coef<C>::get(ord, 2),
            c3 = Coef<C>::get(ord, 3);
    const C dxV = dplus<S, C>(V + o, 1, c0, c1, c2, c3);
    const C dzV = dminus<S, C>(V + o, P, c0, c1, c2, c3);
    const C mux = matv<S, C>(s, 0, o), muz = matv<S, C>(s, 1, o);
    const int nx = s.nx, nz = s.nz, npml = s.npml, B = s.cpml_blk;
    const C *b = s.cpml, *c = s.cpml + B, *k = s.cpml + 2 * B;
    C tx = to_c<C>(Tx[o]), tz = to_c<C>(Tz[o]);
    // components: x: 0 Tx_x 1 V_x ; z (after 2*nx): 0 Tz_z 1 V_z
    if (ix < npml || ix >= nx - npml) {
        const long long p = psi_x_index<C>(ix, iz, nx, npml);
        C *pV = s.psi[0][1];
        const C a = fmaC<C>(b[nx + ix], pV[p], c[nx + ix] * dxV);
        pV[p] = a;
        tx = fmaC<C>(mux, fmaC<C>(dxV, k[nx + ix], a), tx);
    } else {
        tx = fmaC<C>(mux, dxV, tx);
    }
    const bool top = iz < npml && s.topabsorb;
    if (top || iz >= nz - npml) {
        const long long p = psi_z_index(ix, iz, nx, nz, npml, top);
        C *pV = s.psi[0][3];
        const int zb = 2 * nx;
        const C a = fmaC<C>(b[zb + nz + iz], pV[p], c[zb + nz + iz] * dzV);
        pV[p] = a;
        tz = fmaC<C>(muz, fmaC<C>(dzV, k[zb + nz + iz], a), tz);
    } else {
        tz = fmaC<C>(muz, dzV, tz);
    }
    Tx[o] = to_s<S>(tx);
    Tz[o] = to_s<S>(tz);
}

// IMG (the persistent form): the free-surface image Tz(x,0) = -Tz(x,1) of
// this step has not been stored yet; the cells whose z stencil reaches row 0
// read the image value in its place, and the cell of row 0 stores it (the
// same values the two-pass order gives: image first, then the update)
template <class S, class C, bool IMG = false>
__device__ __forceinline__ void sh_velocity_cell(const Shot<S, C> &s, int it, int ix, int iz)
{
    if (!punch_active(s.punch, ix, iz, it)) return;  // outside the tile's step window
    const long long o = s.origin + (long long)iz * s.pitch + ix, P = s.pitch;
    S *V = s.f[0][0];
    const S *Tx = s.f[0][1], *Tz = s.f[0][2];
    const int ord = stencil_order(ix, iz, s.nx, s.nz);
    const C c0 = Coef<C>::get(ord, 0), c1 = Coef<C>::get(ord, 1), c2 = Coef<C>::get(ord, 2),
            c3 = Coef<C>::get(ord, 3);
    const C dxTx = dminus<S, C>(Tx + o, 1, c0, c1, c2, c3);
    C dzTz;
    if (IMG && iz <= 3 && punch_active(s.punch, ix, 0, it)) {
        const long long o0 = s.origin + ix;
        const S img = to_s<S>(-to_c<C>(Tz[o0 + P]));
        if (iz == 0) s.f[0][2][o0] = img;
        auto v = [&](int j) { return iz + j == 0 ? to_c<C>(img) : to_c<C>(Tz[o + j * P]); };
        dzTz = comb<C>(c0, c1, c2, c3, v(1) - v(0), v(2) - v(-1), v(3) - v(-2), v(4) - v(-3));
    } else {
        dzTz = dplus<S, C>(Tz + o, P, c0, c1, c2, c3);
    }
    const C bv = matv<S, C>(s, 2, o);
    const int nx = s.nx, nz = s.nz, npml = s.npml, B = s.cpml_blk;
    const C *b = s.cpml, *c = s.cpml + B, *k = s.cpml + 2 * B;
    C v = to_c<C>(V[o]);
    if (ix < npml || ix >= nx - npml) {
        const long long p = psi_x_index<C>(ix, iz, nx, npml);
        C *pT = s.psi[0][0];
        const C a = fmaC<C>(b[ix], pT[p], c[ix] * dxTx);
        pT[p] = a;
        v = fmaC<C>(bv, fmaC<C>(dxTx, k[ix], a), v);
    } else {
        v = fmaC<C>(bv, dxTx, v);
    }
    const bool top = iz < npml && s.topabsorb;
    if (top || iz >= nz - npml) {
        const long long p = psi_z_index(ix, iz, nx, nz, npml, top);
        C *pT = s.psi[0][2];
        const int zb = 2 * nx;
        const C a = fmaC<C>(b[zb + iz], pT[p], c[zb + iz] * dzTz);
        pT[p] = a;
        v = fmaC<C>(bv, fmaC<C>(dzTz, k[zb + iz], a), v);
    } else {
        v = fmaC<C>(bv, dzTz, v);
    }
    V[o] = to_s<S>(v);
}

// one thread per cell
template <class S, class C>
__global__ void __launch_bounds__(256) psv_stress_2p(Shot<S, C> s, int it)
{
    const int ix = blockIdx.x * 32 + threadIdx.x, iz = blockIdx.y * 8 + threadIdx.y;
    if (ix < s.nx && iz < s.nz) psv_stress_cell<S, C>(s, it, ix, iz);
}
template <class S, class C>
__global__ void __launch_bounds__(256) psv_velocity_2p(Shot<S, C> s, int it)
{
    const int ix = blockIdx.x * 32 + threadIdx.x, iz = blockIdx.y * 8 + threadIdx.y;
    if (ix < s.nx && iz < s.nz) psv_velocity_cell<S, C>(s, it, ix, iz);
}
template <class S, class C>
__global__ void __launch_bounds__(256) sh_stress_2p(Shot<S, C> s, int it)
{
    const int ix = blockIdx.x * 32 + threadIdx.x, iz = blockIdx.y * 8 + threadIdx.y;
    if (ix < s.nx && iz < s.nz) sh_stress_cell<S, C>(s, it, ix, iz);
}
template <class S, class C>
__global__ void __launch_bounds__(256) sh_velocity_2p(Shot<S, C> s, int it)
{
    const int ix = blockIdx.x * 32 + threadIdx.x, iz = blockIdx.y * 8 + threadIdx.y;
    if (ix < s.nx && iz < s.nz) sh_velocity_cell<S, C>(s, it, ix, iz);
}

// Point-source injection after the stress update (terms in order, one thread),
// then for SH the free-surface stress image Tz(x,0) = -Tz(x,1) that the
// reference applies at the top of its velocity kernel (SH/fd/cu_fd.cu:226),
// so only in the tiles that kernel updates at this step.
template <class S, class C>
__global__ void post_stress_2p(Shot<S, C> s, int it, int sh_image)
{
    if (threadIdx.x == 0 && it < s.tamp_nt) {
        for (int t = 0; t < s.nterms; ++t) {
            const int4 tm = s.terms[t];
            S *F = s.f[0][tm.x];
            const long long o = s.origin + (long long)tm.z * s.pitch + tm.y;
            F[o] = to_s<S>(to_c<C>(F[o]) + s.tamp[(long long)t * s.tamp_nt + it]);
        }
    }
    if (sh_image && s.nz > 1) {
        __syncthreads();
        S *Tz = s.f[0][2];
        for (int ix = threadIdx.x; ix < s.nx; ix += blockDim.x) {
            if (!punch_active(s.punch, ix, 0, it)) continue;
            const long long o = s.origin + ix;
            Tz[o] = to_s<S>(-to_c<C>(Tz[o + s.pitch]));
        }
    }
}

// ---------------- persistent form for small grids ----------------
// A grid whose fields sit in L2 steps in a few microseconds of work, less
// than one launch of either sweep costs.  Here one cooperative launch runs
// many steps: every phase of the two-pass update (stress, then velocity) is
// a loop over all cells by all threads of the grid, phases separated by a
// grid-wide barrier, with the two-pass kernels' per-cell code and the same
// in-place updates, so results are those of the two-pass sweep bit for bit.

// Grid barrier (all blocks co-resident: cooperative launch).  Block leaders
// arrive on a counter with an acquire-release add (so the last one has seen
// every other block's writes); the last resets the counter and releases the
// next generation, which the others wait for with acquire loads.  Every wait
// is bounded: past the limit, or when another block has given up, the block
// sets err = 3 and the caller abandons the launch (the host reports a
// timeout).
constexpr int kBarSpin = 1 << 24;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// spin: the wait's iteration limit; extra: arrivals beyond the grid's
// blocks the barrier waits for (0; 1 only in the failure-path check, where
// nothing completes it)
__device__ bool grid_barrier(unsigned *bar, int *err, int spin, int extra)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned *count = bar, *gen = bar + 1;
        unsigned g, old;
        asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(g) : "l"(gen) : "memory");
        asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(count) : "memory");
        int good = 1;
        if (old + 1u == gridDim.x + (unsigned)extra) {
            asm volatile("st.relaxed.gpu.global.u32 [%0], 0;" ::"l"(count) : "memory");
            asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(gen), "r"(g + 1u) : "memory");
        } else {
            for (int i = 0; ld_acquire_u32(gen) == g; ++i) {
                if (i >= spin || ((i & 1023) == 1023 && *(volatile int *)err)) {
                    good = 0;
                    atomicCAS(err, 0, 3);
                    break;
                }
            }
        }
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

template <class S, class C>
__device__ __forceinline__ void persist_record(const Shot<S, C> &s, int row, int t, int nthr)
{
#pragma unroll
    for (int comp = 0; comp < 5; ++comp) {
        const int n = s.nrec[comp];
        for (int i = t; i < n; i += nthr) s.seis[comp][(long long)row * n + i] = to_c<C>(s.f[0][comp][s.rec[comp][i]]);
    }
}

// point-source terms on fields [f0, f1) at step it, each by the thread that
// owns its cell in the phase loops (cell c = iz*nx + ix is thread c % nthr),
// in list order
template <class S, class C>
__device__ __forceinline__ void persist_terms(const Shot<S, C> &s, int it, int f0, int f1, int t, int nthr)
{
    if (it >= s.tamp_nt) return;
    for (int k = 0; k < s.nterms; ++k) {
        const int4 tm = s.terms[k];
        if (tm.x < f0 || tm.x >= f1 || ((long long)tm.z * s.nx + tm.y) % nthr != t) continue;
        S *F = s.f[0][tm.x];
        const long long o = s.origin + (long long)tm.z * s.pitch + tm.y;
        F[o] = to_s<S>(to_c<C>(F[o]) + s.tamp[(long long)k * s.tamp_nt + it]);
    }
}

// steps it0 .. it0+nsteps-1; record rows from rec_row on the steps with
// it % itrecord == 0 (any_rec); rec_sep: some receivers are on stress fields,
// so the gather gets its own phase (else it runs during the next stress
// phase, which leaves the velocities alone)
template <class S, class C, int WAVE>
__global__ void __launch_bounds__(1024, 1) persist_steps(Shot<S, C> s, int it0, int nsteps, int itrecord, int rec_row,
                                                     int any_rec, int rec_sep, unsigned *bar, int *err, int spin,
                                                     int extra)
{
    // a raised error flag stands the run down before it touches anything
    if (*(volatile int *)err) return;
    const int nthr = gridDim.x * blockDim.x, t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = s.nx;
    const long long ncell = (long long)nx * s.nz;
    const int nvel = WAVE == FD23_PSV ? 2 : 1;  // velocity fields come first
    int pending = -1;
    for (int k = 0; k < nsteps; ++k) {
        const int it = it0 + k;
        if (pending >= 0) persist_record<S, C>(s, pending, t, nthr);
        pending = -1;
        for (long long c = t; c < ncell; c += nthr) {
            const int iz = (int)(c / nx), ix = (int)(c - (long long)iz * nx);
            if (WAVE == FD23_PSV) psv_stress_cell<S, C>(s, it, ix, iz);
            else sh_stress_cell<S, C>(s, it, ix, iz);
        }
        persist_terms<S, C>(s, it, nvel, 5, t, nthr);
        if (!grid_barrier(bar, err, spin, extra)) return;
        // SH: the free-surface stress image Tz(x,0) = -Tz(x,1) after the
        // source (SH/fd/cu_fd.cu:226; post_stress_2p) is taken inside the
        // velocity update (IMG), which saves a barrier
        persist_terms<S, C>(s, it, 0, nvel, t, nthr);
        for (long long c = t; c < ncell; c += nthr) {
            const int iz = (int)(c / nx), ix = (int)(c - (long long)iz * nx);
            if (WAVE == FD23_PSV) psv_velocity_cell<S, C>(s, it, ix, iz);
            else sh_velocity_cell<S, C, true>(s, it, ix, iz);
        }
        if (!grid_barrier(bar, err, spin, extra)) return;
        if (any_rec && it % itrecord == 0) {
            if (rec_sep) {
                persist_record<S, C>(s, rec_row, t, nthr);
                if (!grid_barrier(bar, err, spin, extra)) return;
            } else {
                pending = rec_row;
            }
            ++rec_row;
        }
    }
    if (pending >= 0) persist_record<S, C>(s, pending, t, nthr);
}

}  // namespace

template <class S, class C>
int launch_persist(const Shot<S, C> &s, int wave, int it0, int nsteps, int itrecord, int rec_row, int any_rec,
                   unsigned *bar, int *err, cudaStream_t st, bool unreachable_barrier)
{
    void (*k)(Shot<S, C>, int, int, int, int, int, int, unsigned *, int *, int, int) =
        wave == FD23_PSV ? persist_steps<S, C, FD23_PSV> : persist_steps<S, C, FD23_SH>;
    int spin = kBarSpin, extra = 0;
    if (unreachable_barrier) {
        spin = 1 << 14;  // about 10 ms
        extra = 1;
    }
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 1024, 0) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        return FD23_ERR_CUDA;
    }
    const long long cells = (long long)s.nx * s.nz;
    const int blocks = (int)std::max<long long>(1, std::min<long long>((long long)sms * per_sm, (cells + 1023) / 1024));
    int rec_sep = 0;
    for (int c = (wave == FD23_PSV ? 2 : 1); c < 5; ++c) rec_sep |= s.nrec[c] > 0;
    if (cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), st) != cudaSuccess) return FD23_ERR_CUDA;
    void *args[] = {(void *)&s, &it0, &nsteps, &itrecord, &rec_row, &any_rec, &rec_sep, &bar, &err, &spin, &extra};
    const cudaError_t e = cudaLaunchCooperativeKernel((const void *)k, dim3(blocks), dim3(1024), args, 0, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return FD23_ERR_CUDA;
    }
    return FD23_OK;
}

template <class S, class C>
__global__ void record_kernel(Shot<S, C> s, int par, int rec_index)
{
    // PD/record/cu_record.cu:138-148: rec[i] = F[rx[i] + rz[i]*nx], for every
    // wavefield that has receivers
#pragma unroll
    for (int comp = 0; comp < 5; ++comp) {
        const int n = s.nrec[comp];
        const S *F = par ? s.f[1][comp] : s.f[0][comp];
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            s.seis[comp][(long long)rec_index * n + i] = to_c<C>(F[s.rec[comp][i]]);
    }
}

template <class S, class C>
int launch_record(const Shot<S, C> &s, int par, int rec_index, cudaStream_t st)
{
    int n = 0;
    for (int c = 0; c < 5; ++c) n = s.nrec[c] > n ? s.nrec[c] : n;
    if (n <= 0) return FD23_OK;
    record_kernel<S, C><<<(n + 255) / 256, 256, 0, st>>>(s, par, rec_index);
    return cudaPeekAtLastError() == cudaSuccess ? FD23_OK : FD23_ERR_CUDA;
}

template <class S, class C>
int launch_step_twopass(const Shot<S, C> &s, int wave, int it, cudaStream_t st)
{
    const dim3 blk(32, 8), grd((s.nx + 31) / 32, (s.nz + 7) / 8);
    if (wave == FD23_PSV) {
        psv_stress_2p<S, C><<<grd, blk, 0, st>>>(s, it);
        if (s.nterms > 0 && it < s.tamp_nt) post_stress_2p<S, C><<<1, 32, 0, st>>>(s, it, 0);
        if (s.box.on) {
            const int rc = launch_box_ring<S, C>(s, 0, 1, st);  // stresses, after the source
            if (rc) return rc;
        }
        psv_velocity_2p<S, C><<<grd, blk, 0, st>>>(s, it);
    } else {
        sh_stress_2p<S, C><<<grd, blk, 0, st>>>(s, it);
        post_stress_2p<S, C><<<1, 256, 0, st>>>(s, it, 1);
        sh_velocity_2p<S, C><<<grd, blk, 0, st>>>(s, it);
    }
    return cudaPeekAtLastError() == cudaSuccess ? FD23_OK : FD23_ERR_CUDA;
}

// FP64 energy watchdog: sum of squares over every stored wavefield element
// (the padding is zero) and a NaN/Inf flag.
template <class S, class C>
__global__ void norm2_kernel(Shot<S, C> s, int par, int nfields, long long elems, double *out)
{
    double acc = 0.0;
    int bad = 0;
    for (int f = 0; f < nfields; ++f) {
        const S *F = s.f[par][f];
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < elems;
             i += (long long)gridDim.x * blockDim.x) {
            const double v = (double)to_c<C>(F[i]);
            if (!isfinite(v)) bad = 1;
            else acc += v * v;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        acc += __shfl_down_sync(0xffffffffu, acc, o);
        bad |= __shfl_down_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&out[0], acc);
        if (bad) out[1] = 1.0;
    }
}

template <class S, class C>
int launch_norm2(const Shot<S, C> &s, int par, int nfields, long long elems, double *dev_out,
                 cudaStream_t st)
{
    if (cudaMemsetAsync(dev_out, 0, 2 * sizeof(double), st) != cudaSuccess) return FD23_ERR_CUDA;
    norm2_kernel<S, C><<<512, 256, 0, st>>>(s, par, nfields, elems, dev_out);
    return cudaPeekAtLastError() == cudaSuccess ? FD23_OK : FD23_ERR_CUDA;
}

#define FD23_INST(S, C)                                                                    \
    template int launch_step_twopass<S, C>(const Shot<S, C> &, int, int, cudaStream_t);   \
    template int launch_norm2<S, C>(const Shot<S, C> &, int, int, long long, double *, cudaStream_t); \
    template int launch_record<S, C>(const Shot<S, C> &, int, int, cudaStream_t);                 \
    template int launch_persist<S, C>(const Shot<S, C> &, int, int, int, int, int, int, unsigned *, int *, \
                                      cudaStream_t, bool);
FD23_INST(float, float)
FD23_INST(double, double)
FD23_INST(__nv_bfloat16, float)
FD23_INST(__half, float)
#undef FD23_INST

}  // namespace fd23
