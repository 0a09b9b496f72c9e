// Fused single-pass sweep for P-SV and SH on sm_103a.
//
// One launch advances every cell one full time step (stress update, point
// source, velocity update) and reads/writes each wavefield once, instead of
// the reference's two launches (PD/fd/cu_fd.cu:209-501, SH/fd/cu_fd.cu:77-288)
// plus host round trips for the source (PD/point_source/cu_point_source.cu)
// and receivers (PD/record/cu_record.cu:154).
//
// Data flow of one CTA (4 warps x WX; every thread owns 4 adjacent cells):
//   * The CTA works through a list of strips: output columns [x0, x0+TX),
//     rows [z0, z1).  It marches down in blocks of 4 rows.  Iteration i
//     updates the stress of rows z0-4+4i .. z0-1+4i on TX+8 columns (4 halo
//     columns each side, recomputed rather than exchanged) and the velocity of
//     rows z0-8+4i .. z0-5+4i on the TX output columns, so the velocity front
//     trails the stress front by exactly the 4 rows its z-stencil needs.
//   * Rows of the stencil inputs (U, W or V) stream into a ring of NUW 4-row
//     blocks; rows of the point-wise operands (old stresses, material) into
//     NPW stages.  Both are filled with 1-D bulk async copies
//     (cp.async.bulk ... mbarrier::complete_tx) issued by warp 0, two
//     iterations ahead of use, and consumed after an mbarrier wait.
//   * Updated stresses (after the point source) go to a 3-block smem ring that
//     feeds the velocity stencil, and straight to HBM.
//   * Wavefields and memory variables are ping-pong buffers (read set `par`,
//     write set 1-par), so the recomputed halo columns and rows of one CTA
//     never observe another CTA's new values.
//   * All arrays use the zero-padded layout of fd23_internal.h, so every row
//     copy is in bounds and 16-byte aligned and the zero halo of the
//     reference needs no test.
//
// Arithmetic per cell is the canonical sequence of fd23_device.cuh, which is
// bit-identical to the CPU oracle and to the two-pass kernels.
#include <cstdio>

#include "fd23_device.cuh"
#include "fd23_kernels.h"

namespace fd23 {

namespace {

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier + 1-D bulk async copy (TMA engine)
__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait: gives up after ~2 s, sets the error flag and returns false.
__device__ __noinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int *err_flag)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t n = 0;; ++n) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((n & 255u) == 255u && globaltimer_ns() - t0 > 2000000000ull) {
            if (err_flag) atomicExch(err_flag, 1);
            return false;
        }
    }
}

// ---------------------------------------------------------------------------
// vector access of 4 consecutive elements (16 B for float, 32 B for double,
// 8 B for 16-bit types); addresses are aligned by construction
template <class S, class C>
struct Vec4;
template <>
struct Vec4<float, float> {
    static __device__ __forceinline__ void ld(const float *p, float v[4])
    {
        const float4 t = *reinterpret_cast<const float4 *>(p);
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    }
    static __device__ __forceinline__ void st(float *p, const float v[4])
    {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
};
template <>
struct Vec4<double, double> {
    static __device__ __forceinline__ void ld(const double *p, double v[4])
    {
        const double2 a = reinterpret_cast<const double2 *>(p)[0];
        const double2 b = reinterpret_cast<const double2 *>(p)[1];
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    }
    static __device__ __forceinline__ void st(double *p, const double v[4])
    {
        reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
        reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
    }
};
template <class H>
struct Vec4Half {
    static __device__ __forceinline__ void ld(const H *p, float v[4])
    {
        const uint2 t = *reinterpret_cast<const uint2 *>(p);
        H h[4];
        memcpy(h, &t, 8);
#pragma unroll
        for (int e = 0; e < 4; ++e) v[e] = to_c<float>(h[e]);
    }
    static __device__ __forceinline__ void st(H *p, const float v[4])
    {
        H h[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) h[e] = to_s<H>(v[e]);
        uint2 t;
        memcpy(&t, h, 8);
        *reinterpret_cast<uint2 *>(p) = t;
    }
};
template <>
struct Vec4<__nv_bfloat16, float> : Vec4Half<__nv_bfloat16> {};
template <>
struct Vec4<__half, float> : Vec4Half<__half> {};

// round C values through storage S (what a store followed by a load gives)
template <class S, class C>
__device__ __forceinline__ C through(C v) { return to_c<C>(to_s<S>(v)); }

// ---------------------------------------------------------------------------
template <class S, class C, int WAVE, int WX>
struct Cfg {
    static constexpr bool PSV = (WAVE == FD23_PSV);
    static constexpr int NTH = 128 * WX;       // threads (4 row groups x 32*WX)
    static constexpr int SW = 128 * WX;        // stress columns per strip
    static constexpr int TX = SW - 8;          // output columns per strip
    static constexpr int UWW = SW + 8;         // stencil-input row width
    static constexpr int PWOFF = sizeof(S) == 2 ? 4 : 0;  // keeps 16-byte alignment
    static constexpr int PWW = SW + 2 * PWOFF; // point-wise row width
    static constexpr int NV = PSV ? 2 : 1;     // stencil inputs of the stress update
    static constexpr int NT = PSV ? 3 : 2;     // stresses
    static constexpr int NMS = PSV ? 3 : 2;    // stress-update material
    static constexpr int NMV = PSV ? 2 : 1;    // velocity-update material
    static constexpr int NPF = NT + NMS + NMV; // point-wise fields per row
    static constexpr int NUW = 5, NPW = 3, NTR = 3;
    static constexpr int UW_ELEMS = NUW * 4 * NV * UWW;
    static constexpr int PW_ELEMS = NPW * 4 * NPF * PWW;
    static constexpr int TR_ELEMS = NTR * 4 * NT * SW;
    static constexpr int MAX_ITEMS = 8;
    static constexpr int MAX_TERMS = 16;
    static constexpr size_t SMEM = (((size_t)(UW_ELEMS + PW_ELEMS + TR_ELEMS) * sizeof(S) + 15) & ~(size_t)15) + 256 +
                                   MAX_ITEMS * sizeof(int4) + MAX_TERMS * sizeof(int4) * MAX_ITEMS;
};

struct ItemInfo {
    int x0, z0, z1, niter;  // rows [z0, z1), niter = (z1-z0)/4 + 2
};

template <class S, class C, int WAVE, int WX>
__global__ void __launch_bounds__(Cfg<S, C, WAVE, WX>::NTH, 1)
    fused_step(Shot<S, C> sh, const WorkItem *__restrict__ items, const int *__restrict__ item_off,
               int par, int it, int rec_index, int *err_flag)
{
    using K = Cfg<S, C, WAVE, WX>;
    constexpr bool PSV = K::PSV;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    S *uw_s = reinterpret_cast<S *>(smem_raw);
    S *pw_s = uw_s + K::UW_ELEMS;
    S *tr_s = pw_s + K::PW_ELEMS;
    // NUW + NPW barriers, 16-byte aligned after the rings
    uint64_t *bars = reinterpret_cast<uint64_t *>(
        smem_raw + ((((size_t)K::UW_ELEMS + K::PW_ELEMS + K::TR_ELEMS) * sizeof(S) + 15) & ~(size_t)15));
    uint64_t *bar_uw = bars, *bar_pw = bars + K::NUW;
    ItemInfo *info = reinterpret_cast<ItemInfo *>(bars + 16);
    int4 *tlist = reinterpret_cast<int4 *>(info + K::MAX_ITEMS);  // per item: local source terms
    __shared__ int tcount[K::MAX_ITEMS];

    // an earlier launch gave up on a wait: do nothing until the host resets
    if (err_flag && *(volatile int *)err_flag) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = warp / WX;                      // row group 0..3
    const int q = (warp % WX) * 32 + lane;        // 4-cell column chunk
    const int nx = sh.nx, nz = sh.nz, npml = sh.npml, pitch = sh.pitch;
    const long long origin = sh.origin;

    // ---- receivers of the previous step (buffer set `par` is read-only here) ----
    if (rec_index >= 0) {
#pragma unroll
        for (int comp = 0; comp < 2; ++comp) {
            const int n = sh.nrec[comp];
            for (int r = blockIdx.x * K::NTH + tid; r < n; r += gridDim.x * K::NTH)
                sh.seis[comp][(long long)rec_index * n + r] = to_c<C>((comp == 0 ? sh.f[par][0] : sh.f[par][1])[sh.rec[comp][r]]);
        }
    }

    const int ibeg = item_off[blockIdx.x], iend = item_off[blockIdx.x + 1];
    const int nitems = min(iend - ibeg, K::MAX_ITEMS);
    if (nitems <= 0) return;

    // ---- per-item set-up: geometry and the source terms inside its stress region ----
    if (tid < nitems) {
        const WorkItem w = items[ibeg + tid];
        info[tid] = ItemInfo{w.x0, w.z0, w.z1, (w.z1 - w.z0) / 4 + 2};
        int cnt = 0;
        if (it < sh.tamp_nt) {
            for (int t = 0; t < sh.nterms && cnt < K::MAX_TERMS; ++t) {
                const int4 tm = sh.terms[t];
                if (tm.y >= w.x0 - 4 && tm.y < w.x0 - 4 + K::SW && tm.z >= w.z0 - 4 && tm.z < w.z1 + 4)
                    tlist[tid * K::MAX_TERMS + cnt++] = make_int4(tm.x, tm.y, tm.z, t);
            }
        }
        tcount[tid] = cnt;
    }
    if (tid == 0) {
        for (int b = 0; b < K::NUW + K::NPW; ++b) mbar_init(&bars[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    // flat iteration space over the CTA's items
    int total_iters = 0;
    for (int k = 0; k < nitems; ++k) total_iters += info[k].niter;
    // stencil-input stream: item k contributes niter+2 row blocks
    int total_uw = 0;
    for (int k = 0; k < nitems; ++k) total_uw += info[k].niter + 2;

    // read / write pointers selected once (compile-time indices only: a
    // runtime index into the parameter arrays would force a local copy)
    const S *rd[5];
    S *wr[5];
    const C *prd[8];
    C *pwr[8];
#pragma unroll
    for (int f = 0; f < 5; ++f) {
        rd[f] = par ? sh.f[1][f] : sh.f[0][f];
        wr[f] = par ? sh.f[0][f] : sh.f[1][f];
    }
#pragma unroll
    for (int f = 0; f < 8; ++f) {
        prd[f] = par ? sh.psi[1][f] : sh.psi[0][f];
        pwr[f] = par ? sh.psi[0][f] : sh.psi[1][f];
    }
    // base pointer of point-wise field `fidx` (runtime), chosen by unrolled compare
    auto pw_base = [=](int fidx) -> const S * {
        const S *b = rd[K::NV];
#pragma unroll
        for (int f = 0; f < K::NPF; ++f) {
            const S *c = f < K::NT ? rd[K::NV + f] : sh.mat[f - K::NT];
            if (f == fidx) b = c;
        }
        return b;
    };

    // ---- producer: issue stream element `e` of the stencil inputs ----
    auto issue_uw = [=](int e) {
        int k = 0, base = 0;
        while (k < nitems - 1 && e >= base + info[k].niter + 2) { base += info[k].niter + 2; ++k; }
        const int b = e - base;
        const ItemInfo &I = info[k];
        const int slot = e % K::NUW;
        const int r0 = I.z0 - 8 + 4 * b;
        constexpr uint32_t ROWB = K::UWW * sizeof(S);
        if (lane == 0) mbar_arrive_expect_tx(&bar_uw[slot], ROWB * 4 * K::NV);
        __syncwarp();
        if (lane < 4 * K::NV) {
            const int rr = lane & 3, v = lane >> 2;
            const S *src = (v == 0 ? rd[0] : rd[K::NV - 1]) + origin + (long long)(r0 + rr) * pitch + (I.x0 - 8);
            S *dst = uw_s + ((size_t)(slot * 4 + rr) * K::NV + v) * K::UWW;
            bulk_g2s(dst, src, ROWB, &bar_uw[slot]);
        }
    };
    // ---- producer: point-wise operands of flat iteration `e` ----
    auto issue_pw = [=](int e) {
        int k = 0, base = 0;
        while (k < nitems - 1 && e >= base + info[k].niter) { base += info[k].niter; ++k; }
        const int i = e - base;
        const ItemInfo &I = info[k];
        const int slot = e % K::NPW;
        constexpr uint32_t ROWB = K::PWW * sizeof(S);
        if (lane == 0) mbar_arrive_expect_tx(&bar_pw[slot], ROWB * 4 * K::NPF);
        __syncwarp();
        for (int c = lane; c < 4 * K::NPF; c += 32) {
            const int rr = c & 3, fidx = c >> 2;
            // old stresses and stress-update material on stress rows,
            // velocity-update material on velocity rows
            const S *base_ptr = pw_base(fidx);
            const int row = (fidx < K::NT + K::NMS ? I.z0 - 4 : I.z0 - 8) + 4 * i + rr;
            const S *src = base_ptr + origin + (long long)row * pitch + (I.x0 - 4 - K::PWOFF);
            S *dst = pw_s + ((size_t)(slot * K::NPF + fidx) * 4 + rr) * K::PWW;
            bulk_g2s(dst, src, ROWB, &bar_pw[slot]);
        }
    };

    int uw_issued = 0, pw_issued = 0;
    // initial fill: NUW-1 stencil blocks and NPW-1 point-wise stages
    if (warp == 0) {
        for (; uw_issued < min(K::NUW - 1, total_uw); ++uw_issued) issue_uw(uw_issued);
        for (; pw_issued < min(K::NPW - 1, total_iters); ++pw_issued) issue_pw(pw_issued);
    }

    bool ok = true;
    int gflat = 0, uw_base = 0;
    const int bsel = 1 - par;
    const C *cp = sh.cpml;
    const int B = sh.cpml_blk;

    for (int k = 0; k < nitems && ok; ++k) {
        const ItemInfo I = info[k];
        const int ntl = tcount[k];
        const int4 *tl = tlist + k * K::MAX_TERMS;
        for (int i = 0; i < I.niter; ++i, ++gflat) {
            // ---- refill: stream elements whose ring slot has been released ----
            if (warp == 0) {
                while (uw_issued < total_uw && uw_issued < uw_base + i + K::NUW) issue_uw(uw_issued++);
                while (pw_issued < total_iters && pw_issued < gflat + K::NPW) issue_pw(pw_issued++);
            }
            // ---- wait for stencil blocks i..i+2 and point-wise stage of this iteration ----
            for (int b = i; b < i + 3 && ok; ++b) {
                const int e = uw_base + b;
                ok = mbar_wait_bounded(&bar_uw[e % K::NUW], (uint32_t)((e / K::NUW) & 1), err_flag);
            }
            if (ok) ok = mbar_wait_bounded(&bar_pw[gflat % K::NPW], (uint32_t)((gflat / K::NPW) & 1), err_flag);
            // every thread takes the same exit decision before the next barrier
            ok = __syncthreads_and(ok) != 0;
            if (!ok) break;

            const S *pws = pw_s + (size_t)(gflat % K::NPW) * K::NPF * 4 * K::PWW;
            // address of stencil input v, absolute row r, stored column index col (0 = x0-8)
            auto uwrow = [=](int v, int r) -> const S * {
                const int e = uw_base + ((r - (I.z0 - 8)) >> 2);
                return uw_s + ((size_t)((e % K::NUW) * 4 + ((r - (I.z0 - 8)) & 3)) * K::NV + v) * K::UWW;
            };
            // stress ring row (absolute row r of this item)
            auto trrow = [=](int f, int r) -> S * {
                const int ii = (r - (I.z0 - 4)) >> 2;  // iteration that produced row r
                const int slot = (gflat - i + ii) % K::NTR;
                return tr_s + ((size_t)(slot * 4 + ((r - (I.z0 - 4)) & 3)) * K::NT + f) * K::SW;
            };

            // ================= stress phase: row j, cells x .. x+3 =================
            {
                const int j = I.z0 - 4 + 4 * i + g;
                const int x = I.x0 - 4 + 4 * q;
                C tnew[K::NT][4];
                const bool inrow = (j >= 0 && j < nz);
                // point-wise operands
                C told[K::NT][4], ms[K::NMS][4];
#pragma unroll
                for (int f = 0; f < K::NT; ++f)
                    Vec4<S, C>::ld(pws + ((size_t)f * 4 + g) * K::PWW + K::PWOFF + 4 * q, told[f]);
#pragma unroll
                for (int m = 0; m < K::NMS; ++m)
                    Vec4<S, C>::ld(pws + ((size_t)(K::NT + m) * 4 + g) * K::PWW + K::PWOFF + 4 * q, ms[m]);

                const int col = 4 * q + 4;  // stored column of cell x in stencil rows
                if constexpr (PSV) {
                    C ux[4], uz[4], wx[4], wz[4];
                    {
                        C h[12], zc[9][4];
                        const S *r0 = uwrow(0, j);
                        Vec4<S, C>::ld(r0 + col - 4, h);
                        Vec4<S, C>::ld(r0 + col, h + 4);
                        Vec4<S, C>::ld(r0 + col + 4, h + 8);
#pragma unroll
                        for (int d = -4; d <= 3; ++d)
                            if (d != 0) Vec4<S, C>::ld(uwrow(0, j + d) + col, zc[d + 4]);
#pragma unroll
                        for (int e = 0; e < 4; ++e) zc[4][e] = h[4 + e];
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int ix = x + e;
                            C c0 = Coef4<C>::c0, c1 = Coef4<C>::c1, c2 = Coef4<C>::c2, c3 = Coef4<C>::c3;
                            if (!(ix >= 4 && ix <= nx - 5 && j >= 4 && j <= nz - 5)) {
                                const int o = (ix >= 0 && ix < nx && inrow) ? stencil_order(ix, j, nx, nz) : 4;
                                c0 = Coef<C>::get(o, 0); c1 = Coef<C>::get(o, 1);
                                c2 = Coef<C>::get(o, 2); c3 = Coef<C>::get(o, 3);
                            }
                            ux[e] = comb<C>(c0, c1, c2, c3, h[4 + e] - h[3 + e], h[5 + e] - h[2 + e],
                                            h[6 + e] - h[1 + e], h[7 + e] - h[e]);
                            uz[e] = comb<C>(c0, c1, c2, c3, zc[4][e] - zc[3][e], zc[5][e] - zc[2][e],
                                            zc[6][e] - zc[1][e], zc[7][e] - zc[0][e]);
                        }
                    }
                    {
                        C h[12], zc[9][4];
                        const S *r0 = uwrow(1, j);
                        Vec4<S, C>::ld(r0 + col - 4, h);
                        Vec4<S, C>::ld(r0 + col, h + 4);
                        Vec4<S, C>::ld(r0 + col + 4, h + 8);
#pragma unroll
                        for (int d = -3; d <= 4; ++d)
                            if (d != 0) Vec4<S, C>::ld(uwrow(1, j + d) + col, zc[d + 4]);
#pragma unroll
                        for (int e = 0; e < 4; ++e) zc[4][e] = h[4 + e];
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int ix = x + e;
                            C c0 = Coef4<C>::c0, c1 = Coef4<C>::c1, c2 = Coef4<C>::c2, c3 = Coef4<C>::c3;
                            if (!(ix >= 4 && ix <= nx - 5 && j >= 4 && j <= nz - 5)) {
                                const int o = (ix >= 0 && ix < nx && inrow) ? stencil_order(ix, j, nx, nz) : 4;
                                c0 = Coef<C>::get(o, 0); c1 = Coef<C>::get(o, 1);
                                c2 = Coef<C>::get(o, 2); c3 = Coef<C>::get(o, 3);
                            }
                            wx[e] = comb<C>(c0, c1, c2, c3, h[5 + e] - h[4 + e], h[6 + e] - h[3 + e],
                                            h[7 + e] - h[2 + e], h[8 + e] - h[1 + e]);
                            wz[e] = comb<C>(c0, c1, c2, c3, zc[5][e] - zc[4][e], zc[6][e] - zc[3][e],
                                            zc[7][e] - zc[2][e], zc[8][e] - zc[1][e]);
                        }
                    }
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int ix = x + e;
                        if (!inrow || ix < 0 || ix >= nx) {
                            tnew[0][e] = tnew[1][e] = tnew[2][e] = (C)0;
                            continue;
                        }
                        const bool own = ix >= I.x0 && ix < I.x0 + K::TX && j >= I.z0 && j < I.z1;
                        const C lam = ms[0][e], mu = ms[1][e], mua = ms[2][e];
                        const C gam = lam + (C)2 * mu;
                        C txx = told[0][e], txz = told[1][e], tzz = told[2][e];
                        if (ix < npml || ix >= nx - npml) {
                            const long long p = ix < npml ? (long long)ix + (long long)j * 2 * npml
                                                          : (long long)npml + nx - 1 - ix + (long long)j * 2 * npml;
                            const C pu = fmaC<C>(cp[2 * nx + ix], prd[2][p], cp[B + 2 * nx + ix] * ux[e]);
                            const C t = fmaC<C>(ux[e], cp[2 * B + 2 * nx + ix], pu);
                            txx = fmaC<C>(gam, t, txx);
                            tzz = fmaC<C>(lam, t, tzz);
                            const C pw = fmaC<C>(cp[3 * nx + ix], prd[3][p], cp[B + 3 * nx + ix] * wx[e]);
                            txz = fmaC<C>(mua, fmaC<C>(wx[e], cp[2 * B + 3 * nx + ix], pw), txz);
                            if (own) { pwr[2][p] = pu; pwr[3][p] = pw; }
                        } else if (j != 0) {
                            txx = fmaC<C>(gam, ux[e], txx);
                            tzz = fmaC<C>(lam, ux[e], tzz);
                            txz = fmaC<C>(mua, wx[e], txz);
                        }
                        const bool top = j < npml && sh.topabsorb;
                        if (top || j >= nz - npml) {
                            const long long p = top ? (long long)j * nx + ix : (long long)(npml + nz - 1 - j) * nx + ix;
                            const int zb = 4 * nx;
                            const C pw = fmaC<C>(cp[zb + 3 * nz + j], prd[7][p], cp[B + zb + 3 * nz + j] * wz[e]);
                            const C t = fmaC<C>(wz[e], cp[2 * B + zb + 3 * nz + j], pw);
                            txx = fmaC<C>(lam, t, txx);
                            tzz = fmaC<C>(gam, t, tzz);
                            const C pu = fmaC<C>(cp[zb + 2 * nz + j], prd[6][p], cp[B + zb + 2 * nz + j] * uz[e]);
                            txz = fmaC<C>(mua, fmaC<C>(uz[e], cp[2 * B + zb + 2 * nz + j], pu), txz);
                            if (own) { pwr[7][p] = pw; pwr[6][p] = pu; }
                        } else if (j == 0) {
                            txx = fmaC<C>((C)2 * mu, ux[e], txx);
                            tzz = (C)0;
                            txz = (C)0;
                        } else {
                            txx = fmaC<C>(lam, wz[e], txx);
                            tzz = fmaC<C>(gam, wz[e], tzz);
                            txz = fmaC<C>(mua, uz[e], txz);
                        }
                        // storage order of stresses: Txx, Txz, Tzz
                        tnew[0][e] = txx;
                        tnew[1][e] = txz;
                        tnew[2][e] = tzz;
                    }
                } else {
                    // SH stress: dxV = D+x V, dzV = D-z V (SH/fd/cu_fd.cu:77-171)
                    C dxv[4], dzv[4];
                    {
                        C h[12], zc[9][4];
                        const S *r0 = uwrow(0, j);
                        Vec4<S, C>::ld(r0 + col - 4, h);
                        Vec4<S, C>::ld(r0 + col, h + 4);
                        Vec4<S, C>::ld(r0 + col + 4, h + 8);
#pragma unroll
                        for (int d = -4; d <= 3; ++d)
                            if (d != 0) Vec4<S, C>::ld(uwrow(0, j + d) + col, zc[d + 4]);
#pragma unroll
                        for (int e = 0; e < 4; ++e) zc[4][e] = h[4 + e];
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int ix = x + e;
                            C c0 = Coef4<C>::c0, c1 = Coef4<C>::c1, c2 = Coef4<C>::c2, c3 = Coef4<C>::c3;
                            if (!(ix >= 4 && ix <= nx - 5 && j >= 4 && j <= nz - 5)) {
                                const int o = (ix >= 0 && ix < nx && inrow) ? stencil_order(ix, j, nx, nz) : 4;
                                c0 = Coef<C>::get(o, 0); c1 = Coef<C>::get(o, 1);
                                c2 = Coef<C>::get(o, 2); c3 = Coef<C>::get(o, 3);
                            }
                            dxv[e] = comb<C>(c0, c1, c2, c3, h[5 + e] - h[4 + e], h[6 + e] - h[3 + e],
                                             h[7 + e] - h[2 + e], h[8 + e] - h[1 + e]);
                            dzv[e] = comb<C>(c0, c1, c2, c3, zc[4][e] - zc[3][e], zc[5][e] - zc[2][e],
                                             zc[6][e] - zc[1][e], zc[7][e] - zc[0][e]);
                        }
                    }
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int ix = x + e;
                        if (!inrow || ix < 0 || ix >= nx) {
                            tnew[0][e] = tnew[1][e] = (C)0;
                            continue;
                        }
                        const bool own = ix >= I.x0 && ix < I.x0 + K::TX && j >= I.z0 && j < I.z1;
                        C tx = told[0][e], tz = told[1][e];
                        const bool xp = ix < npml || ix >= nx - npml;
                        const bool top = j < npml && sh.topabsorb;
                        const bool zp = top || j >= nz - npml;
                        const long long px = ix < npml ? (long long)ix + (long long)j * 2 * npml
                                                       : (long long)npml + nx - 1 - ix + (long long)j * 2 * npml;
                        const long long pz = top ? (long long)j * nx + ix : (long long)(npml + nz - 1 - j) * nx + ix;
                        if (ix == 0 || ix >= nx - 1 || j >= nz - 1) {
                            // skipped by the reference: carry the old values over
                            if (own && xp) pwr[1][px] = prd[1][px];
                            if (own && zp) pwr[3][pz] = prd[3][pz];
                        } else {
                            const C mux = ms[0][e], muz = ms[1][e];
                            if (xp) {
                                const C a = fmaC<C>(cp[nx + ix], prd[1][px], cp[B + nx + ix] * dxv[e]);
                                if (own) pwr[1][px] = a;
                                tx = fmaC<C>(mux, fmaC<C>(dxv[e], cp[2 * B + nx + ix], a), tx);
                            } else {
                                tx = fmaC<C>(mux, dxv[e], tx);
                            }
                            if (zp) {
                                const int zb = 2 * nx;
                                const C a = fmaC<C>(cp[zb + nz + j], prd[3][pz], cp[B + zb + nz + j] * dzv[e]);
                                if (own) pwr[3][pz] = a;
                                tz = fmaC<C>(muz, fmaC<C>(dzv[e], cp[2 * B + zb + nz + j], a), tz);
                            } else {
                                tz = fmaC<C>(muz, dzv[e], tz);
                            }
                        }
                        tnew[0][e] = tx;
                        tnew[1][e] = tz;
                    }
                }
                // ---- point source (terms in list order), then storage rounding ----
                if (ntl > 0) {
                    for (int t = 0; t < ntl; ++t) {
                        const int4 tm = tl[t];  // (field, ix, iz, term index)
                        const int fi = tm.x - K::NV;
                        if (fi >= 0 && tm.z == j && tm.y >= x && tm.y < x + 4) {
                            const C a = sh.tamp[(long long)tm.w * sh.tamp_nt + it];
#pragma unroll
                            for (int f = 0; f < K::NT; ++f)
#pragma unroll
                                for (int e = 0; e < 4; ++e)
                                    if (f == fi && e == tm.y - x) tnew[f][e] = through<S, C>(tnew[f][e]) + a;
                        }
                    }
                }
                // write the stress ring and, for owned cells, HBM
#pragma unroll
                for (int f = 0; f < K::NT; ++f) {
                    C v[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) v[e] = tnew[f][e];
                    Vec4<S, C>::st(trrow(f, j) + 4 * q, v);
                }
                if (inrow && j >= I.z0 && j < I.z1 && q >= 1 && q <= 32 * WX - 2) {
                    const long long o = origin + (long long)j * pitch + x;
                    if (x + 3 < nx) {
#pragma unroll
                        for (int f = 0; f < K::NT; ++f) {
                            C v[4];
#pragma unroll
                            for (int e = 0; e < 4; ++e) v[e] = tnew[f][e];
                            Vec4<S, C>::st(wr[K::NV + f] + o, v);
                        }
                    } else {
#pragma unroll
                        for (int f = 0; f < K::NT; ++f)
#pragma unroll
                            for (int e = 0; e < 4; ++e)
                                if (x + e < nx) wr[K::NV + f][o + e] = to_s<S>(tnew[f][e]);
                    }
                }
            }
            __syncthreads();

            if constexpr (!PSV) {
                // free-surface stress image Tz(x,0) = -Tz(x,1), SH/fd/cu_fd.cu:226,
                // applied once rows 0 and 1 of the new stresses exist
                if (I.z0 == 0 && i == 1) {
                    for (int c = tid; c < K::SW; c += K::NTH) {
                        S *r0 = trrow(1, 0), *r1 = trrow(1, 1);
                        const C v = -to_c<C>(r1[c]);
                        r0[c] = to_s<S>(v);
                        const int ix = I.x0 - 4 + c;
                        if (ix >= I.x0 && ix < I.x0 + K::TX && ix < nx && nz > 1)
                            wr[K::NV + 1][origin + ix] = to_s<S>(v);
                    }
                    __syncthreads();
                }
            }

            // ================= velocity phase: row a, cells x .. x+3 =================
            {
                const int a = I.z0 - 8 + 4 * i + g;
                const int x = I.x0 - 4 + 4 * q;
                if (a >= I.z0 && a < nz && q >= 1 && q <= 32 * WX - 2 && x < nx) {
                    C mv[K::NMV][4];
#pragma unroll
                    for (int m = 0; m < K::NMV; ++m)
                        Vec4<S, C>::ld(pws + ((size_t)(K::NT + K::NMS + m) * 4 + g) * K::PWW + K::PWOFF + 4 * q, mv[m]);
                    const int colv = 4 * q + 4;
                    C vold[K::NV][4];
#pragma unroll
                    for (int v = 0; v < K::NV; ++v) Vec4<S, C>::ld(uwrow(v, a) + colv, vold[v]);
                    const int cs = 4 * q;  // stored column of cell x in stress rows
                    C vnew[K::NV][4];
                    if constexpr (PSV) {
                        C dxTxx[4], dzTzz[4], dxTxz[4], dzTxz[4];
                        C hxx[12], hxz[12], zzz[9][4], zxz[9][4];
                        {
                            const S *r = trrow(0, a);
                            Vec4<S, C>::ld(r + cs - 4, hxx);
                            Vec4<S, C>::ld(r + cs, hxx + 4);
                            Vec4<S, C>::ld(r + cs + 4, hxx + 8);
                            const S *rz = trrow(1, a);
                            Vec4<S, C>::ld(rz + cs - 4, hxz);
                            Vec4<S, C>::ld(rz + cs, hxz + 4);
                            Vec4<S, C>::ld(rz + cs + 4, hxz + 8);
#pragma unroll
                            for (int d = -4; d <= 4; ++d) {
                                if (d <= 3) Vec4<S, C>::ld(trrow(2, a + d) + cs, zzz[d + 4]);
                                if (d >= -3 && d != 0) Vec4<S, C>::ld(trrow(1, a + d) + cs, zxz[d + 4]);
                            }
#pragma unroll
                            for (int e = 0; e < 4; ++e) zxz[4][e] = hxz[4 + e];
                        }
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int ix = x + e;
                            C c0 = Coef4<C>::c0, c1 = Coef4<C>::c1, c2 = Coef4<C>::c2, c3 = Coef4<C>::c3;
                            if (!(ix >= 4 && ix <= nx - 5 && a >= 4 && a <= nz - 5)) {
                                const int o = ix < nx ? stencil_order(ix, a, nx, nz) : 4;
                                c0 = Coef<C>::get(o, 0); c1 = Coef<C>::get(o, 1);
                                c2 = Coef<C>::get(o, 2); c3 = Coef<C>::get(o, 3);
                            }
                            dxTxx[e] = comb<C>(c0, c1, c2, c3, hxx[5 + e] - hxx[4 + e], hxx[6 + e] - hxx[3 + e],
                                               hxx[7 + e] - hxx[2 + e], hxx[8 + e] - hxx[1 + e]);
                            dzTzz[e] = comb<C>(c0, c1, c2, c3, zzz[4][e] - zzz[3][e], zzz[5][e] - zzz[2][e],
                                               zzz[6][e] - zzz[1][e], zzz[7][e] - zzz[0][e]);
                            dxTxz[e] = comb<C>(c0, c1, c2, c3, hxz[4 + e] - hxz[3 + e], hxz[5 + e] - hxz[2 + e],
                                               hxz[6 + e] - hxz[1 + e], hxz[7 + e] - hxz[e]);
                            dzTxz[e] = comb<C>(c0, c1, c2, c3, zxz[5][e] - zxz[4][e], zxz[6][e] - zxz[3][e],
                                               zxz[7][e] - zxz[2][e], zxz[8][e] - zxz[1][e]);
                        }
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int ix = x + e;
                            C u = vold[0][e], w = vold[1][e];
                            if (ix >= nx) { vnew[0][e] = u; vnew[1][e] = w; continue; }
                            const C bu = mv[0][e], bw = mv[1][e];
                            if (ix < npml || ix >= nx - npml) {
                                const long long p = ix < npml ? (long long)ix + (long long)a * 2 * npml
                                                              : (long long)npml + nx - 1 - ix + (long long)a * 2 * npml;
                                const C pa = fmaC<C>(cp[ix], prd[0][p], cp[B + ix] * dxTxx[e]);
                                pwr[0][p] = pa;
                                u = fmaC<C>(bu, fmaC<C>(dxTxx[e], cp[2 * B + ix], pa), u);
                                const C pb = fmaC<C>(cp[nx + ix], prd[1][p], cp[B + nx + ix] * dxTxz[e]);
                                pwr[1][p] = pb;
                                w = fmaC<C>(bw, fmaC<C>(dxTxz[e], cp[2 * B + nx + ix], pb), w);
                            } else if (a != 0) {
                                u = fmaC<C>(bu, dxTxx[e], u);
                                w = fmaC<C>(bw, dxTxz[e], w);
                            }
                            const bool top = a < npml && sh.topabsorb;
                            if (top || a >= nz - npml) {
                                const long long p = top ? (long long)a * nx + ix : (long long)(npml + nz - 1 - a) * nx + ix;
                                const int zb = 4 * nx;
                                const C pa = fmaC<C>(cp[zb + nz + a], prd[5][p], cp[B + zb + nz + a] * dzTxz[e]);
                                const C pb = fmaC<C>(cp[zb + a], prd[4][p], cp[B + zb + a] * dzTzz[e]);
                                pwr[5][p] = pa;
                                pwr[4][p] = pb;
                                u = fmaC<C>(bu, fmaC<C>(dzTxz[e], cp[2 * B + zb + nz + a], pa), u);
                                w = fmaC<C>(bw, fmaC<C>(dzTzz[e], cp[2 * B + zb + a], pb), w);
                            } else if (a == 0) {
                                u = fmaC<C>(bu, dxTxx[e] + dzTxz[e], u);
                                w = (C)0;
                            } else {
                                u = fmaC<C>(bu, dzTxz[e], u);
                                w = fmaC<C>(bw, dzTzz[e], w);
                            }
                            vnew[0][e] = u;
                            vnew[1][e] = w;
                        }
                    } else {
                        C dxT[4], dzT[4];
                        C hx[12], zz[9][4];
                        {
                            const S *r = trrow(0, a);
                            Vec4<S, C>::ld(r + cs - 4, hx);
                            Vec4<S, C>::ld(r + cs, hx + 4);
                            Vec4<S, C>::ld(r + cs + 4, hx + 8);
#pragma unroll
                            for (int d = -3; d <= 4; ++d) Vec4<S, C>::ld(trrow(1, a + d) + cs, zz[d + 4]);
                        }
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int ix = x + e;
                            C c0 = Coef4<C>::c0, c1 = Coef4<C>::c1, c2 = Coef4<C>::c2, c3 = Coef4<C>::c3;
                            if (!(ix >= 4 && ix <= nx - 5 && a >= 4 && a <= nz - 5)) {
                                const int o = ix < nx ? stencil_order(ix, a, nx, nz) : 4;
                                c0 = Coef<C>::get(o, 0); c1 = Coef<C>::get(o, 1);
                                c2 = Coef<C>::get(o, 2); c3 = Coef<C>::get(o, 3);
                            }
                            dxT[e] = comb<C>(c0, c1, c2, c3, hx[4 + e] - hx[3 + e], hx[5 + e] - hx[2 + e],
                                             hx[6 + e] - hx[1 + e], hx[7 + e] - hx[e]);
                            dzT[e] = comb<C>(c0, c1, c2, c3, zz[5][e] - zz[4][e], zz[6][e] - zz[3][e],
                                             zz[7][e] - zz[2][e], zz[8][e] - zz[1][e]);
                        }
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int ix = x + e;
                            C v = vold[0][e];
                            if (ix >= nx) { vnew[0][e] = v; continue; }
                            // line force on V, injected before the velocity update
                            if (ntl > 0)
                                for (int t = 0; t < ntl; ++t) {
                                    const int4 tm = tl[t];
                                    if (tm.x == FD23_V && tm.z == a && tm.y == ix)
                                        v = through<S, C>(v) + sh.tamp[(long long)tm.w * sh.tamp_nt + it];
                                }
                            const C bv = mv[0][e];
                            if (ix < npml || ix >= nx - npml) {
                                const long long p = ix < npml ? (long long)ix + (long long)a * 2 * npml
                                                              : (long long)npml + nx - 1 - ix + (long long)a * 2 * npml;
                                const C pa = fmaC<C>(cp[ix], prd[0][p], cp[B + ix] * dxT[e]);
                                pwr[0][p] = pa;
                                v = fmaC<C>(bv, fmaC<C>(dxT[e], cp[2 * B + ix], pa), v);
                            } else {
                                v = fmaC<C>(bv, dxT[e], v);
                            }
                            const bool top = a < npml && sh.topabsorb;
                            if (top || a >= nz - npml) {
                                const long long p = top ? (long long)a * nx + ix : (long long)(npml + nz - 1 - a) * nx + ix;
                                const int zb = 2 * nx;
                                const C pa = fmaC<C>(cp[zb + a], prd[2][p], cp[B + zb + a] * dzT[e]);
                                pwr[2][p] = pa;
                                v = fmaC<C>(bv, fmaC<C>(dzT[e], cp[2 * B + zb + a], pa), v);
                            } else {
                                v = fmaC<C>(bv, dzT[e], v);
                            }
                            vnew[0][e] = v;
                        }
                    }
                    const long long o = origin + (long long)a * pitch + x;
                    if (x + 3 < nx) {
#pragma unroll
                        for (int v = 0; v < K::NV; ++v) Vec4<S, C>::st(wr[v] + o, vnew[v]);
                    } else {
#pragma unroll
                        for (int v = 0; v < K::NV; ++v)
#pragma unroll
                            for (int e = 0; e < 4; ++e)
                                if (x + e < nx) wr[v][o + e] = to_s<S>(vnew[v][e]);
                    }
                }
            }
            __syncthreads();
        }
        uw_base += I.niter + 2;
    }
    if (!ok && warp == 0) {
        // a wait gave up: let the copies already issued land before the CTA
        // exits (each wait is bounded again)
#pragma unroll
        for (int e = max(0, uw_issued - K::NUW); e < uw_issued; ++e)
            mbar_wait_bounded(&bar_uw[e % K::NUW], (uint32_t)((e / K::NUW) & 1), nullptr);
#pragma unroll
        for (int e = max(0, pw_issued - K::NPW); e < pw_issued; ++e)
            mbar_wait_bounded(&bar_pw[e % K::NPW], (uint32_t)((e / K::NPW) & 1), nullptr);
    }
}

template <class S, class C, int WAVE, int WX>
int launch_fused_impl(const Shot<S, C> &s, const WorkItem *items, const int *item_off, int nblocks,
                      int par, int it, int rec_index, int *err_flag, cudaStream_t st)
{
    using K = Cfg<S, C, WAVE, WX>;
    fused_step<S, C, WAVE, WX><<<nblocks, K::NTH, K::SMEM, st>>>(s, items, item_off, par, it,
                                                                   rec_index, err_flag);
    return cudaPeekAtLastError() == cudaSuccess ? FD23_OK : FD23_ERR_CUDA;
}

}  // namespace

FusedGeom fused_geom(int wave, int prec)
{
    (void)wave;
    (void)prec;
    return FusedGeom{120, 4};  // WX = 1: 128 stress columns, 120 output columns
}

template <class S, class C>
int launch_step_fused(const Shot<S, C> &s, int wave, const WorkItem *items, const int *item_off,
                      int nblocks, int par, int it, int rec_index, int *err_flag, cudaStream_t st)
{
    if (wave == FD23_PSV)
        return launch_fused_impl<S, C, FD23_PSV, 1>(s, items, item_off, nblocks, par, it, rec_index,
                                                    err_flag, st);
    return launch_fused_impl<S, C, FD23_SH, 1>(s, items, item_off, nblocks, par, it, rec_index,
                                              err_flag, st);
}

template <class S, class C, int WAVE>
static int prepare_one()
{
    using K = Cfg<S, C, WAVE, 1>;
    return cudaFuncSetAttribute(fused_step<S, C, WAVE, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)K::SMEM) == cudaSuccess
               ? FD23_OK
               : FD23_ERR_CUDA;
}

int fused_prepare(int wave, int prec)
{
    // opt in to the large dynamic shared memory on the current device
    if (wave == FD23_PSV) {
        switch (prec) {
            case FD23_F64: return prepare_one<double, double, FD23_PSV>();
            case FD23_BF16: return prepare_one<__nv_bfloat16, float, FD23_PSV>();
            case FD23_F16: return prepare_one<__half, float, FD23_PSV>();
            default: return prepare_one<float, float, FD23_PSV>();
        }
    }
    switch (prec) {
        case FD23_F64: return prepare_one<double, double, FD23_SH>();
        case FD23_BF16: return prepare_one<__nv_bfloat16, float, FD23_SH>();
        case FD23_F16: return prepare_one<__half, float, FD23_SH>();
        default: return prepare_one<float, float, FD23_SH>();
    }
}

size_t fused_smem_bytes(int wave, int prec)
{
    if (wave == FD23_PSV) {
        switch (prec) {
            case FD23_F64: return Cfg<double, double, FD23_PSV, 1>::SMEM;
            case FD23_BF16: return Cfg<__nv_bfloat16, float, FD23_PSV, 1>::SMEM;
            case FD23_F16: return Cfg<__half, float, FD23_PSV, 1>::SMEM;
            default: return Cfg<float, float, FD23_PSV, 1>::SMEM;
        }
    }
    switch (prec) {
        case FD23_F64: return Cfg<double, double, FD23_SH, 1>::SMEM;
        case FD23_BF16: return Cfg<__nv_bfloat16, float, FD23_SH, 1>::SMEM;
        case FD23_F16: return Cfg<__half, float, FD23_SH, 1>::SMEM;
        default: return Cfg<float, float, FD23_SH, 1>::SMEM;
    }
}

#define FD23_INST(S, C)                                                                            \
    template int launch_step_fused<S, C>(const Shot<S, C> &, int, const WorkItem *, const int *, \
                                         int, int, int, int, int *, cudaStream_t);
FD23_INST(float, float)
FD23_INST(double, double)
FD23_INST(__nv_bfloat16, float)
FD23_INST(__half, float)
#undef FD23_INST

}  // namespace fd23
