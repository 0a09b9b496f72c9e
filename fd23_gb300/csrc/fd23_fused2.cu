// Two-step fused sweep for P-SV on sm_103a (FP32 wavefields and arithmetic).
//
// One launch advances every cell two full time steps (it and it+1): stress,
// point source, velocity, stress, point source, velocity.  Each wavefield is
// read from HBM once and written once per two steps, and the material is
// read from HBM once per two steps, so the bytes per cell-update are about
// half those of the one-step sweep (fd23_fused.cuh); the arithmetic is the
// same operation sequence, so the results are bit-identical to two
// launches of the one-step sweep (and to the CPU oracle).  The reference
// computes the same two steps as four launches of its stress and velocity
// kernels (PD/fd/cu_fd.cu:209-501) with host round trips for the source
// (PD/point_source/cu_point_source.cu) and the receivers
// (PD/record/cu_record.cu:154).
//
// Data flow of one CTA (one per SM: 8 compute warps = 4 rows x 2 column
// halves, every compute thread owning 4 adjacent cells of a row, plus one
// producer warp):
//   * A strip of TX = 232 output columns [x0, x0+TX) and rows [z0, z1) is
//     worked through in blocks of 4 rows.  Iteration i runs four phases,
//     each 4 rows behind the one before (the reach of the z-stencil):
//       S1  stress of step it       rows z0-12+4i .. +3, columns x0-12 .. x0+243
//       V1  velocity of step it     rows z0-16+4i .. +3, columns x0-8  .. x0+239
//       S2  stress of step it+1     rows z0-20+4i .. +3, columns x0-4  .. x0+235
//       V2  velocity of step it+1   rows z0-24+4i .. +3, columns x0    .. x0+231
//     Each phase recomputes the 4 columns either side that the next phase's
//     x-stencil needs, instead of exchanging them between CTAs.
//   * The producer streams 4-row blocks of U, W (step it) into a 4-slot ring
//     and, per iteration, the old stresses and the material of S1 and V1 into
//     2 stages, with tiled tensor copies (TMA) gated by full/empty mbarriers.
//   * S1 writes its stresses into a 3-block ring (read by V1's stencil and as
//     S2's old stresses), V1 its velocities into a 3-block ring (S2's stencil,
//     V2's old velocities), S2 its stresses into a third ring (V2's stencil)
//     and to HBM.  V2 writes to HBM only.  Three barriers over the compute
//     warps per iteration order the rings.
//   * The material of S2 and V2 is the material S1 and V1 used two
//     iterations earlier: read again through the read-only path, it comes
//     from L2.
//   * Memory variables of step it+1 (written by S1, V1 for every cell they
//     compute, halo cells included -- every CTA computing a cell writes the
//     same value) go to a third set and are read back by S2, V2 of the same
//     thread; S2 and V2 write the step-(it+2) set for the cells they own.
//   * Receivers of step it are recorded where V1 (velocities) and S1
//     (stresses) compute the cell, from per-item lists built on the host;
//     those of step it+1 are gathered by the next launch.
//   * Interior cells outside the CPML take the branch-free path with packed
//     FP32 pairs; x-interior cells of z-CPML rows the packed differences with
//     the z chain; edge, CPML, free-surface and outside cells the general
//     per-cell path -- the one-step sweep's three paths.
#include "fd23_fused.cuh"

namespace fd23 {

namespace {

// tiled 4-D tensor copy (TMA) of one box at (c0, c1, c2, c3)
__device__ __forceinline__ void tma_load_4d(void *dst, const void *map, int c0, int c1, int c2, int c3,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

template <class M, int W>
struct Cfg2 {
    static constexpr int NCWX = W / 128;       // compute warps per row
    static constexpr int NCW = 4 * NCWX;       // compute warps: 4 rows x NCWX column parts
    static constexpr int NCT = 32 * NCW;       // compute threads
    static constexpr int NTH = NCT + 32;       // + one producer warp
    static constexpr int NTR = W / 4;          // column groups (threads) per row
    static constexpr int MINB = 256 / W;       // CTAs per SM the registers are budgeted for
    static constexpr int W1 = W;               // columns of S1 = ring row width
    static constexpr int TX = W1 - 24;         // output columns per strip
    static constexpr int UWW = W1 + 8;         // input rows: columns x0-16 .. x0+W1-9
    static constexpr int MOFF = sizeof(M) == 2 ? 4 : 0;  // 16-byte aligned copy starts
    static constexpr int MWW = W1 + 2 * MOFF;  // material rows
    static constexpr int NUW = 4, NPW = 2, NR = 3;
    static constexpr int MAX_ITEMS = 4, MAX_TERMS = 16;
    static constexpr int al128(int b) { return (b + 127) / 128 * 128; }
    // U and W inputs in two rings of 4 * NUW rows (a power of two) with a
    // uniform row stride, so a row's address is one mask and one multiply
    static constexpr int UW_RING = 4 * NUW * UWW;  // floats per input ring
    static constexpr int TOLD_B = 3 * 4 * W1 * 4;                   // [Txx Txz Tzz][4 rows][W1] floats
    static constexpr int MS_B = al128(3 * 4 * MWW * (int)sizeof(M));  // [LAM MU MUA][4][MWW]
    static constexpr int MV_B = al128(2 * 4 * MWW * (int)sizeof(M));  // [BU BW][4][MWW]
    static constexpr int STAGE_B = TOLD_B + MS_B + MV_B;
    static constexpr int TR_ROW = 3 * W1;  // floats per stress-ring row: [Txx Txz Tzz][W1]
    static constexpr int VR_ROW = 2 * W1;  // velocity-ring row: [U W][W1]
    static constexpr int OFF_UW = 0;
    static constexpr int OFF_PW = OFF_UW + 2 * UW_RING * 4;
    static constexpr int OFF_TR = OFF_PW + NPW * STAGE_B;
    static constexpr int OFF_VR = OFF_TR + NR * 4 * TR_ROW * 4;
    static constexpr int OFF_T2 = OFF_VR + NR * 4 * VR_ROW * 4;
    static constexpr int OFF_BAR = OFF_T2 + NR * 4 * TR_ROW * 4;
    static constexpr int OFF_INFO = OFF_BAR + 128;
    static constexpr int OFF_TL = OFF_INFO + MAX_ITEMS * 16;
    static constexpr size_t SMEM = (size_t)OFF_TL + MAX_ITEMS * MAX_TERMS * 16;
    static constexpr uint32_t UW_TX = (uint32_t)(2 * 4 * UWW * 4);
    static constexpr uint32_t PW_TX = (uint32_t)(TOLD_B + 5 * 4 * MWW * sizeof(M));
    static_assert(W == 128 || W == 256, "strip widths");
    static_assert((4 * UWW * 4) % 128 == 0, "input slots land 128-byte aligned");
    static_assert(OFF_PW % 128 == 0 && STAGE_B % 128 == 0 && OFF_TR % 128 == 0, "copy destinations");
    static_assert(2 * (NUW + NPW) * 8 <= 128, "barrier space");
    static_assert(UWW % 8 == 0 && (kXPad - 16) % 8 == 0 && TX % 8 == 0, "input copies start on 8-column groups");
};

// ring row (rb + d) of a ring of 12 rows, rb in [0, 12): no division
__device__ __forceinline__ int ring12(int rb, int d)
{
    const int r = rb + d;
    return r >= 12 ? r - 12 : r;
}

// P-SV stress update of cells x .. x+3 of row j (PD/fd/cu_fd.cu:209-358).
// ur[d]: U at row j-4+d (d = 0..8) at this thread's first cell; W at
// ur[d] + WOF.  told: old Txx Txz Tzz; ms: LAM MU MUA.  prd / pwr: memory
// variables read / written; own(ix) says which cells write theirs.
template <int WOF, class Own>
__device__ __forceinline__ void stress4(const Shot<float, float> &sh, const float *const *prd, float *const *pwr,
                                        int j, int x, bool xfast, const float *const ur[9], const float told[3][4],
                                        const float ms[3][4], Own own, float tnew[3][4])
{
    using C = float;
    using S = float;
    const int nx = sh.nx, nz = sh.nz, npml = sh.npml;
    const C *cp = sh.cpml;
    const int B = sh.cpml_blk;
    constexpr C c0 = Coef4<C>::c0, c1 = Coef4<C>::c1, c2 = Coef4<C>::c2, c3 = Coef4<C>::c3;
    using P = P4<C>;
    const bool zfast = j >= 4 && j <= nz - 5 && j < nz - npml && !(sh.topabsorb && j < npml);
    if (xfast && zfast) {
        // interior: packed operands; gam = fma(2, mu, lam) equals lam + 2*mu
        C h[12], ux[4], wx[4];
        ld12<S, C>(ur[4], h);
#pragma unroll
        for (int e = 0; e < 4; ++e) ux[e] = dmx<C>(h, e, c0, c1, c2, c3);
        ld12<S, C>(ur[4] + WOF, h);
#pragma unroll
        for (int e = 0; e < 4; ++e) wx[e] = dpx<C>(h, e, c0, c1, c2, c3);
        const P lam = P::from(ms[0]), mua = P::from(ms[2]);
        const P gam = P::fmak(P::splat((C)2), P::from(ms[1]), lam);
        const P UX = P::from(ux), WX = P::from(wx);
        P t0 = P::fma(gam, UX, P::from(told[0]));
        P t2 = P::fma(lam, UX, P::from(told[2]));
        P t1 = P::fma(mua, WX, P::from(told[1]));
        const P UZ = dmz4p<S, C>(ur, 0), WZ = dpz4p<S, C>(ur, WOF);
        P::fma(lam, WZ, t0).to(tnew[0]);
        P::fma(gam, WZ, t2).to(tnew[2]);
        P::fma(mua, UZ, t1).to(tnew[1]);
        return;
    }
    if (xfast && j >= 4 && j <= nz - 5) {
        // x-interior cells of a z-CPML row (8th order everywhere)
        const bool top = j < npml && sh.topabsorb;
        const long long pz0 = top ? (long long)j * nx + x : (long long)(npml + nz - 1 - j) * nx + x;
        C psw[4], psu[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            psw[e] = prd[7][pz0 + e];
            psu[e] = prd[6][pz0 + e];
        }
        C h[12], ux[4], wx[4], uz[4], wz[4];
        ld12<S, C>(ur[4], h);
#pragma unroll
        for (int e = 0; e < 4; ++e) ux[e] = dmx<C>(h, e, c0, c1, c2, c3);
        ld12<S, C>(ur[4] + WOF, h);
#pragma unroll
        for (int e = 0; e < 4; ++e) wx[e] = dpx<C>(h, e, c0, c1, c2, c3);
        dmz4p<S, C>(ur, 0).to(uz);
        dpz4p<S, C>(ur, WOF).to(wz);
        const int zb = 4 * nx;
        const C bW = __ldg(cp + (zb + 3 * nz + j)), cW = __ldg(cp + (B + zb + 3 * nz + j)),
                kW = __ldg(cp + (2 * B + zb + 3 * nz + j));
        const C bU = __ldg(cp + (zb + 2 * nz + j)), cU = __ldg(cp + (B + zb + 2 * nz + j)),
                kU = __ldg(cp + (2 * B + zb + 2 * nz + j));
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const C lam = ms[0][e], mu = ms[1][e], mua = ms[2][e];
            const C gam = lam + (C)2 * mu;
            C txx = told[0][e], txz = told[1][e], tzz = told[2][e];
            txx = fmaC<C>(gam, ux[e], txx);
            tzz = fmaC<C>(lam, ux[e], tzz);
            txz = fmaC<C>(mua, wx[e], txz);
            const C pw = fmaC<C>(bW, psw[e], cW * wz[e]);
            const C t = fmaC<C>(wz[e], kW, pw);
            txx = fmaC<C>(lam, t, txx);
            tzz = fmaC<C>(gam, t, tzz);
            const C pu = fmaC<C>(bU, psu[e], cU * uz[e]);
            txz = fmaC<C>(mua, fmaC<C>(uz[e], kU, pu), txz);
            tnew[0][e] = txx;
            tnew[1][e] = txz;
            tnew[2][e] = tzz;
            if (own(x + e)) {
                pwr[7][pz0 + e] = pw;
                pwr[6][pz0 + e] = pu;
            }
        }
        return;
    }
    // ---- general cells: edges (reduced order), CPML, free surface, outside ----
    const bool inrow = j >= 0 && j < nz;
    const bool top = j < npml && sh.topabsorb;
    C psx[2][4], psz[2][4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int ix = x + e;
        psx[0][e] = psx[1][e] = psz[0][e] = psz[1][e] = (C)0;
        if (!inrow || ix < 0 || ix >= nx) continue;
        if (ix < npml || ix >= nx - npml) {
            const long long px = ix < npml ? (long long)ix + (long long)j * 2 * npml
                                           : (long long)npml + nx - 1 - ix + (long long)j * 2 * npml;
            psx[0][e] = prd[2][px];
            psx[1][e] = prd[3][px];
        }
        if (top || j >= nz - npml) {
            const long long pz = top ? (long long)j * nx + ix : (long long)(npml + nz - 1 - j) * nx + ix;
            psz[0][e] = prd[7][pz];
            psz[1][e] = prd[6][pz];
        }
    }
    C cc[4][4];
#pragma unroll
    for (int e = 0; e < 4; ++e) cell_coef<C>(x + e, j, nx, nz, cc[e][0], cc[e][1], cc[e][2], cc[e][3]);
    C dA[4], dB[4], dC[4], dD[4];  // ux, uz, wx, wz
    {
        C h[12], zv[9][4];
        ld12<S, C>(ur[4], h);
        zcol<S, C>(ur, 0, zv);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            dA[e] = dmx<C>(h, e, cc[e][0], cc[e][1], cc[e][2], cc[e][3]);
            dB[e] = comb<C>(cc[e][0], cc[e][1], cc[e][2], cc[e][3], zv[4][e] - zv[3][e], zv[5][e] - zv[2][e],
                            zv[6][e] - zv[1][e], zv[7][e] - zv[0][e]);
        }
    }
    {
        C h[12], zv[9][4];
        ld12<S, C>(ur[4] + WOF, h);
        zcol<S, C>(ur, WOF, zv);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            dC[e] = dpx<C>(h, e, cc[e][0], cc[e][1], cc[e][2], cc[e][3]);
            dD[e] = comb<C>(cc[e][0], cc[e][1], cc[e][2], cc[e][3], zv[5][e] - zv[4][e], zv[6][e] - zv[3][e],
                            zv[7][e] - zv[2][e], zv[8][e] - zv[1][e]);
        }
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int ix = x + e;
        if (!inrow || ix < 0 || ix >= nx) {
#pragma unroll
            for (int f = 0; f < 3; ++f) tnew[f][e] = (C)0;
            continue;
        }
        const bool ow = own(ix);
        const bool xp = ix < npml || ix >= nx - npml;
        const bool zp = top || j >= nz - npml;
        const long long px = ix < npml ? (long long)ix + (long long)j * 2 * npml
                                       : (long long)npml + nx - 1 - ix + (long long)j * 2 * npml;
        const long long pz = top ? (long long)j * nx + ix : (long long)(npml + nz - 1 - j) * nx + ix;
        const C ux = dA[e], uz = dB[e], wx = dC[e], wz = dD[e];
        const C lam = ms[0][e], mu = ms[1][e], mua = ms[2][e];
        const C gam = lam + (C)2 * mu;
        C txx = told[0][e], txz = told[1][e], tzz = told[2][e];
        // x chain, PD/fd/cu_fd.cu:303-326
        if (xp) {
            const C pu = fmaC<C>(__ldg(cp + (2 * nx + ix)), psx[0][e], __ldg(cp + (B + 2 * nx + ix)) * ux);
            const C t = fmaC<C>(ux, __ldg(cp + (2 * B + 2 * nx + ix)), pu);
            txx = fmaC<C>(gam, t, txx);
            tzz = fmaC<C>(lam, t, tzz);
            const C pw = fmaC<C>(__ldg(cp + (3 * nx + ix)), psx[1][e], __ldg(cp + (B + 3 * nx + ix)) * wx);
            txz = fmaC<C>(mua, fmaC<C>(wx, __ldg(cp + (2 * B + 3 * nx + ix)), pw), txz);
            if (ow) {
                pwr[2][px] = pu;
                pwr[3][px] = pw;
            }
        } else if (j != 0) {
            txx = fmaC<C>(gam, ux, txx);
            tzz = fmaC<C>(lam, ux, tzz);
            txz = fmaC<C>(mua, wx, txz);
        }
        // z chain, :328-355
        if (zp) {
            const int zb = 4 * nx;
            const C pw = fmaC<C>(__ldg(cp + (zb + 3 * nz + j)), psz[0][e], __ldg(cp + (B + zb + 3 * nz + j)) * wz);
            const C t = fmaC<C>(wz, __ldg(cp + (2 * B + zb + 3 * nz + j)), pw);
            txx = fmaC<C>(lam, t, txx);
            tzz = fmaC<C>(gam, t, tzz);
            const C pu = fmaC<C>(__ldg(cp + (zb + 2 * nz + j)), psz[1][e], __ldg(cp + (B + zb + 2 * nz + j)) * uz);
            txz = fmaC<C>(mua, fmaC<C>(uz, __ldg(cp + (2 * B + zb + 2 * nz + j)), pu), txz);
            if (ow) {
                pwr[7][pz] = pw;
                pwr[6][pz] = pu;
            }
        } else if (j == 0) {
            txx = fmaC<C>((C)2 * mu, ux, txx);
            tzz = (C)0;
            txz = (C)0;
        } else {
            txx = fmaC<C>(lam, wz, txx);
            tzz = fmaC<C>(gam, wz, tzz);
            txz = fmaC<C>(mua, uz, txz);
        }
        tnew[0][e] = txx;
        tnew[1][e] = txz;
        tnew[2][e] = tzz;
    }
}

// P-SV velocity update of cells x .. x+3 of row a (PD/fd/cu_fd.cu:359-501).
// tr[d]: Txx at row a-4+d (d = 0..8) at this thread's first cell, Txz at
// tr[d] + W1, Tzz at tr[d] + 2*W1.  vold: old U W; mv: BU BW.
template <int W1, class Own>
__device__ __forceinline__ void velocity4(const Shot<float, float> &sh, const float *const *prd, float *const *pwr,
                                          int a, int x, bool xfast, const float *const tr[9], const float vold[2][4],
                                          const float mv[2][4], Own own, float vnew[2][4])
{
    using C = float;
    using S = float;
    const int nx = sh.nx, nz = sh.nz, npml = sh.npml;
    const C *cp = sh.cpml;
    const int B = sh.cpml_blk;
    constexpr C c0 = Coef4<C>::c0, c1 = Coef4<C>::c1, c2 = Coef4<C>::c2, c3 = Coef4<C>::c3;
    using P = P4<C>;
    const bool zfast = a >= 4 && a <= nz - 5 && a < nz - npml && !(sh.topabsorb && a < npml);
    if (xfast && zfast) {
        C h[12], dx[4];
        const P bu = P::from(mv[0]), bw = P::from(mv[1]);
        ld12<S, C>(tr[4], h);  // Txx
#pragma unroll
        for (int e = 0; e < 4; ++e) dx[e] = dpx<C>(h, e, c0, c1, c2, c3);
        P u = P::fma(bu, P::from(dx), P::from(vold[0]));
        ld12<S, C>(tr[4] + W1, h);  // Txz
#pragma unroll
        for (int e = 0; e < 4; ++e) dx[e] = dmx<C>(h, e, c0, c1, c2, c3);
        P w = P::fma(bw, P::from(dx), P::from(vold[1]));
        P::fma(bu, dpz4p<S, C>(tr, W1), u).to(vnew[0]);      // d/dz Txz
        P::fma(bw, dmz4p<S, C>(tr, 2 * W1), w).to(vnew[1]);  // d/dz Tzz
        return;
    }
    if (xfast && a >= 4 && a <= nz - 5) {
        // x-interior cells of a z-CPML row
        const bool top = a < npml && sh.topabsorb;
        const long long pz0 = top ? (long long)a * nx + x : (long long)(npml + nz - 1 - a) * nx + x;
        C psa[4], psb[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            psa[e] = prd[5][pz0 + e];
            psb[e] = prd[4][pz0 + e];
        }
        C h[12], dxTxx[4], dxTxz[4], dzTxz[4], dzTzz[4];
        ld12<S, C>(tr[4], h);
#pragma unroll
        for (int e = 0; e < 4; ++e) dxTxx[e] = dpx<C>(h, e, c0, c1, c2, c3);
        ld12<S, C>(tr[4] + W1, h);
#pragma unroll
        for (int e = 0; e < 4; ++e) dxTxz[e] = dmx<C>(h, e, c0, c1, c2, c3);
        dpz4p<S, C>(tr, W1).to(dzTxz);
        dmz4p<S, C>(tr, 2 * W1).to(dzTzz);
        const int zb = 4 * nx;
        const C bA = __ldg(cp + (zb + nz + a)), cA = __ldg(cp + (B + zb + nz + a)), kA = __ldg(cp + (2 * B + zb + nz + a));
        const C bB = __ldg(cp + (zb + a)), cB = __ldg(cp + (B + zb + a)), kB = __ldg(cp + (2 * B + zb + a));
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const C bu = mv[0][e], bw = mv[1][e];
            C u = vold[0][e], w = vold[1][e];
            u = fmaC<C>(bu, dxTxx[e], u);
            w = fmaC<C>(bw, dxTxz[e], w);
            const C pa = fmaC<C>(bA, psa[e], cA * dzTxz[e]);
            const C pb = fmaC<C>(bB, psb[e], cB * dzTzz[e]);
            u = fmaC<C>(bu, fmaC<C>(dzTxz[e], kA, pa), u);
            w = fmaC<C>(bw, fmaC<C>(dzTzz[e], kB, pb), w);
            vnew[0][e] = u;
            vnew[1][e] = w;
            if (own(x + e)) {
                pwr[5][pz0 + e] = pa;
                pwr[4][pz0 + e] = pb;
            }
        }
        return;
    }
    // ---- general cells ----
    const bool inrow = a >= 0 && a < nz;
    const bool top = a < npml && sh.topabsorb;
    C psx[2][4], psz[2][4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int ix = x + e;
        psx[0][e] = psx[1][e] = psz[0][e] = psz[1][e] = (C)0;
        if (!inrow || ix < 0 || ix >= nx) continue;
        if (ix < npml || ix >= nx - npml) {
            const long long px = ix < npml ? (long long)ix + (long long)a * 2 * npml
                                           : (long long)npml + nx - 1 - ix + (long long)a * 2 * npml;
            psx[0][e] = prd[0][px];
            psx[1][e] = prd[1][px];
        }
        if (top || a >= nz - npml) {
            const long long pz = top ? (long long)a * nx + ix : (long long)(npml + nz - 1 - a) * nx + ix;
            psz[0][e] = prd[5][pz];
            psz[1][e] = prd[4][pz];
        }
    }
    C cc[4][4];
#pragma unroll
    for (int e = 0; e < 4; ++e) cell_coef<C>(x + e, a, nx, nz, cc[e][0], cc[e][1], cc[e][2], cc[e][3]);
    // dA = d/dx Txx, dB = d/dx Txz, dC = d/dz Txz, dD = d/dz Tzz
    C dA[4], dB[4], dC[4], dD[4];
    {
        C h[12];
        ld12<S, C>(tr[4], h);
#pragma unroll
        for (int e = 0; e < 4; ++e) dA[e] = dpx<C>(h, e, cc[e][0], cc[e][1], cc[e][2], cc[e][3]);
    }
    {
        C h[12], zv[9][4];
        ld12<S, C>(tr[4] + W1, h);
        zcol<S, C>(tr, W1, zv);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            dB[e] = dmx<C>(h, e, cc[e][0], cc[e][1], cc[e][2], cc[e][3]);
            dC[e] = comb<C>(cc[e][0], cc[e][1], cc[e][2], cc[e][3], zv[5][e] - zv[4][e], zv[6][e] - zv[3][e],
                            zv[7][e] - zv[2][e], zv[8][e] - zv[1][e]);
        }
    }
    {
        C zv[9][4];
        zcol<S, C>(tr, 2 * W1, zv);
#pragma unroll
        for (int e = 0; e < 4; ++e)
            dD[e] = comb<C>(cc[e][0], cc[e][1], cc[e][2], cc[e][3], zv[4][e] - zv[3][e], zv[5][e] - zv[2][e],
                            zv[6][e] - zv[1][e], zv[7][e] - zv[0][e]);
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int ix = x + e;
        if (!inrow || ix < 0 || ix >= nx) {
            vnew[0][e] = vnew[1][e] = (C)0;
            continue;
        }
        const bool ow = own(ix);
        const bool xp = ix < npml || ix >= nx - npml;
        const bool zp = top || a >= nz - npml;
        const long long px = ix < npml ? (long long)ix + (long long)a * 2 * npml
                                       : (long long)npml + nx - 1 - ix + (long long)a * 2 * npml;
        const long long pz = top ? (long long)a * nx + ix : (long long)(npml + nz - 1 - a) * nx + ix;
        const C dxTxx = dA[e], dxTxz = dB[e], dzTxz = dC[e], dzTzz = dD[e];
        const C bu = mv[0][e], bw = mv[1][e];
        C u = vold[0][e], w = vold[1][e];
        // x chain, PD/fd/cu_fd.cu:455-474
        if (xp) {
            const C pa = fmaC<C>(__ldg(cp + (ix)), psx[0][e], __ldg(cp + (B + ix)) * dxTxx);
            u = fmaC<C>(bu, fmaC<C>(dxTxx, __ldg(cp + (2 * B + ix)), pa), u);
            const C pb = fmaC<C>(__ldg(cp + (nx + ix)), psx[1][e], __ldg(cp + (B + nx + ix)) * dxTxz);
            w = fmaC<C>(bw, fmaC<C>(dxTxz, __ldg(cp + (2 * B + nx + ix)), pb), w);
            if (ow) {
                pwr[0][px] = pa;
                pwr[1][px] = pb;
            }
        } else if (a != 0) {
            u = fmaC<C>(bu, dxTxx, u);
            w = fmaC<C>(bw, dxTxz, w);
        }
        // z chain, :476-499
        if (zp) {
            const int zb = 4 * nx;
            const C pa = fmaC<C>(__ldg(cp + (zb + nz + a)), psz[0][e], __ldg(cp + (B + zb + nz + a)) * dzTxz);
            const C pb = fmaC<C>(__ldg(cp + (zb + a)), psz[1][e], __ldg(cp + (B + zb + a)) * dzTzz);
            u = fmaC<C>(bu, fmaC<C>(dzTxz, __ldg(cp + (2 * B + zb + nz + a)), pa), u);
            w = fmaC<C>(bw, fmaC<C>(dzTzz, __ldg(cp + (2 * B + zb + a)), pb), w);
            if (ow) {
                pwr[5][pz] = pa;
                pwr[4][pz] = pb;
            }
        } else if (a == 0) {
            u = fmaC<C>(bu, dxTxx + dzTxz, u);
            w = (C)0;
        } else {
            u = fmaC<C>(bu, dzTxz, u);
            w = fmaC<C>(bw, dzTzz, w);
        }
        vnew[0][e] = u;
        vnew[1][e] = w;
    }
}

// material of 4 cells from shared memory or global memory
template <class M>
__device__ __forceinline__ void ld_mat4(const M *p, float v[4])
{
    Vec4<M, float>::ld(p, v);
}
template <class M>
__device__ __forceinline__ void ldg_mat4(const M *p, float v[4])
{
    if constexpr (sizeof(M) == 4) {
        const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    } else {
        const uint2 t = __ldg(reinterpret_cast<const uint2 *>(p));
        M h[4];
        memcpy(h, &t, 8);
#pragma unroll
        for (int e = 0; e < 4; ++e) v[e] = to_c<float>(h[e]);
    }
}

// point-source terms of step `it` on the 4 cells of stress row j
__device__ __forceinline__ void add_terms(const Shot<float, float> &sh, const int4 *tl, int ntl, int j, int x, int it,
                                          float tnew[3][4])
{
    if (ntl <= 0 || it >= sh.tamp_nt) return;
    for (int t = 0; t < ntl; ++t) {
        const int4 tm = tl[t];  // (field, ix, iz, term index)
        if (tm.x >= FD23_TXX && tm.z == j && tm.y >= x && tm.y < x + 4) {
            const float amp = sh.tamp[(long long)tm.w * sh.tamp_nt + it];
            // compile-time indices only (a runtime index would put tnew in local memory)
#pragma unroll
            for (int f = 0; f < 3; ++f)
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (tm.x == FD23_TXX + f && tm.y == x + e) tnew[f][e] = tnew[f][e] + amp;
        }
    }
}

template <class M, int W>
__global__ void __launch_bounds__(Cfg2<M, W>::NTH, Cfg2<M, W>::MINB)
    fused2_step(const __grid_constant__ Shot<float, float> sh, const WorkItem *__restrict__ items,
                const int *__restrict__ item_off, int par, int it, int rec_index, int rec_mid, int *err_flag)
{
    using K = Cfg2<M, W>;
    using C = float;
    constexpr int W1 = K::W1;
    if (err_flag && *(volatile int *)err_flag) return;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    if (smem_u32(smem_raw) & 127u) {
        if (threadIdx.x == 0 && err_flag) atomicExch(err_flag, 2);
        return;
    }
    float *uw_s = reinterpret_cast<float *>(smem_raw + K::OFF_UW);  // U ring, then W ring
    unsigned char *pw_b = smem_raw + K::OFF_PW;
    float *tr_s = reinterpret_cast<float *>(smem_raw + K::OFF_TR);
    float *vr_s = reinterpret_cast<float *>(smem_raw + K::OFF_VR);
    float *t2_s = reinterpret_cast<float *>(smem_raw + K::OFF_T2);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw + K::OFF_BAR);
    uint64_t *full_uw = bars, *empty_uw = bars + K::NUW;
    uint64_t *full_pw = bars + 2 * K::NUW, *empty_pw = full_pw + K::NPW;
    ItemInfo *info = reinterpret_cast<ItemInfo *>(smem_raw + K::OFF_INFO);
    int4 *tlist = reinterpret_cast<int4 *>(smem_raw + K::OFF_TL);
    __shared__ int tcount[K::MAX_ITEMS];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ibeg = item_off[blockIdx.x], iend = item_off[blockIdx.x + 1];
    const int nitems = min(iend - ibeg, K::MAX_ITEMS);
    const int nx = sh.nx, nz = sh.nz, pitch = sh.pitch;
    const int origin = (int)sh.origin;  // padded arrays hold fewer than 2^31 elements

    // ---- per-item set-up: geometry and the source terms inside its S1 region ----
    if (tid < nitems) {
        const WorkItem w = items[ibeg + tid];
        info[tid] = ItemInfo{w.x0, w.z0, w.z1, (w.z1 - w.z0) / 4 + 6};
        int cnt = 0;
        if (it < sh.tamp_nt) {
            for (int t = 0; t < sh.nterms && cnt < K::MAX_TERMS; ++t) {
                const int4 tm = sh.terms[t];
                if (tm.y >= w.x0 - 12 && tm.y < w.x0 - 12 + W1 && tm.z >= w.z0 - 12 && tm.z < w.z1 + 12)
                    tlist[tid * K::MAX_TERMS + cnt++] = make_int4(tm.x, tm.y, tm.z, t);
            }
        }
        tcount[tid] = cnt;
    }
    if (tid == 0) {
        for (int b = 0; b < K::NUW; ++b) {
            mbar_init(&full_uw[b], 1);
            mbar_init(&empty_uw[b], K::NCW);
        }
        for (int b = 0; b < K::NPW; ++b) {
            mbar_init(&full_pw[b], 1);
            mbar_init(&empty_pw[b], K::NCW);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // the next launch may start its prologue; it waits before touching any
    // wavefield or memory variable
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");

    int total_iters = 0;
    for (int k = 0; k < nitems; ++k) total_iters += info[k].niter;

    // ======================= producer warp =======================
    if (warp == K::NCW) {
        const ShotMaps2 *maps = sh.maps2;
        // input block e -> item k, block b (rows z0-16+4b .. +3), into rows
        // 4*(e % NUW) .. +3 of the U ring and of the W ring
        auto issue_uw = [=](int e) {
            int k = 0, base = 0;
            while (k < nitems - 1 && e >= base + info[k].niter + 2) {
                base += info[k].niter + 2;
                ++k;
            }
            const ItemInfo I = info[k];
            const int slot = e % K::NUW;
            const int r0 = I.z0 - 16 + 4 * (e - base);
            if (lane == 0) {
                // rows wider than a box dimension's 256 elements: the map views
                // the columns as [column / 8][8], the copy starts on a group
                mbar_arrive_expect_tx(&full_uw[slot], K::UW_TX);
                const int gx = (kXPad + I.x0 - 16) / 8;
                tma_load_4d(uw_s + slot * 4 * K::UWW, &maps->uw[par], 0, gx, kZPad + r0, FD23_U, &full_uw[slot]);
                tma_load_4d(uw_s + K::UW_RING + slot * 4 * K::UWW, &maps->uw[par], 0, gx, kZPad + r0, FD23_W,
                            &full_uw[slot]);
            }
        };
        // stage of iteration i: old stresses and stress-update material on S1
        // rows, velocity-update material on V1 rows.  part 1: arm the stage
        // and copy the material only (it does not depend on the previous
        // step); 2: the old stresses only; 0: everything
        auto issue_pw = [=](int g, const ItemInfo &I, int i, int part) {
            const int slot = g % K::NPW;
            if (lane == 0) {
                unsigned char *st = pw_b + slot * K::STAGE_B;
                if (part != 2) mbar_arrive_expect_tx(&full_pw[slot], K::PW_TX);
                const int xs = kXPad + I.x0 - 12;
                const int ys = kZPad + I.z0 - 12 + 4 * i, yv = ys - 4;
                if (part != 1) tma_load_3d(st, &maps->t[par], xs, ys, FD23_TXX, &full_pw[slot]);
                if (part != 2) {
                    tma_load_3d(st + K::TOLD_B, &maps->ms, xs - K::MOFF, ys, 0, &full_pw[slot]);
                    tma_load_3d(st + K::TOLD_B + K::MS_B, &maps->mv, xs - K::MOFF, yv, 3, &full_pw[slot]);
                }
            }
        };
        bool ok = true;
        int e_uw = 0, g_pw = 0;
        int k = 0, base_it = 0, base_uw = 0;
        const int npre = min(K::NPW, total_iters);
        {
            int kk = 0, bit = 0;
            for (int g = 0; g < npre; ++g) {
                while (g >= bit + info[kk].niter) {
                    bit += info[kk].niter;
                    ++kk;
                }
                issue_pw(g, info[kk], g - bit, 1);
            }
        }
        asm volatile("griddepcontrol.wait;" ::: "memory");
        for (int g = 0; g < total_iters && ok; ++g) {
            while (g >= base_it + info[k].niter) {
                base_it += info[k].niter;
                base_uw += info[k].niter + 2;
                ++k;
            }
            const int i = g - base_it;
            const int need = base_uw + i + 2;  // iteration g reads blocks need-2 .. need
            while (ok && e_uw <= need) {
                if (e_uw >= K::NUW)
                    ok = mbar_wait_bounded(&empty_uw[e_uw % K::NUW], (uint32_t)(((e_uw / K::NUW) - 1) & 1), err_flag);
                if (ok) issue_uw(e_uw++);
            }
            if (!ok) break;
            if (g >= K::NPW)
                ok = mbar_wait_bounded(&empty_pw[g % K::NPW], (uint32_t)(((g / K::NPW) - 1) & 1), err_flag);
            if (ok) {
                issue_pw(g, info[k], i, g < npre ? 2 : 0);
                g_pw = g + 1;
            }
        }
        // every copy issued must land before this CTA can release its shared memory
        for (int e = max(0, e_uw - K::NUW); e < e_uw; ++e)
            mbar_wait_bounded(&full_uw[e % K::NUW], (uint32_t)((e / K::NUW) & 1), nullptr);
        for (int g = max(0, g_pw - K::NPW); g < g_pw; ++g)
            mbar_wait_bounded(&full_pw[g % K::NPW], (uint32_t)((g / K::NPW) & 1), nullptr);
        return;
    }

    // ======================= compute warps =======================
    asm volatile("griddepcontrol.wait;" ::: "memory");
    // ---- receivers of the previous launch's last step (buffer set `par` is read-only here) ----
    if (rec_index >= 0) {
#pragma unroll
        for (int c = 0; c < 5; ++c)
            for (int r = ((int)blockIdx.x - sh.cta0) * K::NCT + tid; r < sh.nrec[c]; r += sh.ncta * K::NCT)
                sh.seis[c][(long long)rec_index * sh.nrec[c] + r] = sh.f[par][c][sh.rec[c][r]];
    }

    const int g = warp & 3;                   // row of the 4-row block
    const int t = 32 * (warp >> 2) + lane;    // column group 0 .. NTR-1
    constexpr int NTR = K::NTR;
    const bool v1_t = t >= 1 && t <= NTR - 2, s2_t = t >= 2 && t <= NTR - 3, v2_t = t >= 3 && t <= NTR - 4;
    // this thread's column in the input rings and in the 12-row rings
    const float *const u_col = uw_s + 4 + 4 * t;
    float *const tr_col = tr_s + 4 * t;
    float *const vr_col = vr_s + 4 * t;
    float *const t2_col = t2_s + 4 * t;
    float *const *psi_rd = sh.psi[par];
    float *const *psi_wr = sh.psi[1 - par];
    float *const *psi_mid = sh.psim;
    const M *gmat[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) gmat[m] = reinterpret_cast<const M *>(sh.mat16[m] ? sh.mat16[m] : (const void *)sh.mat[m]);
    float *wr[5];
#pragma unroll
    for (int f = 0; f < 5; ++f) wr[f] = sh.f[1 - par][f];

    bool ok = true;
    int uw_ready = 0, gflat = 0, uw_base = 0;
    for (int k = 0; k < nitems && ok; ++k) {
        const ItemInfo I = info[k];
        const int ntl = tcount[k];
        const int4 *tl = tlist + k * K::MAX_TERMS;
        const int x = I.x0 - 12 + 4 * t;  // first of this thread's 4 cells
        const bool xin = x + 3 >= 0 && x < nx;
        const bool xfast = x >= max(4, sh.npml) && x + 3 <= min(nx - 5, nx - sh.npml - 1);
        // owned cells: the output columns of the strip, rows [z0, z1)
        const int ox0 = I.x0, ox1 = I.x0 + K::TX;
        // receivers of the step in between owned by this item (sorted by row)
        int cv = 0, cs = 0, ce = 0;
        if (rec_mid >= 0 && sh.rec2_off) {
            const int kk = ibeg + k;
            cv = __ldg(sh.rec2_off + 2 * kk);
            cs = __ldg(sh.rec2_off + 2 * kk + 1);
            ce = __ldg(sh.rec2_off + 2 * kk + 2);
        }
        const int cs0 = cs;  // end of the velocity entries
        // 12-row ring rows (block b, row r) = (4b + r) mod 12: rb = row of
        // (block i-2, row g), wb = row of (block i, row g); advanced by 4 per
        // iteration
        int rb = (12 - 8 + g) % 12, wb = g;
        for (int i = 0; i < I.niter; ++i, ++gflat, rb = ring12(rb, 4), wb = ring12(wb, 4)) {
            for (; ok && uw_ready <= uw_base + i + 2; ++uw_ready)
                ok = mbar_wait_bounded(&full_uw[uw_ready % K::NUW], (uint32_t)((uw_ready / K::NUW) & 1), err_flag);
            if (ok) ok = mbar_wait_bounded(&full_pw[gflat % K::NPW], (uint32_t)((gflat / K::NPW) & 1), err_flag);
            const unsigned char *stg = pw_b + (gflat % K::NPW) * K::STAGE_B;
            const float *told_s = reinterpret_cast<const float *>(stg);
            const int ub = (4 * (uw_base + i) + g) & (4 * K::NUW - 1);  // input ring row of (block i, row g)
            const M *ms_s = reinterpret_cast<const M *>(stg + K::TOLD_B);
            const M *mv_s = reinterpret_cast<const M *>(stg + K::TOLD_B + K::MS_B);
            const int j1 = I.z0 - 12 + 4 * i + g, a1 = j1 - 4, j2 = j1 - 8, a2 = j1 - 12;
            const bool v1_on = i >= 2, s2_on = i >= 4, v2_on = i >= 6;

            // material of S2 and V2 (read by S1 and V1 two iterations ago: from L2)
            float ms2[3][4], mv2[2][4];
#pragma unroll
            for (int e = 0; e < 4; ++e) ms2[0][e] = ms2[1][e] = ms2[2][e] = mv2[0][e] = mv2[1][e] = 0.f;
            if (s2_on && s2_t && xin && j2 >= 0 && j2 < nz) {
                const int o = origin + j2 * pitch + x;
#pragma unroll
                for (int m = 0; m < 3; ++m) ldg_mat4<M>(gmat[m] + o, ms2[m]);
            }
            if (v2_on && v2_t && xin && a2 >= 0 && a2 < nz) {
                const int o = origin + a2 * pitch + x;
#pragma unroll
                for (int m = 0; m < 2; ++m) ldg_mat4<M>(gmat[3 + m] + o, mv2[m]);
            }

            // ================= S1: stress of step it, row j1 =================
            {
                const float *ur[9];
#pragma unroll
                for (int d = 0; d < 9; ++d) ur[d] = u_col + ((ub + d) & (4 * K::NUW - 1)) * K::UWW;
                float tnew[3][4];
                if (j1 < 0 || j1 >= nz || !xin) {
#pragma unroll
                    for (int f = 0; f < 3; ++f)
#pragma unroll
                        for (int e = 0; e < 4; ++e) tnew[f][e] = 0.f;
                } else {
                    float told[3][4], ms[3][4];
#pragma unroll
                    for (int f = 0; f < 3; ++f) Vec4<float, float>::ld(told_s + (f * 4 + g) * W1 + 4 * t, told[f]);
#pragma unroll
                    for (int m = 0; m < 3; ++m) ld_mat4<M>(ms_s + (m * 4 + g) * K::MWW + K::MOFF + 4 * t, ms[m]);
                    stress4<K::UW_RING>(sh, psi_rd, psi_mid, j1, x, xfast, ur, told, ms, [](int) { return true; }, tnew);
                    add_terms(sh, tl, ntl, j1, x, it, tnew);
                    // stress receivers of step it
                    if (cs < ce && j1 >= I.z0 && j1 < I.z1) {
                        while (cs < ce && __ldg(&sh.rec2[cs].z) < j1) ++cs;
                        for (int c = cs; c < ce; ++c) {
                            const int4 r = __ldg(sh.rec2 + c);
                            if (r.z != j1) break;
                            if (r.y >= x && r.y < x + 4) {
                                float v = 0.f;
#pragma unroll
                                for (int f = 0; f < 3; ++f)
#pragma unroll
                                    for (int e = 0; e < 4; ++e)
                                        if (r.x == FD23_TXX + f && r.y == x + e) v = tnew[f][e];
                                sh.seis[r.x][(long long)rec_mid * sh.nrec[r.x] + r.w] = v;
                            }
                        }
                    }
                }
                float *dst = tr_col + wb * K::TR_ROW;
#pragma unroll
                for (int f = 0; f < 3; ++f) Vec4<float, float>::st(dst + f * W1, tnew[f]);
            }
            ok = compute_bar_and(K::NCT, ok) != 0;
            if (!ok) break;

            // ================= V1: velocity of step it, row a1 =================
            if (v1_on && v1_t) {
                float vnew[2][4];
                if (a1 < 0 || a1 >= nz || !xin) {
#pragma unroll
                    for (int e = 0; e < 4; ++e) vnew[0][e] = vnew[1][e] = 0.f;
                } else {
                    const float *tr[9];
#pragma unroll
                    for (int d = 0; d < 9; ++d) tr[d] = tr_col + ring12(rb, d) * K::TR_ROW;
                    const float *vo = u_col + ub * K::UWW;
                    float vold[2][4], mv[2][4];
                    Vec4<float, float>::ld(vo, vold[0]);
                    Vec4<float, float>::ld(vo + K::UW_RING, vold[1]);
#pragma unroll
                    for (int m = 0; m < 2; ++m) ld_mat4<M>(mv_s + (m * 4 + g) * K::MWW + K::MOFF + 4 * t, mv[m]);
                    velocity4<W1>(sh, psi_rd, psi_mid, a1, x, xfast, tr, vold, mv, [](int) { return true; }, vnew);
                    // velocity receivers of step it
                    if (cv < cs0 && a1 >= I.z0 && a1 < I.z1) {
                        while (cv < cs0 && __ldg(&sh.rec2[cv].z) < a1) ++cv;
                        for (int c = cv; c < cs0; ++c) {
                            const int4 r = __ldg(sh.rec2 + c);
                            if (r.z != a1) break;
                            if (r.y >= x && r.y < x + 4) {
                                float v = 0.f;
#pragma unroll
                                for (int e = 0; e < 4; ++e)
                                    if (r.y == x + e) v = r.x == FD23_U ? vnew[0][e] : vnew[1][e];
                                sh.seis[r.x][(long long)rec_mid * sh.nrec[r.x] + r.w] = v;
                            }
                        }
                    }
                }
                float *dst = vr_col + wb * K::VR_ROW;
                Vec4<float, float>::st(dst, vnew[0]);
                Vec4<float, float>::st(dst + W1, vnew[1]);
            }
            // S1 and V1 were the last readers of input block i and of this stage
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&empty_uw[(uw_base + i) % K::NUW]);
                if (i == I.niter - 1) {
                    mbar_arrive(&empty_uw[(uw_base + i + 1) % K::NUW]);
                    mbar_arrive(&empty_uw[(uw_base + i + 2) % K::NUW]);
                }
                mbar_arrive(&empty_pw[gflat % K::NPW]);
            }
            ok = compute_bar_and(K::NCT, ok) != 0;
            if (!ok) break;

            // ================= S2: stress of step it+1, row j2 =================
            if (s2_on && s2_t) {
                float tnew[3][4];
                if (j2 < 0 || j2 >= nz || !xin) {
#pragma unroll
                    for (int f = 0; f < 3; ++f)
#pragma unroll
                        for (int e = 0; e < 4; ++e) tnew[f][e] = 0.f;
                } else {
                    const float *vr[9];
#pragma unroll
                    for (int d = 0; d < 9; ++d) vr[d] = vr_col + ring12(rb, d) * K::VR_ROW;
                    const float *to = tr_col + rb * K::TR_ROW;
                    float told[3][4];
#pragma unroll
                    for (int f = 0; f < 3; ++f) Vec4<float, float>::ld(to + f * W1, told[f]);
                    const bool orow = j2 >= I.z0 && j2 < I.z1;
                    stress4<W1>(sh, psi_mid, psi_wr, j2, x, xfast, vr, told, ms2,
                                [=](int ix) { return orow && ix >= ox0 && ix < ox1; }, tnew);
                    add_terms(sh, tl, ntl, j2, x, it + 1, tnew);
                    if (orow && v2_t) {
                        const int o = origin + j2 * pitch + x;
                        if (x + 3 < nx) {
#pragma unroll
                            for (int f = 0; f < 3; ++f) Vec4<float, float>::st(wr[FD23_TXX + f] + o, tnew[f]);
                        } else {
#pragma unroll
                            for (int f = 0; f < 3; ++f)
#pragma unroll
                                for (int e = 0; e < 4; ++e)
                                    if (x + e < nx) wr[FD23_TXX + f][o + e] = tnew[f][e];
                        }
                    }
                }
                float *dst = t2_col + wb * K::TR_ROW;
#pragma unroll
                for (int f = 0; f < 3; ++f) Vec4<float, float>::st(dst + f * W1, tnew[f]);
            }
            ok = compute_bar_and(K::NCT, ok) != 0;
            if (!ok) break;

            // ================= V2: velocity of step it+1, row a2 =================
            if (v2_on && v2_t && a2 >= I.z0 && a2 < I.z1 && a2 < nz && x < nx) {
                const float *tr[9];
#pragma unroll
                for (int d = 0; d < 9; ++d) tr[d] = t2_col + ring12(rb, d) * K::TR_ROW;
                const float *vo = vr_col + rb * K::VR_ROW;
                float vold[2][4], vnew[2][4];
                Vec4<float, float>::ld(vo, vold[0]);
                Vec4<float, float>::ld(vo + W1, vold[1]);
                velocity4<W1>(sh, psi_mid, psi_wr, a2, x, xfast, tr, vold, mv2,
                              [=](int ix) { return ix >= ox0 && ix < ox1; }, vnew);
                const int o = origin + a2 * pitch + x;
                if (x + 3 < nx) {
                    Vec4<float, float>::st(wr[FD23_U] + o, vnew[0]);
                    Vec4<float, float>::st(wr[FD23_W] + o, vnew[1]);
                } else {
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (x + e < nx) {
                            wr[FD23_U][o + e] = vnew[0][e];
                            wr[FD23_W][o + e] = vnew[1][e];
                        }
                }
            }
        }
        uw_base += I.niter + 2;
    }
}

template <class M, int W>
int prepare2()
{
    using K = Cfg2<M, W>;
    return cudaFuncSetAttribute(fused2_step<M, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)K::SMEM) ==
                   cudaSuccess
               ? FD23_OK
               : FD23_ERR_CUDA;
}

template <class M, int W>
int launch2(const Shot<float, float> &s, const WorkItem *items, const int *item_off, int nblocks, int par, int it,
            int rec_index, int rec_mid, int *err_flag, cudaStream_t st)
{
    using K = Cfg2<M, W>;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)nblocks);
    cfg.blockDim = dim3(K::NTH);
    cfg.dynamicSmemBytes = K::SMEM;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e =
        cudaLaunchKernelEx(&cfg, fused2_step<M, W>, s, items, item_off, par, it, rec_index, rec_mid, err_flag);
    return e == cudaSuccess ? FD23_OK : FD23_ERR_CUDA;
}

}  // namespace

template <class M>
int launch_step_fused2(const Shot<float, float> &s, int width, const WorkItem *items, const int *item_off,
                       int nblocks, int par, int it, int rec_index, int rec_mid, int *err_flag, cudaStream_t st)
{
    return width == 128 ? launch2<M, 128>(s, items, item_off, nblocks, par, it, rec_index, rec_mid, err_flag, st)
                        : launch2<M, 256>(s, items, item_off, nblocks, par, it, rec_index, rec_mid, err_flag, st);
}

int fused2_prepare(bool half_material, int width)
{
    if (width == 128) return half_material ? prepare2<__half, 128>() : prepare2<float, 128>();
    return half_material ? prepare2<__half, 256>() : prepare2<float, 256>();
}

int fused2_tile_x(int width) { return width == 128 ? Cfg2<float, 128>::TX : Cfg2<float, 256>::TX; }

int fused2_per_sm(int width) { return width == 128 ? Cfg2<float, 128>::MINB : Cfg2<float, 256>::MINB; }

Fused2Boxes fused2_boxes(bool half_material, int width)
{
    if (width == 128)
        return half_material ? Fused2Boxes{Cfg2<__half, 128>::UWW, Cfg2<__half, 128>::W1, Cfg2<__half, 128>::MWW}
                             : Fused2Boxes{Cfg2<float, 128>::UWW, Cfg2<float, 128>::W1, Cfg2<float, 128>::MWW};
    return half_material ? Fused2Boxes{Cfg2<__half, 256>::UWW, Cfg2<__half, 256>::W1, Cfg2<__half, 256>::MWW}
                         : Fused2Boxes{Cfg2<float, 256>::UWW, Cfg2<float, 256>::W1, Cfg2<float, 256>::MWW};
}

template int launch_step_fused2<float>(const Shot<float, float> &, int, const WorkItem *, const int *, int, int, int,
                                       int, int, int *, cudaStream_t);
template int launch_step_fused2<__half>(const Shot<float, float> &, int, const WorkItem *, const int *, int, int, int,
                                        int, int, int *, cudaStream_t);

}  // namespace fd23
