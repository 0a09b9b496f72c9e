// Fused single-pass sweep for P-SV and SH on sm_103a.
//
// One launch advances every cell one full time step (stress update, point
// source, velocity update) and reads/writes each wavefield once, instead of
// the reference's two launches (PD/fd/cu_fd.cu:209-501, SH/fd/cu_fd.cu:77-288)
// plus host round trips for the source (PD/point_source/cu_point_source.cu)
// and receivers (PD/record/cu_record.cu:154).
//
// Data flow of one CTA (4 compute warps + 1 producer warp; every compute
// thread owns 4 adjacent cells of one row):
//   * The CTA works through a list of strips: output columns [x0, x0+TX),
//     rows [z0, z1).  It marches down in blocks of 4 rows.  Iteration i
//     updates the stress of rows z0-4+4i .. z0-1+4i on TX+8 columns (4 halo
//     columns each side, recomputed rather than exchanged) and the velocity of
//     rows z0-8+4i .. z0-5+4i on the TX output columns, so the velocity front
//     trails the stress front by exactly the 4 rows its z-stencil needs.
//   * The producer warp streams 4-row blocks of the stencil inputs (U, W or
//     V) into a ring of NUW slots and the point-wise operands (old stresses,
//     material) into NPW stages with tiled tensor copies (TMA,
//     cp.async.bulk.tensor.3d ... mbarrier::complete_tx): the wavefields of a
//     buffer set and the materials are each one allocation, viewed as
//     [field][row][column], so one box carries every field of a block -- four
//     copies per iteration.  Full/empty mbarrier pairs gate each slot, so the
//     producer runs ahead as far as the rings allow and the compute warps
//     never wait on it except for data.
//   * Updated stresses (after the point source) go to a 4-block smem ring that
//     feeds the velocity stencil, and straight to HBM; one barrier over the
//     compute warps per iteration orders the ring.
//   * Interior cells outside the CPML take a branch-free path with constant
//     coefficients; edge, CPML, free-surface and outside cells take the
//     general per-cell path.
//   * Wavefields and memory variables are ping-pong buffers (read set `par`,
//     write set 1-par), so the recomputed halo columns and rows of one CTA
//     never observe another CTA's new values.
//   * With a hybrid box (P-SV), add-ring stresses keep the value of their
//     old-stress slot, r + s, which the residual stress update stored there
//     before this launch; the rest of the box exchange runs in fd23_box.cu.
//   * All arrays use the zero-padded layout of fd23_internal.h, so every row
//     copy is in bounds and 16-byte aligned and the zero halo of the
//     reference needs no test.
//
// Arithmetic per cell is the canonical sequence of fd23_device.cuh, which is
// bit-identical to the CPU oracle and to the two-pass kernels.
//
// This header holds the kernel template; fd23_fused.cu instantiates the
// plain sweep and fd23_fused_punch.cu the sweep with tile step windows, so
// the two compile in parallel.
#pragma once
#include <climits>
#include <cstddef>
#include <cstdio>
#include <type_traits>

#include "fd23_device.cuh"
#include "fd23_kernels.h"
#include "fd23_pack.cuh"

namespace fd23 {

namespace {

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier + tiled tensor copy (TMA engine)
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
// tiled 3-D tensor copy (TMA) of one box at (x, y, z) of a tensor map
__device__ __forceinline__ void tma_load_2d(void *dst, const void *map, int x, int y, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_load_3d(void *dst, const void *map, int x, int y, int z, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait: gives up after ~2 s, sets the error flag and returns false.
// The first try is inlined; the polling loop is out of line.
__device__ __noinline__ bool mbar_wait_slow(uint64_t *bar, uint32_t parity, int *err_flag)
{
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t n = 0;; ++n) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((n & 255u) == 255u && globaltimer_ns() - t0 > 2000000000ull) {
            if (err_flag) atomicExch(err_flag, 1);
            return false;
        }
    }
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int *err_flag)
{
    return mbar_try_wait(bar, parity) || mbar_wait_slow(bar, parity, err_flag);
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
struct Vec4<__nv_bfloat16, float> : Vec4Half<__nv_bfloat16> {
    // a BF16 value is the upper half of the FP32 value it converts to
    // (exactly): one shift or one mask per value of a packed pair
    static __device__ __forceinline__ void ld(const __nv_bfloat16 *p, float v[4])
    {
        const uint2 t = *reinterpret_cast<const uint2 *>(p);
        v[0] = __uint_as_float(t.x << 16);
        v[1] = __uint_as_float(t.x & 0xffff0000u);
        v[2] = __uint_as_float(t.y << 16);
        v[3] = __uint_as_float(t.y & 0xffff0000u);
    }
};
template <>
struct Vec4<__half, float> : Vec4Half<__half> {};

// round C values through storage S (what a store followed by a load gives)
template <class S, class C>
__device__ __forceinline__ C through(C v) { return to_c<C>(to_s<S>(v)); }

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// barrier over the compute warps only, with an AND vote
__device__ __forceinline__ int compute_bar_and(int nthreads, int pred)
{
    int r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.s32 p, %1, 0;\n"
        " bar.red.and.pred q, 1, %2, p;\n selp.s32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"(pred), "r"(nthreads)
        : "memory");
    return r;
}
__device__ __forceinline__ void compute_bar(int nthreads)
{
    asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}

// 12 consecutive values x-4 .. x+7 of a stored row (three 4-wide loads)
template <class S, class C>
__device__ __forceinline__ void ld12(const S *p, C h[12])
{
    Vec4<S, C>::ld(p - 4, h);
    Vec4<S, C>::ld(p, h + 4);
    Vec4<S, C>::ld(p + 4, h + 8);
}
// x differences of the 4 cells at h[4..7]: backward (D-minus) / forward (D-plus)
template <class C>
__device__ __forceinline__ C dmx(const C h[12], int e, C c0, C c1, C c2, C c3)
{
    return comb<C>(c0, c1, c2, c3, h[4 + e] - h[3 + e], h[5 + e] - h[2 + e], h[6 + e] - h[1 + e],
                   h[7 + e] - h[e]);
}
template <class C>
__device__ __forceinline__ C dpx(const C h[12], int e, C c0, C c1, C c2, C c3)
{
    return comb<C>(c0, c1, c2, c3, h[5 + e] - h[4 + e], h[6 + e] - h[3 + e], h[7 + e] - h[2 + e],
                   h[8 + e] - h[1 + e]);
}
// z differences with interior coefficients, streaming two rows at a time:
// rows[k] points at row (j-4+k), column already applied.
template <class S, class C>
__device__ __forceinline__ void dmz4(const S *const rows[9], int off, C out[4])
{
    C a[4], b[4];
    Vec4<S, C>::ld(rows[4] + off, a);
    Vec4<S, C>::ld(rows[3] + off, b);
#pragma unroll
    for (int e = 0; e < 4; ++e) out[e] = Coef4<C>::c0 * (a[e] - b[e]);
    Vec4<S, C>::ld(rows[5] + off, a);
    Vec4<S, C>::ld(rows[2] + off, b);
#pragma unroll
    for (int e = 0; e < 4; ++e) out[e] = fmaC<C>(-Coef4<C>::c1, a[e] - b[e], out[e]);
    Vec4<S, C>::ld(rows[6] + off, a);
    Vec4<S, C>::ld(rows[1] + off, b);
#pragma unroll
    for (int e = 0; e < 4; ++e) out[e] = fmaC<C>(Coef4<C>::c2, a[e] - b[e], out[e]);
    Vec4<S, C>::ld(rows[7] + off, a);
    Vec4<S, C>::ld(rows[0] + off, b);
#pragma unroll
    for (int e = 0; e < 4; ++e) out[e] = fmaC<C>(-Coef4<C>::c3, a[e] - b[e], out[e]);
}
template <class S, class C>
__device__ __forceinline__ void dpz4(const S *const rows[9], int off, C out[4])
{
    C a[4], b[4];
    Vec4<S, C>::ld(rows[5] + off, a);
    Vec4<S, C>::ld(rows[4] + off, b);
#pragma unroll
    for (int e = 0; e < 4; ++e) out[e] = Coef4<C>::c0 * (a[e] - b[e]);
    Vec4<S, C>::ld(rows[6] + off, a);
    Vec4<S, C>::ld(rows[3] + off, b);
#pragma unroll
    for (int e = 0; e < 4; ++e) out[e] = fmaC<C>(-Coef4<C>::c1, a[e] - b[e], out[e]);
    Vec4<S, C>::ld(rows[7] + off, a);
    Vec4<S, C>::ld(rows[2] + off, b);
#pragma unroll
    for (int e = 0; e < 4; ++e) out[e] = fmaC<C>(Coef4<C>::c2, a[e] - b[e], out[e]);
    Vec4<S, C>::ld(rows[8] + off, a);
    Vec4<S, C>::ld(rows[1] + off, b);
#pragma unroll
    for (int e = 0; e < 4; ++e) out[e] = fmaC<C>(-Coef4<C>::c3, a[e] - b[e], out[e]);
}
// 4 stored values as packed operands
template <class S, class C>
__device__ __forceinline__ P4<C> ld4p(const S *p)
{
    if constexpr (std::is_same<S, float>::value) {
        const ulonglong2 t = *reinterpret_cast<const ulonglong2 *>(p);
        return P4<C>{t.x, t.y};
    } else {
        C v[4];
        Vec4<S, C>::ld(p, v);
        return P4<C>::from(v);
    }
}
// the z differences above on packed operands (same operation sequence)
template <class S, class C>
__device__ __forceinline__ P4<C> dmz4p(const S *const rows[9], int off)
{
    using P = P4<C>;
    const typename P::K k0 = P::splat(Coef4<C>::c0), k1 = P::splat(-Coef4<C>::c1), k2 = P::splat(Coef4<C>::c2),
                        k3 = P::splat(-Coef4<C>::c3);
    P d = P::mulk(k0, ld4p<S, C>(rows[4] + off) - ld4p<S, C>(rows[3] + off));
    d = P::fmak(k1, ld4p<S, C>(rows[5] + off) - ld4p<S, C>(rows[2] + off), d);
    d = P::fmak(k2, ld4p<S, C>(rows[6] + off) - ld4p<S, C>(rows[1] + off), d);
    return P::fmak(k3, ld4p<S, C>(rows[7] + off) - ld4p<S, C>(rows[0] + off), d);
}
template <class S, class C>
__device__ __forceinline__ P4<C> dpz4p(const S *const rows[9], int off)
{
    using P = P4<C>;
    const typename P::K k0 = P::splat(Coef4<C>::c0), k1 = P::splat(-Coef4<C>::c1), k2 = P::splat(Coef4<C>::c2),
                        k3 = P::splat(-Coef4<C>::c3);
    P d = P::mulk(k0, ld4p<S, C>(rows[5] + off) - ld4p<S, C>(rows[4] + off));
    d = P::fmak(k1, ld4p<S, C>(rows[6] + off) - ld4p<S, C>(rows[3] + off), d);
    d = P::fmak(k2, ld4p<S, C>(rows[7] + off) - ld4p<S, C>(rows[2] + off), d);
    return P::fmak(k3, ld4p<S, C>(rows[8] + off) - ld4p<S, C>(rows[1] + off), d);
}

// z differences with per-cell coefficient rows (edge cells)
template <class S, class C>
__device__ __forceinline__ void zcol(const S *const rows[9], int off, C v[9][4])
{
#pragma unroll
    for (int k = 0; k < 9; ++k) Vec4<S, C>::ld(rows[k] + off, v[k]);
}

template <class C>
__device__ __forceinline__ void cell_coef(int ix, int iz, int nx, int nz, C &c0, C &c1, C &c2, C &c3)
{
    int o = 4;
    if (ix >= 0 && ix < nx && iz >= 0 && iz < nz) o = stencil_order(ix, iz, nx, nz);
    c0 = Coef<C>::get(o, 0);
    c1 = Coef<C>::get(o, 1);
    c2 = Coef<C>::get(o, 2);
    c3 = Coef<C>::get(o, 3);
}

// ---------------------------------------------------------------------------
template <class S, class C, int WAVE, bool TABLE = false>
struct Cfg {
    static constexpr bool PSV = (WAVE == FD23_PSV);
    static constexpr int NCW = 4;              // compute warps (one per row of a 4-row block)
    static constexpr int NTH = 32 * (NCW + 1); // + one producer warp
    static constexpr int SW = 128;             // stress columns per strip
    static constexpr int TX = SW - 8;          // output columns per strip
    static constexpr int UWW = SW + 8;         // stencil-input row width
    static constexpr int PWOFF = sizeof(S) == 2 ? 4 : 0;  // keeps 16-byte alignment
    static constexpr int PWW = SW + 2 * PWOFF; // point-wise row width
    static constexpr int NV = PSV ? 2 : 1;     // stencil inputs of the stress update
    static constexpr int NT = PSV ? 3 : 2;     // stresses
    static constexpr int NMS = PSV ? 3 : 2;    // stress-update material
    static constexpr int NMV = PSV ? 2 : 1;    // velocity-update material
    static constexpr int NPF = NT + NMS + NMV; // point-wise fields per row
#ifndef FD23_FUSED_NPW
#define FD23_FUSED_NPW 2
#endif
#ifndef FD23_FUSED_NUW
#define FD23_FUSED_NUW 4
#endif
    // ring depths (NUW and NTR powers of two): sized so that three CTAs of the
    // 4-byte forms fit in the 228 KB of shared memory of one SM
    static constexpr int NUW = FD23_FUSED_NUW, NPW = FD23_FUSED_NPW, NTR = 4;
    // Tensor copies land 128-byte aligned: a stencil-input slot holds one box
    // [NV fields][4 rows][UWW], a point-wise stage three boxes (old stresses,
    // stress-update material, velocity-update material) [fields][4 rows][PWW],
    // each group starting on a 128-byte boundary.  Sizes in elements.
    static constexpr __host__ __device__ int al128(int bytes) { return (bytes + 127) / 128 * 128 / (int)sizeof(S); }
    static constexpr int UWF = 4 * UWW;                                  // field stride in a slot
    static constexpr int UW_SLOT = al128(NV * 4 * UWW * (int)sizeof(S));
    static constexpr int UW_ELEMS = NUW * UW_SLOT;
    static constexpr int PG_MS = al128(NT * 4 * PWW * (int)sizeof(S));
    // with a material table the material groups give way to one box of
    // 8 index rows (velocity rows, then stress rows) of kIdxBoxW bytes
    static constexpr int PG_MV = TABLE ? PG_MS : PG_MS + al128(NMS * 4 * PWW * (int)sizeof(S));
    static constexpr int PW_STAGE =
        TABLE ? PG_MS + al128(8 * kIdxBoxW) : PG_MV + al128(NMV * 4 * PWW * (int)sizeof(S));
    static constexpr int PW_ELEMS = NPW * PW_STAGE;
    static constexpr int TR_ELEMS = NTR * 4 * NT * SW;
    static constexpr int TAB_ELEMS = TABLE ? (NMS + NMV) * kTabEntries : 0;  // the table, per CTA
    // Uniform fast iterations (interior rows of all-interior warps with no
    // per-lane branch) for the single-shot 16-bit sweep, which is held by
    // instruction issue: 14 % fewer instructions, C1 FP16 9.11e10
    // cell-updates/s against 8.71e10, C3 FP16 1.26e11 against 1.10e11.  The
    // FP32 sweep is held by latency: 13 % fewer instructions gave C1 8.03e10
    // against 8.13e10.  In the batched sweeps the extra registers spill
    // (C4 FP32 7.28e10 against 7.81e10, C4 FP16 8.14e10 against 8.64e10).
    // The single-shot FP32 sweep has a second instantiation with them
    // (FASTF), which the autotuner picks where it is faster.
    static constexpr bool FAST_ITER = sizeof(S) == 2;
    // 16-bit storage: the strip's x-CPML coefficients (b, c, k of the four
    // staggered positions, 12 x SW) in shared memory for the general path,
    // which otherwise waits on a read-only global load per use (there is no
    // room for the table beside three CTAs of the 4-byte forms)
    static constexpr bool XTAB = sizeof(S) == 2;
    static constexpr int XT_ELEMS = XTAB ? 12 * SW : 0;
    // bytes the copies of one point-wise stage deliver
    static constexpr uint32_t PW_TX =
        TABLE ? (uint32_t)(NT * 4 * PWW * sizeof(S) + 8 * kIdxBoxW) : (uint32_t)(NPF * 4 * PWW * sizeof(S));
    // start of point-wise field f (stresses, then the two material groups) in a stage
    static constexpr __host__ __device__ int pw_field(int f)
    {
        return f < NT ? f * 4 * PWW : (f < NT + NMS ? PG_MS + (f - NT) * 4 * PWW : PG_MV + (f - NT - NMS) * 4 * PWW);
    }
    static constexpr int MAX_ITEMS = 4;
    static constexpr int MAX_TERMS = 16;
    // CTAs per SM the register budget is built for: three (shared memory
    // allows three) except FP64 (one).  With the stress ring in the
    // arithmetic type, a two-CTA budget let the single-shot P-SV 16-bit
    // sweep grow to 144 registers (two CTAs per SM), C1 FP16 7.67e10
    // cell-updates/s against 8.71e10 with three (measured)
    template <bool BATCH>
    static constexpr int minb() { return sizeof(S) == 8 ? 1 : 3; }
    // the stress ring holds arithmetic-type values (rounded through S when
    // written): the velocity update reads each of them many times
    static constexpr size_t RING_BYTES = (((size_t)(UW_ELEMS + PW_ELEMS + TAB_ELEMS) * sizeof(S) +
                                           (size_t)(TR_ELEMS + XT_ELEMS) * sizeof(C) + 15) &
                                          ~(size_t)15);
    static constexpr size_t SMEM = RING_BYTES + 256 /* 2*(NUW+NPW) barriers */ + MAX_ITEMS * 16 +
                                   (size_t)MAX_ITEMS * MAX_TERMS * 16;
};

struct ItemInfo {
    int x0, z0, z1, niter;  // rows [z0, z1), niter = (z1-z0)/4 + 2
};

// BATCH = false: one shot, described by the kernel parameter.  BATCH = true:
// the shot table `shots`; every CTA works on one shot (the shot of its first
// item) and copies that shot's descriptor into shared memory.
// PUNCH = true: the shots may carry tile step windows (usepunch).  Cells
// outside their tile's window keep their values; every item first drops the
// rows of tiles that are steady at this step (left alone at this step and
// the last, so both buffer sets already hold their values).
// TABLE = true: the shots carry material tables; the material of a cell is
// its index byte looked up in the CTA's shared-memory copy of the table.
// FASTF = true: the uniform fast iterations in a sweep whose storage does
// not take them by default (FP32; a separate instantiation, so that the
// plain one compiles as before).
template <class S, class C, int WAVE, bool BATCH, bool PUNCH, bool TABLE, bool FASTF = false>
__global__ void __launch_bounds__(Cfg<S, C, WAVE>::NTH, Cfg<S, C, WAVE>::template minb<BATCH>())
    fused_step(const __grid_constant__ Shot<S, C> sh_param, const Shot<S, C> *__restrict__ shots,
               const WorkItem *__restrict__ items, const int *__restrict__ item_off, int par, int it,
               int rec_index, int *err_flag)
{
    using K = Cfg<S, C, WAVE, TABLE>;
    constexpr bool PSV = K::PSV;
    constexpr int NCT = 32 * K::NCW;  // compute threads
    // an earlier launch gave up on a wait: do nothing until the host resets
    if (err_flag && *(volatile int *)err_flag) return;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // tensor copies need 128-byte aligned destinations: refuse to run otherwise
    if (smem_u32(smem_raw) & 127u) {
        if (threadIdx.x == 0 && err_flag) atomicExch(err_flag, 2);
        return;
    }
    S *uw_s = reinterpret_cast<S *>(smem_raw);
    S *pw_s = uw_s + K::UW_ELEMS;
    C *tr_s = reinterpret_cast<C *>(pw_s + K::PW_ELEMS);  // stress ring (arithmetic type)
    C *cx_s = tr_s + K::TR_ELEMS;                          // x-CPML coefficients of the strip (XTAB)
    S *tab_s = reinterpret_cast<S *>(cx_s + K::XT_ELEMS);  // the material table (TABLE only)
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw + K::RING_BYTES);
    uint64_t *full_uw = bars, *empty_uw = bars + K::NUW;
    uint64_t *full_pw = bars + 2 * K::NUW, *empty_pw = full_pw + K::NPW;
    ItemInfo *info = reinterpret_cast<ItemInfo *>(bars + 32);
    int4 *tlist = reinterpret_cast<int4 *>(info + K::MAX_ITEMS);
    __shared__ int tcount[K::MAX_ITEMS];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ibeg = item_off[blockIdx.x], iend = item_off[blockIdx.x + 1];
    int nitems = min(iend - ibeg, K::MAX_ITEMS);

    const Shot<S, C> *shp;
    if constexpr (BATCH) {
        // the descriptor up to the fields only single shots use (the two-step
        // sweep's, the box), as 16-byte words: three CTAs per SM still fit
        using ShotT = Shot<S, C>;
        constexpr int kHead = (int)((offsetof(ShotT, maps2) + 15) / 16 * 16);
        static_assert(kHead <= (int)sizeof(ShotT) && sizeof(ShotT) % 16 == 0, "descriptor head");
        __shared__ alignas(16) unsigned char sh_head[kHead];
        const int4 *src = reinterpret_cast<const int4 *>(shots + items[ibeg].shot);
        int4 *dst = reinterpret_cast<int4 *>(sh_head);
        for (int w = tid; w < kHead / 16; w += K::NTH) dst[w] = src[w];
        __syncthreads();
        shp = reinterpret_cast<const Shot<S, C> *>(sh_head);
    } else {
        shp = &sh_param;
    }
    const Shot<S, C> &sh = *shp;
    const int nx = sh.nx, nz = sh.nz, npml = sh.npml, pitch = sh.pitch;
    const long long origin = sh.origin;

    // read / write pointers selected once (compile-time indices only)
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
    if constexpr (PUNCH) {
        // ---- tile step windows: keep each item's rows from the first to the
        // last tile row that is not steady at this step (the windows are
        // static, so this runs ahead of the dependency wait) ----
        __shared__ int span_lo[K::MAX_ITEMS], span_hi[K::MAX_ITEMS], n_live;
        const Punch pu = sh.punch;
        if (pu.win) {
            if (tid < nitems) {
                span_lo[tid] = INT_MAX;
                span_hi[tid] = -1;
            }
            __syncthreads();
            for (int k = 0; k < nitems; ++k) {
                const ItemInfo I = info[k];
                const int tz0 = I.z0 / kPunchTZ, tz1 = (min(I.z1, nz) - 1) / kPunchTZ;
                const int tx0 = max(I.x0, 0) / kPunchTX, tx1 = (min(I.x0 + K::TX, nx) - 1) / kPunchTX;
                for (int tz = tz0 + tid; tz <= tz1; tz += K::NTH) {
                    bool live = false;
                    for (int tx = tx0; tx <= tx1; ++tx) live |= !punch_steady(__ldg(&pu.win[tz * pu.nbx + tx]), it);
                    if (live) {
                        atomicMin(&span_lo[k], tz);
                        atomicMax(&span_hi[k], tz);
                    }
                }
                // cells with a source term change while the source runs and
                // once more when it stops (the two sets differ there)
                if (it <= sh.tamp_nt)
                    for (int t = tid; t < sh.nterms; t += K::NTH) {
                        const int4 tm = sh.terms[t];
                        if (tm.y >= I.x0 && tm.y < I.x0 + K::TX && tm.z >= I.z0 && tm.z < I.z1) {
                            atomicMin(&span_lo[k], tm.z / kPunchTZ);
                            atomicMax(&span_hi[k], tm.z / kPunchTZ);
                        }
                    }
            }
            __syncthreads();
            if (tid == 0) {
                // narrow the items, drop the empty ones (the source lists move along)
                int n = 0;
                for (int k = 0; k < nitems; ++k) {
                    if (span_hi[k] < 0) continue;
                    ItemInfo I = info[k];
                    I.z0 = max(I.z0, span_lo[k] * kPunchTZ);
                    I.z1 = min(I.z1, (span_hi[k] + 1) * kPunchTZ);
                    I.niter = (I.z1 - I.z0) / 4 + 2;
                    info[n] = I;
                    tcount[n] = tcount[k];
                    for (int t = 0; t < tcount[k]; ++t) tlist[n * K::MAX_TERMS + t] = tlist[k * K::MAX_TERMS + t];
                    ++n;
                }
                n_live = n;
            }
            __syncthreads();
            nitems = n_live;
        }
    }
    if constexpr (TABLE) {
        // the table is static: copy it ahead of the dependency wait
        for (int k = tid; k < K::TAB_ELEMS; k += K::NTH) tab_s[k] = sh.mtab[k];
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
    // Programmatic dependent launch: the next step's grid may start its
    // prologue now; it waits (griddepcontrol.wait) before it touches any
    // wavefield or memory variable, all of which this grid still reads/writes.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");

    int total_iters = 0;
    for (int k = 0; k < nitems; ++k) total_iters += info[k].niter;

    // ======================= producer warp =======================
    if (warp == K::NCW) {
        // stencil-input stream element e -> item k, block b
        auto issue_uw = [=](int e) {
            int k = 0, base = 0;
            while (k < nitems - 1 && e >= base + info[k].niter + 2) { base += info[k].niter + 2; ++k; }
            const int b = e - base;
            const ItemInfo I = info[k];
            const int slot = e % K::NUW;
            const int r0 = I.z0 - 8 + 4 * b;
            // one box: NV fields x rows r0 .. r0+3 x columns x0-8 .. x0+UWW-9
            if (lane == 0) {
                mbar_arrive_expect_tx(&full_uw[slot], (uint32_t)(K::NV * 4 * K::UWW * sizeof(S)));
                tma_load_3d(uw_s + slot * K::UW_SLOT, &sh.maps->uw[par], kXPad + I.x0 - 8, kZPad + r0, 0,
                            &full_uw[slot]);
            }
        };
        // point-wise operands of iteration i of item I into stage g % NPW
        // part 0: everything; 1: arm the stage and copy the material rows only
        // (they do not depend on the previous step); 2: the old stresses only
        auto issue_pw = [=](int g, const ItemInfo &I, int i, int part) {
            const int slot = g % K::NPW;
            if (lane == 0) {
                S *st = pw_s + slot * K::PW_STAGE;
                if (part != 2) mbar_arrive_expect_tx(&full_pw[slot], K::PW_TX);
                // old stresses and stress-update material on stress rows,
                // velocity-update material on velocity rows
                const int xs = kXPad + I.x0 - 4 - K::PWOFF;
                const int ys = kZPad + I.z0 - 4 + 4 * i, yv = kZPad + I.z0 - 8 + 4 * i;
                if (part != 1) tma_load_3d(st, &sh.maps->t[par], xs, ys, K::NV, &full_pw[slot]);
                if (part != 2) {
                    if constexpr (TABLE) {
                        // index rows yv .. yv+7 from the 16-byte boundary at or before xs
                        tma_load_2d(st + K::PG_MS, &sh.maps->idx, xs & ~15, yv, &full_pw[slot]);
                    } else {
                        tma_load_3d(st + K::PG_MS, &sh.maps->ms, xs, ys, 0, &full_pw[slot]);
                        tma_load_3d(st + K::PG_MV, &sh.maps->mv, xs, yv, K::NMS, &full_pw[slot]);
                    }
                }
            }
        };
        bool ok = true;
        int e_uw = 0, g_pw = 0;
        int k = 0, base_it = 0, base_uw = 0;
        // material rows of the first stages ahead of the dependency wait
        const int npre = min(K::NPW, total_iters);
        {
            int kk = 0, bit = 0;
            for (int g = 0; g < npre; ++g) {
                while (g >= bit + info[kk].niter) { bit += info[kk].niter; ++kk; }
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
    // ---- receivers of the previous step (buffer set `par` is read-only here) ----
    if (rec_index >= 0) {
#pragma unroll
        for (int c = 0; c < K::NV + K::NT; ++c)
            for (int r = ((int)blockIdx.x - sh.cta0) * NCT + tid; r < sh.nrec[c]; r += sh.ncta * NCT)
                sh.seis[c][(long long)rec_index * sh.nrec[c] + r] = to_c<C>(rd[c][sh.rec[c][r]]);
    }

    const int grp = warp;  // row of the 4-row block this warp updates
    const C *cp = sh.cpml;
    const int B = sh.cpml_blk;
    bool ok = true;
    int uw_ready = 0, gflat = 0, uw_base = 0;
    for (int k = 0; k < nitems && ok; ++k) {
        const ItemInfo I = info[k];
        const int ntl = tcount[k];
        const int4 *tl = tlist + k * K::MAX_TERMS;
        const int x = I.x0 - 4 + 4 * lane;  // first of this thread's 4 cells
        // lanes 1 .. 30 own their cells (0 and 31: halo); a strip whose origin
        // lies left of column 0 owns no cells there (x is a multiple of 4)
        const bool own_x = lane >= 1 && lane <= 30 && x >= 0;
        // byte offset of this thread's 4 cells in a row of the index box
        const int ixo = ((kXPad + I.x0 - 4 - K::PWOFF) & 15) + K::PWOFF + 4 * lane;
        // the 4 cells are interior (8th order), outside the x-CPML and inside the grid
        const bool xfast = x >= max(4, npml) && x + 3 <= min(nx - 5, nx - npml - 1);
        // x-CPML coefficient kc (0 b, 1 c, 2 k) of staggered position ac at
        // column ix of this item's strip
        auto cxc = [&](int kc, int ac, int ix) -> C {
            if constexpr (K::XTAB) return cx_s[(4 * kc + ac) * K::SW + 4 * lane + (ix - x)];  // ix - x: the cell
            else return __ldg(cp + (kc * B + ac * nx + ix));
        };
        if constexpr (K::XTAB) {
            // an item whose strip reaches into the x-CPML fills the table; the
            // test is the same for every compute warp (one item for all)
            if (npml > 0 && (I.x0 - 4 < npml || I.x0 - 4 + K::SW > nx - npml)) {
                compute_bar(NCT);  // the previous item's reads of the table are done
                for (int q = tid; q < K::XT_ELEMS; q += NCT) {
                    const int r = q / K::SW, ix = I.x0 - 4 + (q - r * K::SW);
                    cx_s[q] = ix >= 0 && ix < nx ? __ldg(cp + ((r >> 2) * B + (r & 3) * nx + ix)) : (C)0;
                }
                compute_bar(NCT);
            }
        }
        // ---- interior arithmetic (8th order, no CPML), shared by the uniform
        // fast iteration below and the per-lane path: one operation sequence.
        // Stress: packed operands (x differences stay per cell);
        // gam = fma(2, mu, lam) equals lam + 2*mu (2*mu is exact)
        auto stress_interior = [&](const S *const *urow, const C (*told)[4], const C (*ms)[4], C (*tnew)[4]) {
            constexpr C c0 = Coef4<C>::c0, c1 = Coef4<C>::c1, c2 = Coef4<C>::c2, c3 = Coef4<C>::c3;
            using P = P4<C>;
            if constexpr (PSV) {
                C h[12];
                C ux[4], wx[4];
                ld12<S, C>(urow[4], h);
#pragma unroll
                for (int e = 0; e < 4; ++e) ux[e] = dmx<C>(h, e, c0, c1, c2, c3);
                ld12<S, C>(urow[4] + K::UWF, h);
#pragma unroll
                for (int e = 0; e < 4; ++e) wx[e] = dpx<C>(h, e, c0, c1, c2, c3);
                const P lam = P::from(ms[0]), mua = P::from(ms[2]);
                const P gam = P::fmak(P::splat((C)2), P::from(ms[1]), lam);
                const P UX = P::from(ux), WX = P::from(wx);
                P t0 = P::fma(gam, UX, P::from(told[0]));
                P t2 = P::fma(lam, UX, P::from(told[2]));
                P t1 = P::fma(mua, WX, P::from(told[1]));
                const P UZ = dmz4p<S, C>(urow, 0), WZ = dpz4p<S, C>(urow, K::UWF);
                P::fma(lam, WZ, t0).to(tnew[0]);
                P::fma(gam, WZ, t2).to(tnew[2]);
                P::fma(mua, UZ, t1).to(tnew[1]);
            } else {
                C h[12], dx[4];
                ld12<S, C>(urow[4], h);
#pragma unroll
                for (int e = 0; e < 4; ++e) dx[e] = dpx<C>(h, e, c0, c1, c2, c3);
                P::fma(P::from(ms[0]), P::from(dx), P::from(told[0])).to(tnew[0]);
                P::fma(P::from(ms[1]), dmz4p<S, C>(urow, 0), P::from(told[1])).to(tnew[1]);
            }
        };
        auto velocity_interior = [&](const C *const *trow, const C (*mv)[4], const C (*vold)[4], C (*vnew)[4]) {
            constexpr C c0 = Coef4<C>::c0, c1 = Coef4<C>::c1, c2 = Coef4<C>::c2, c3 = Coef4<C>::c3;
            using P = P4<C>;
            if constexpr (PSV) {
                C h[12], dx[4];
                const P bu = P::from(mv[0]), bw = P::from(mv[1]);
                ld12<C, C>(trow[4], h);  // Txx
#pragma unroll
                for (int e = 0; e < 4; ++e) dx[e] = dpx<C>(h, e, c0, c1, c2, c3);
                P u = P::fma(bu, P::from(dx), P::from(vold[0]));
                ld12<C, C>(trow[4] + K::SW, h);  // Txz
#pragma unroll
                for (int e = 0; e < 4; ++e) dx[e] = dmx<C>(h, e, c0, c1, c2, c3);
                P w = P::fma(bw, P::from(dx), P::from(vold[1]));
                P::fma(bu, dpz4p<C, C>(trow, K::SW), u).to(vnew[0]);      // d/dz Txz
                P::fma(bw, dmz4p<C, C>(trow, 2 * K::SW), w).to(vnew[1]);  // d/dz Tzz
            } else {
                C h[12], dx[4];
                const P bv = P::from(mv[0]);
                ld12<C, C>(trow[4], h);  // Tx
#pragma unroll
                for (int e = 0; e < 4; ++e) dx[e] = dmx<C>(h, e, c0, c1, c2, c3);
                const P t = P::fma(bv, P::from(dx), P::from(vold[0]));
                P::fma(bv, dpz4p<C, C>(trow, K::SW), t).to(vnew[0]);  // d/dz Tz
            }
        };
        // Uniform fast iterations for this warp: every lane (the halo lanes
        // too) x-interior, no source term in the item, no hybrid box.  An
        // iteration is fast when its stress row j and its velocity row j-4
        // are z-interior rows (8th order, outside the z-CPML) and the
        // velocity row belongs to the item, i.e. j in [fjlo, fjhi] (an empty
        // range when the item is not fast): every lane then takes the
        // interior arithmetic with no per-lane branch.
        constexpr bool kFast = (K::FAST_ITER || FASTF) && !BATCH && !PUNCH;
        bool item_fast = kFast && __all_sync(0xffffffffu, xfast) && ntl == 0;
        if constexpr (PSV && std::is_same<S, C>::value && !BATCH) item_fast = item_fast && !sh.box.on;
        const int fjlo = item_fast ? max(I.z0, max(4, sh.topabsorb ? npml : 0)) + 4 : INT_MAX;
        const int fjhi = min(nz - 5, nz - npml - 1);
        for (int i = 0; i < I.niter; ++i, ++gflat) {
            for (; ok && uw_ready <= uw_base + i + 2; ++uw_ready)
                ok = mbar_wait_bounded(&full_uw[uw_ready % K::NUW], (uint32_t)((uw_ready / K::NUW) & 1), err_flag);
            if (ok) ok = mbar_wait_bounded(&full_pw[gflat % K::NPW], (uint32_t)((gflat / K::NPW) & 1), err_flag);
            const S *pws = pw_s + (gflat % K::NPW) * K::PW_STAGE;
            auto pwrow = [=](int f) { return pws + K::pw_field(f) + grp * K::PWW + K::PWOFF + 4 * lane; };
            // stress ring row r (absolute): ring row (4*(gflat-i) + r-(z0-4)) mod 4*NTR
            const int tseq = 4 * (gflat - i) - (I.z0 - 4);
            auto trrow = [=](int r) -> const C * {
                return tr_s + ((tseq + r) & (4 * K::NTR - 1)) * (K::NT * K::SW) + 4 * lane;
            };
            const int jf = I.z0 - 4 + 4 * i + grp;  // stress row; the velocity row is jf - 4
            // (an SH item starting at row 0 meets its free-surface barrier at
            // i = 1, where jf < 4: never fast, so every warp takes it)
            if (kFast && jf >= fjlo && jf <= fjhi) {
                // ---- stress of row jf, every lane ----
                {
                    const S *urow[9];
                    const int rseq = 4 * (uw_base + i) + grp;
#pragma unroll
                    for (int d = 0; d < 9; ++d) {
                        const int r = (rseq + d) & (4 * K::NUW - 1);
                        urow[d] = uw_s + (r >> 2) * K::UW_SLOT + (r & 3) * K::UWW + 4 * lane + 4;
                    }
                    C told[K::NT][4], ms[K::NMS][4], tnew[K::NT][4];
#pragma unroll
                    for (int f = 0; f < K::NT; ++f) Vec4<S, C>::ld(pwrow(f), told[f]);
                    if constexpr (TABLE) {
                        const uint32_t q = *reinterpret_cast<const uint32_t *>(
                            reinterpret_cast<const unsigned char *>(pws + K::PG_MS) + (4 + grp) * kIdxBoxW + ixo);
#pragma unroll
                        for (int m = 0; m < K::NMS; ++m)
#pragma unroll
                            for (int e = 0; e < 4; ++e)
                                ms[m][e] = to_c<C>(tab_s[m * kTabEntries + ((q >> (8 * e)) & 255u)]);
                    } else {
#pragma unroll
                        for (int m = 0; m < K::NMS; ++m) Vec4<S, C>::ld(pwrow(K::NT + m), ms[m]);
                    }
                    stress_interior(urow, told, ms, tnew);
                    C *tr = tr_s + ((4 * gflat + grp) & (4 * K::NTR - 1)) * (K::NT * K::SW) + 4 * lane;
#pragma unroll
                    for (int f = 0; f < K::NT; ++f) {
                        C r[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) r[e] = through<S, C>(tnew[f][e]);
                        Vec4<C, C>::st(tr + f * K::SW, r);
                    }
                    if (own_x && jf < I.z1) {
                        const long long o = origin + (long long)jf * pitch + x;
#pragma unroll
                        for (int f = 0; f < K::NT; ++f) Vec4<S, C>::st(wr[K::NV + f] + o, tnew[f]);
                    }
                }
                ok = compute_bar_and(NCT, ok) != 0;
                if (!ok) break;
                // ---- velocity of row jf - 4, every lane.  The halo lanes 0 and
                // 31 read their neighbours' operands (lanes 1 and 30), so a
                // warp's loads span the same shared-memory wavefronts as the
                // owned lanes' alone, and their results are not stored ----
                {
                    const int a = jf - 4;
                    // (the lane id read here, not held across the loop)
                    uint32_t lid;
                    asm volatile("mov.u32 %0, %%laneid;" : "=r"(lid));
                    const int dl = lid == 0 ? 4 : (lid == 31 ? -4 : 0);  // 0 on the owned lanes
                    const C *trow[9];
#pragma unroll
                    for (int d = 0; d < 9; ++d) trow[d] = trrow(a - 4 + d) + dl;
                    C mv[K::NMV][4];
                    if constexpr (TABLE) {
                        const uint32_t q = *reinterpret_cast<const uint32_t *>(
                            reinterpret_cast<const unsigned char *>(pws + K::PG_MS) + grp * kIdxBoxW + ixo + dl);
#pragma unroll
                        for (int m = 0; m < K::NMV; ++m)
#pragma unroll
                            for (int e = 0; e < 4; ++e)
                                mv[m][e] = to_c<C>(tab_s[(K::NMS + m) * kTabEntries + ((q >> (8 * e)) & 255u)]);
                    } else {
#pragma unroll
                        for (int m = 0; m < K::NMV; ++m) Vec4<S, C>::ld(pwrow(K::NT + K::NMS + m) + dl, mv[m]);
                    }
                    const int vr = (4 * (uw_base + i) + grp) & (4 * K::NUW - 1);
                    const S *vrow = uw_s + (vr >> 2) * K::UW_SLOT + (vr & 3) * K::UWW + 4 * lane + 4 + dl;
                    C vold[K::NV][4], vnew[K::NV][4];
#pragma unroll
                    for (int v = 0; v < K::NV; ++v) Vec4<S, C>::ld(vrow + v * K::UWF, vold[v]);
                    velocity_interior(trow, mv, vold, vnew);
                    if (own_x) {
                        const long long o = origin + (long long)a * pitch + x;
#pragma unroll
                        for (int v = 0; v < K::NV; ++v) Vec4<S, C>::st(wr[v] + o, vnew[v]);
                    }
                }
            } else {
            // ================= stress: row j, cells x .. x+3 =================
            {
                const int j = I.z0 - 4 + 4 * i + grp;
                // stencil rows j-4 .. j+4: ring row (4*(uw_base+i) + grp + d) mod 4*NUW
                const S *urow[9];
                const int rseq = 4 * (uw_base + i) + grp;
#pragma unroll
                for (int d = 0; d < 9; ++d) {
                    const int r = (rseq + d) & (4 * K::NUW - 1);
                    urow[d] = uw_s + (r >> 2) * K::UW_SLOT + (r & 3) * K::UWW + 4 * lane + 4;
                }
                const bool inrow = j >= 0 && j < nz;
                const bool zfast = j >= 4 && j <= nz - 5 && j < nz - npml && !(sh.topabsorb && j < npml);
                // the 4 cells share one tile: updated at this step or not
                bool act = true;
                if constexpr (PUNCH) act = punch_active(sh.punch, min(max(x, 0), nx - 1), min(max(j, 0), nz - 1), it);
                C tnew[K::NT][4];
                C told[K::NT][4], ms[K::NMS][4];
#pragma unroll
                for (int f = 0; f < K::NT; ++f) Vec4<S, C>::ld(pwrow(f), told[f]);
                if constexpr (TABLE) {
                    const uint32_t q = *reinterpret_cast<const uint32_t *>(
                        reinterpret_cast<const unsigned char *>(pws + K::PG_MS) + (4 + grp) * kIdxBoxW + ixo);
#pragma unroll
                    for (int m = 0; m < K::NMS; ++m)
#pragma unroll
                        for (int e = 0; e < 4; ++e) ms[m][e] = to_c<C>(tab_s[m * kTabEntries + ((q >> (8 * e)) & 255u)]);
                } else {
#pragma unroll
                    for (int m = 0; m < K::NMS; ++m) Vec4<S, C>::ld(pwrow(K::NT + m), ms[m]);
                }
                if (xfast && zfast) {
                    stress_interior(urow, told, ms, tnew);
                } else if (!PUNCH && xfast && j >= 4 && j <= nz - 5) {
                    // x-interior cells of a z-CPML row (8th order everywhere): the
                    // interior's packed differences, then the general path's chains
                    // with the z memory variables (coefficients uniform in the row)
                    if constexpr (!PSV) {
                        constexpr C c0 = Coef4<C>::c0, c1 = Coef4<C>::c1, c2 = Coef4<C>::c2, c3 = Coef4<C>::c3;
                        const bool top = j < npml && sh.topabsorb;
                        const long long pz0 = top ? (long long)j * nx + x : (long long)(npml + nz - 1 - j) * nx + x;
                        C psv[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) psv[e] = prd[3][pz0 + e];
                        C h[12], dxv[4], dzv[4];
                        ld12<S, C>(urow[4], h);
#pragma unroll
                        for (int e = 0; e < 4; ++e) dxv[e] = dpx<C>(h, e, c0, c1, c2, c3);
                        dmz4p<S, C>(urow, 0).to(dzv);
                        const int zb = 2 * nx;
                        const C bZ = __ldg(cp + (zb + nz + j)), cZ = __ldg(cp + (B + zb + nz + j)),
                                kZ = __ldg(cp + (2 * B + zb + nz + j));
                        const bool own_row = j >= I.z0 && j < I.z1;
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const C a = fmaC<C>(bZ, psv[e], cZ * dzv[e]);
                            tnew[0][e] = fmaC<C>(ms[0][e], dxv[e], told[0][e]);
                            tnew[1][e] = fmaC<C>(ms[1][e], fmaC<C>(dzv[e], kZ, a), told[1][e]);
                            const int ix = x + e;
                            if (own_row && ix >= I.x0 && ix < I.x0 + K::TX) pwr[3][pz0 + e] = a;
                        }
                    }
                    if constexpr (PSV) {
                        constexpr C c0 = Coef4<C>::c0, c1 = Coef4<C>::c1, c2 = Coef4<C>::c2, c3 = Coef4<C>::c3;
                        const bool top = j < npml && sh.topabsorb;
                        const long long pz0 = top ? (long long)j * nx + x : (long long)(npml + nz - 1 - j) * nx + x;
                        C psw[4], psu[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            psw[e] = prd[7][pz0 + e];
                            psu[e] = prd[6][pz0 + e];
                        }
                        C h[12], ux[4], wx[4], uz[4], wz[4];
                        ld12<S, C>(urow[4], h);
#pragma unroll
                        for (int e = 0; e < 4; ++e) ux[e] = dmx<C>(h, e, c0, c1, c2, c3);
                        ld12<S, C>(urow[4] + K::UWF, h);
#pragma unroll
                        for (int e = 0; e < 4; ++e) wx[e] = dpx<C>(h, e, c0, c1, c2, c3);
                        dmz4p<S, C>(urow, 0).to(uz);
                        dpz4p<S, C>(urow, K::UWF).to(wz);
                        const int zb = 4 * nx;
                        const C bW = __ldg(cp + (zb + 3 * nz + j)), cW = __ldg(cp + (B + zb + 3 * nz + j)),
                                kW = __ldg(cp + (2 * B + zb + 3 * nz + j));
                        const C bU = __ldg(cp + (zb + 2 * nz + j)), cU = __ldg(cp + (B + zb + 2 * nz + j)),
                                kU = __ldg(cp + (2 * B + zb + 2 * nz + j));
                        const bool own_row = j >= I.z0 && j < I.z1;
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            C pw = psw[e], pu = psu[e];
                            if (act) {
                                const C lam = ms[0][e], mu = ms[1][e], mua = ms[2][e];
                                const C gam = lam + (C)2 * mu;
                                C txx = told[0][e], txz = told[1][e], tzz = told[2][e];
                                txx = fmaC<C>(gam, ux[e], txx);
                                tzz = fmaC<C>(lam, ux[e], tzz);
                                txz = fmaC<C>(mua, wx[e], txz);
                                pw = fmaC<C>(bW, psw[e], cW * wz[e]);
                                const C t = fmaC<C>(wz[e], kW, pw);
                                txx = fmaC<C>(lam, t, txx);
                                tzz = fmaC<C>(gam, t, tzz);
                                pu = fmaC<C>(bU, psu[e], cU * uz[e]);
                                txz = fmaC<C>(mua, fmaC<C>(uz[e], kU, pu), txz);
                                tnew[0][e] = txx;
                                tnew[1][e] = txz;
                                tnew[2][e] = tzz;
                            }
                            const int ix = x + e;
                            if (own_row && ix >= I.x0 && ix < I.x0 + K::TX) {
                                pwr[7][pz0 + e] = pw;
                                pwr[6][pz0 + e] = pu;
                            }
                        }
                    }
                } else {
                    // ---- general cells: edges (reduced order), CPML, free surface, outside ----
                    // memory variables first, so their load latency overlaps the derivatives.
                    // The CPML coefficients are read through the read-only path
                    // (__ldg): written once at set-up, so their loads may move
                    // ahead of this thread's memory-variable stores.
                    C psx[2][4], psz[2][4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int ix = x + e;
                        psx[0][e] = psx[1][e] = psz[0][e] = psz[1][e] = (C)0;
                        if (!inrow || ix < 0 || ix >= nx) continue;
                        const bool top = j < npml && sh.topabsorb;
                        if (ix < npml || ix >= nx - npml) {
                            const long long px = ix < npml ? (long long)ix + (long long)j * 2 * npml
                                                           : (long long)npml + nx - 1 - ix + (long long)j * 2 * npml;
                            if constexpr (PSV) { psx[0][e] = prd[2][px]; psx[1][e] = prd[3][px]; }
                            else psx[0][e] = prd[1][px];
                        }
                        if (top || j >= nz - npml) {
                            const long long pz = top ? (long long)j * nx + ix : (long long)(npml + nz - 1 - j) * nx + ix;
                            if constexpr (PSV) { psz[0][e] = prd[7][pz]; psz[1][e] = prd[6][pz]; }
                            else psz[0][e] = prd[3][pz];
                        }
                    }
                    C cc[4][4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) cell_coef<C>(x + e, j, nx, nz, cc[e][0], cc[e][1], cc[e][2], cc[e][3]);
                    // derivatives field by field: P-SV ux, uz (U) then wx, wz (W); SH dxV, dzV
                    C dA[4], dB[4], dC[4], dD[4];
                    {
                        C h[12], zv[9][4];
                        ld12<S, C>(urow[4], h);
                        zcol<S, C>(urow, 0, zv);
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            
                            dA[e] = PSV ? dmx<C>(h, e, cc[e][0], cc[e][1], cc[e][2], cc[e][3]) : dpx<C>(h, e, cc[e][0], cc[e][1], cc[e][2], cc[e][3]);
                            dB[e] = comb<C>(cc[e][0], cc[e][1], cc[e][2], cc[e][3], zv[4][e] - zv[3][e], zv[5][e] - zv[2][e],
                                            zv[6][e] - zv[1][e], zv[7][e] - zv[0][e]);
                        }
                    }
                    if constexpr (PSV) {
                        C h[12], zv[9][4];
                        ld12<S, C>(urow[4] + K::UWF, h);
                        zcol<S, C>(urow, K::UWF, zv);
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
#pragma unroll
                        for (int f = 0; f < K::NT; ++f) tnew[f][e] = told[f][e];
                        if (!inrow || ix < 0 || ix >= nx) {
#pragma unroll
                            for (int f = 0; f < K::NT; ++f) tnew[f][e] = (C)0;
                            continue;
                        }
                        const bool own = ix >= I.x0 && ix < I.x0 + K::TX && j >= I.z0 && j < I.z1;
                        const bool xp = ix < npml || ix >= nx - npml;
                        const bool top = j < npml && sh.topabsorb;
                        const bool zp = top || j >= nz - npml;
                        const long long px = ix < npml ? (long long)ix + (long long)j * 2 * npml
                                                       : (long long)npml + nx - 1 - ix + (long long)j * 2 * npml;
                        const long long pz = top ? (long long)j * nx + ix : (long long)(npml + nz - 1 - j) * nx + ix;
                        if constexpr (PUNCH) {
                            if (!act) {  // outside the step window: memory variables carry over too
                                if (own && xp) {
                                    if constexpr (PSV) { pwr[2][px] = psx[0][e]; pwr[3][px] = psx[1][e]; }
                                    else pwr[1][px] = psx[0][e];
                                }
                                if (own && zp) {
                                    if constexpr (PSV) { pwr[7][pz] = psz[0][e]; pwr[6][pz] = psz[1][e]; }
                                    else pwr[3][pz] = psz[0][e];
                                }
                                continue;
                            }
                        }
                        if constexpr (PSV) {
                            const C ux = dA[e], uz = dB[e], wx = dC[e], wz = dD[e];
                            const C lam = ms[0][e], mu = ms[1][e], mua = ms[2][e];
                            const C gam = lam + (C)2 * mu;
                            C txx = told[0][e], txz = told[1][e], tzz = told[2][e];
                            // x chain, PD/fd/cu_fd.cu:303-326
                            if (xp) {
                                const C pu = fmaC<C>(cxc(0, 2, ix), psx[0][e], cxc(1, 2, ix) * ux);
                                const C t = fmaC<C>(ux, cxc(2, 2, ix), pu);
                                txx = fmaC<C>(gam, t, txx);
                                tzz = fmaC<C>(lam, t, tzz);
                                const C pw = fmaC<C>(cxc(0, 3, ix), psx[1][e], cxc(1, 3, ix) * wx);
                                txz = fmaC<C>(mua, fmaC<C>(wx, cxc(2, 3, ix), pw), txz);
                                if (own) { pwr[2][px] = pu; pwr[3][px] = pw; }
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
                                if (own) { pwr[7][pz] = pw; pwr[6][pz] = pu; }
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
                        } else {
                            // SH stress, SH/fd/cu_fd.cu:77-171; cells skipped there keep their values
                            if (ix == 0 || ix >= nx - 1 || j >= nz - 1) {
                                if (own && xp) pwr[1][px] = psx[0][e];
                                if (own && zp) pwr[3][pz] = psz[0][e];
                                continue;
                            }
                            const C dxv = dA[e], dzv = dB[e];
                            const C mux = ms[0][e], muz = ms[1][e];
                            C tx = told[0][e], tz = told[1][e];
                            if (xp) {
                                const C a = fmaC<C>(cxc(0, 1, ix), psx[0][e], cxc(1, 1, ix) * dxv);
                                if (own) pwr[1][px] = a;
                                tx = fmaC<C>(mux, fmaC<C>(dxv, cxc(2, 1, ix), a), tx);
                            } else {
                                tx = fmaC<C>(mux, dxv, tx);
                            }
                            if (zp) {
                                const int zb = 2 * nx;
                                const C a = fmaC<C>(__ldg(cp + (zb + nz + j)), psz[0][e], __ldg(cp + (B + zb + nz + j)) * dzv);
                                if (own) pwr[3][pz] = a;
                                tz = fmaC<C>(muz, fmaC<C>(dzv, __ldg(cp + (2 * B + zb + nz + j)), a), tz);
                            } else {
                                tz = fmaC<C>(muz, dzv, tz);
                            }
                            tnew[0][e] = tx;
                            tnew[1][e] = tz;
                        }
                    }
                }
                if constexpr (PUNCH) {
                    if (!act)
#pragma unroll
                        for (int f = 0; f < K::NT; ++f)
#pragma unroll
                            for (int e = 0; e < 4; ++e) tnew[f][e] = told[f][e];
                }
                // ---- stress ring (every column) ----
                C *tr = tr_s + ((4 * gflat + grp) & (4 * K::NTR - 1)) * (K::NT * K::SW) + 4 * lane;
#pragma unroll
                for (int f = 0; f < K::NT; ++f) {
                    C r[4];  // the values the stored stresses will hold
#pragma unroll
                    for (int e = 0; e < 4; ++e) r[e] = through<S, C>(tnew[f][e]);
                    Vec4<C, C>::st(tr + f * K::SW, r);
                }
                // ---- point source (terms in list order), as read-modify-writes of
                // the ring cells just written (keeps tnew in registers) ----
                if (ntl > 0) {
                    bool hit = false;
                    for (int t = 0; t < ntl; ++t) {
                        const int4 tm = tl[t];  // (field, ix, iz, term index)
                        const int fi = tm.x - K::NV;
                        if (fi >= 0 && tm.z == j && tm.y >= x && tm.y < x + 4) {
                            C *cell = tr + fi * K::SW + (tm.y - x);
                            *cell = through<S, C>(*cell + sh.tamp[(long long)tm.w * sh.tamp_nt + it]);
                            hit = true;
                        }
                    }
                    if (hit) {
#pragma unroll
                        for (int f = 0; f < K::NT; ++f) Vec4<C, C>::ld(tr + f * K::SW, tnew[f]);
                    }
                }
                // ---- hybrid box, after the point source: an add-ring cell takes
                // the value its old-stress slot holds, r + s, written there by
                // the residual stress update before this launch (every column:
                // halo columns feed the velocity stencil too).  Shared-memory
                // copies only: the old stresses are still in the point-wise stage.
                if constexpr (PSV && std::is_same<S, C>::value && !BATCH) {  // batches have no box
                    const int aj = j - sh.box.z0 - 4, ai0 = x - sh.box.x0 - 4;
                    const int aw = sh.box.bx - 8, ah = sh.box.bz - 8;
                    if (sh.box.on && aj >= 0 && aj < ah && ai0 + 3 >= 0 && ai0 < aw &&
                        (aj < 4 || aj >= ah - 4 || ai0 < 4 || ai0 + 3 >= aw - 4)) {
                        bool changed = false;
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int ai = ai0 + e;
                            if (ai >= 0 && ai < aw && (aj < 4 || aj >= ah - 4 || ai < 4 || ai >= aw - 4)) {
#pragma unroll
                                for (int f = 0; f < K::NT; ++f) tr[f * K::SW + e] = to_c<C>(pwrow(f)[e]);
                                changed = true;
                            }
                        }
                        if (changed) {
#pragma unroll
                            for (int f = 0; f < K::NT; ++f) Vec4<C, C>::ld(tr + f * K::SW, tnew[f]);
                        }
                    }
                }
                // ---- HBM (owned cells) ----
                if (inrow && own_x && j >= I.z0 && j < I.z1 && x < nx) {
                    const long long o = origin + (long long)j * pitch + x;
                    if (x + 3 < nx) {
#pragma unroll
                        for (int f = 0; f < K::NT; ++f) Vec4<S, C>::st(wr[K::NV + f] + o, tnew[f]);
                    } else {
#pragma unroll
                        for (int f = 0; f < K::NT; ++f)
#pragma unroll
                            for (int e = 0; e < 4; ++e)
                                if (x + e < nx) wr[K::NV + f][o + e] = to_s<S>(tnew[f][e]);
                    }
                }
            }
            // stresses of this block visible to every compute warp; all agree to go on
            ok = compute_bar_and(NCT, ok) != 0;
            if (!ok) break;

            if constexpr (!PSV) {
                // free-surface stress image Tz(x,0) = -Tz(x,1), SH/fd/cu_fd.cu:226,
                // once rows 0 and 1 of the new stresses exist
                if (I.z0 == 0 && i == 1) {
                    bool img = grp == 0;
                    if constexpr (PUNCH) img = img && punch_active(sh.punch, min(max(x, 0), nx - 1), 0, it);
                    if (img) {
                        C *r0 = const_cast<C *>(trrow(0)) + K::SW;
                        const C *r1 = trrow(1) + K::SW;
                        C v1[4], v0[4];
                        Vec4<C, C>::ld(r1, v1);
#pragma unroll
                        for (int e = 0; e < 4; ++e) v0[e] = -v1[e];
                        Vec4<C, C>::st(r0, v0);
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            if (own_x && x + e < nx && nz > 1) wr[K::NV + 1][origin + x + e] = to_s<S>(v0[e]);
                    }
                    compute_bar(NCT);
                }
            }

            // ================= velocity: row a, cells x .. x+3 =================
            {
                const int a = I.z0 - 8 + 4 * i + grp;
                if (a >= I.z0 && a < nz && own_x && x < nx) {
                    const C *trow[9];
#pragma unroll
                    for (int d = 0; d < 9; ++d) trow[d] = trrow(a - 4 + d);
                    C mv[K::NMV][4];
                    if constexpr (TABLE) {
                        const uint32_t q = *reinterpret_cast<const uint32_t *>(
                            reinterpret_cast<const unsigned char *>(pws + K::PG_MS) + grp * kIdxBoxW + ixo);
#pragma unroll
                        for (int m = 0; m < K::NMV; ++m)
#pragma unroll
                            for (int e = 0; e < 4; ++e)
                                mv[m][e] = to_c<C>(tab_s[(K::NMS + m) * kTabEntries + ((q >> (8 * e)) & 255u)]);
                    } else {
#pragma unroll
                        for (int m = 0; m < K::NMV; ++m) Vec4<S, C>::ld(pwrow(K::NT + K::NMS + m), mv[m]);
                    }
                    const int rel = 4 * i + grp;  // a - (z0-8): block i, row grp
                    const int vr = (4 * (uw_base + i) + (rel & 3)) & (4 * K::NUW - 1);
                    const S *vrow = uw_s + (vr >> 2) * K::UW_SLOT + (vr & 3) * K::UWW + 4 * lane + 4;
                    C vold[K::NV][4];
#pragma unroll
                    for (int v = 0; v < K::NV; ++v) Vec4<S, C>::ld(vrow + v * K::UWF, vold[v]);
                    const bool zfast = a >= 4 && a <= nz - 5 && a < nz - npml && !(sh.topabsorb && a < npml);
                    bool vact = true;
                    if constexpr (PUNCH) vact = punch_active(sh.punch, x, a, it);
                    C vnew[K::NV][4];
                    // line force on V, injected before the velocity update (SH only);
                    // read-modify-write of this thread's own cell of stencil row a,
                    // which no stress update reads any more
                    if constexpr (!PSV) {
                        if (ntl > 0) {
                            bool hit = false;
                            for (int t = 0; t < ntl; ++t) {
                                const int4 tm = tl[t];
                                if (tm.x == FD23_V && tm.z == a && tm.y >= x && tm.y < x + 4) {
                                    S *cell = const_cast<S *>(vrow) + (tm.y - x);
                                    *cell = to_s<S>(to_c<C>(*cell) + sh.tamp[(long long)tm.w * sh.tamp_nt + it]);
                                    hit = true;
                                }
                            }
                            if (hit) Vec4<S, C>::ld(vrow, vold[0]);
                        }
                    }
                    if (xfast && zfast) {
                        velocity_interior(trow, mv, vold, vnew);
                    } else if (!PUNCH && xfast && a >= 4 && a <= nz - 5) {
                        // x-interior cells of a z-CPML row, as in the stress update
                        if constexpr (!PSV) {
                            constexpr C c0 = Coef4<C>::c0, c1 = Coef4<C>::c1, c2 = Coef4<C>::c2, c3 = Coef4<C>::c3;
                            const bool top = a < npml && sh.topabsorb;
                            const long long pz0 = top ? (long long)a * nx + x : (long long)(npml + nz - 1 - a) * nx + x;
                            C pst[4];
#pragma unroll
                            for (int e = 0; e < 4; ++e) pst[e] = prd[2][pz0 + e];
                            C h[12], dxT[4], dzT[4];
                            ld12<C, C>(trow[4], h);  // Tx
#pragma unroll
                            for (int e = 0; e < 4; ++e) dxT[e] = dmx<C>(h, e, c0, c1, c2, c3);
                            dpz4p<C, C>(trow, K::SW).to(dzT);  // d/dz Tz
                            const int zb = 2 * nx;
                            const C bT = __ldg(cp + (zb + a)), cT = __ldg(cp + (B + zb + a)),
                                    kT = __ldg(cp + (2 * B + zb + a));
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                const C bv = mv[0][e];
                                const C pa = fmaC<C>(bT, pst[e], cT * dzT[e]);
                                const C v = fmaC<C>(bv, dxT[e], vold[0][e]);
                                vnew[0][e] = fmaC<C>(bv, fmaC<C>(dzT[e], kT, pa), v);
                                pwr[2][pz0 + e] = pa;
                            }
                        }
                        if constexpr (PSV) {
                            constexpr C c0 = Coef4<C>::c0, c1 = Coef4<C>::c1, c2 = Coef4<C>::c2, c3 = Coef4<C>::c3;
                            const bool top = a < npml && sh.topabsorb;
                            const long long pz0 = top ? (long long)a * nx + x : (long long)(npml + nz - 1 - a) * nx + x;
                            C psa[4], psb[4];
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                psa[e] = prd[5][pz0 + e];
                                psb[e] = prd[4][pz0 + e];
                            }
                            C h[12], dxTxx[4], dxTxz[4], dzTxz[4], dzTzz[4];
                            ld12<C, C>(trow[4], h);  // Txx
#pragma unroll
                            for (int e = 0; e < 4; ++e) dxTxx[e] = dpx<C>(h, e, c0, c1, c2, c3);
                            ld12<C, C>(trow[4] + K::SW, h);  // Txz
#pragma unroll
                            for (int e = 0; e < 4; ++e) dxTxz[e] = dmx<C>(h, e, c0, c1, c2, c3);
                            dpz4p<C, C>(trow, K::SW).to(dzTxz);
                            dmz4p<C, C>(trow, 2 * K::SW).to(dzTzz);
                            const int zb = 4 * nx;
                            const C bA = __ldg(cp + (zb + nz + a)), cA = __ldg(cp + (B + zb + nz + a)),
                                    kA = __ldg(cp + (2 * B + zb + nz + a));
                            const C bB = __ldg(cp + (zb + a)), cB = __ldg(cp + (B + zb + a)),
                                    kB = __ldg(cp + (2 * B + zb + a));
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                C pa = psa[e], pb = psb[e];
                                vnew[0][e] = vold[0][e];
                                vnew[1][e] = vold[1][e];
                                if (vact) {
                                    const C bu = mv[0][e], bw = mv[1][e];
                                    C u = vold[0][e], w = vold[1][e];
                                    u = fmaC<C>(bu, dxTxx[e], u);
                                    w = fmaC<C>(bw, dxTxz[e], w);
                                    pa = fmaC<C>(bA, psa[e], cA * dzTxz[e]);
                                    pb = fmaC<C>(bB, psb[e], cB * dzTzz[e]);
                                    u = fmaC<C>(bu, fmaC<C>(dzTxz[e], kA, pa), u);
                                    w = fmaC<C>(bw, fmaC<C>(dzTzz[e], kB, pb), w);
                                    vnew[0][e] = u;
                                    vnew[1][e] = w;
                                }
                                pwr[5][pz0 + e] = pa;
                                pwr[4][pz0 + e] = pb;
                            }
                        }
                    } else {
                        C psx[2][4], psz[2][4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int ix = x + e;
                            psx[0][e] = psx[1][e] = psz[0][e] = psz[1][e] = (C)0;
                            if (ix >= nx) continue;
                            const bool top = a < npml && sh.topabsorb;
                            if (ix < npml || ix >= nx - npml) {
                                const long long px = ix < npml ? (long long)ix + (long long)a * 2 * npml
                                                               : (long long)npml + nx - 1 - ix + (long long)a * 2 * npml;
                                psx[0][e] = prd[0][px];
                                if constexpr (PSV) psx[1][e] = prd[1][px];
                            }
                            if (top || a >= nz - npml) {
                                const long long pz = top ? (long long)a * nx + ix : (long long)(npml + nz - 1 - a) * nx + ix;
                                if constexpr (PSV) { psz[0][e] = prd[5][pz]; psz[1][e] = prd[4][pz]; }
                                else psz[0][e] = prd[2][pz];
                            }
                        }
                        C cc[4][4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) cell_coef<C>(x + e, a, nx, nz, cc[e][0], cc[e][1], cc[e][2], cc[e][3]);
                        // P-SV: dA = d/dx Txx, dB = d/dx Txz, dC = d/dz Txz, dD = d/dz Tzz
                        // SH:   dA = d/dx Tx,  dC = d/dz Tz
                        C dA[4], dB[4], dC[4], dD[4];
                        {
                            C h[12];
                            ld12<C, C>(trow[4], h);
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                
                                dA[e] = PSV ? dpx<C>(h, e, cc[e][0], cc[e][1], cc[e][2], cc[e][3]) : dmx<C>(h, e, cc[e][0], cc[e][1], cc[e][2], cc[e][3]);
                            }
                        }
                        {
                            C h[12], zv[9][4];
                            if constexpr (PSV) ld12<C, C>(trow[4] + K::SW, h);
                            zcol<C, C>(trow, K::SW, zv);
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                
                                if constexpr (PSV) dB[e] = dmx<C>(h, e, cc[e][0], cc[e][1], cc[e][2], cc[e][3]);
                                dC[e] = comb<C>(cc[e][0], cc[e][1], cc[e][2], cc[e][3], zv[5][e] - zv[4][e], zv[6][e] - zv[3][e],
                                                zv[7][e] - zv[2][e], zv[8][e] - zv[1][e]);
                            }
                        }
                        if constexpr (PSV) {
                            C zv[9][4];
                            zcol<C, C>(trow, 2 * K::SW, zv);
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                
                                dD[e] = comb<C>(cc[e][0], cc[e][1], cc[e][2], cc[e][3], zv[4][e] - zv[3][e], zv[5][e] - zv[2][e],
                                                zv[6][e] - zv[1][e], zv[7][e] - zv[0][e]);
                            }
                        }
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int ix = x + e;
#pragma unroll
                            for (int v = 0; v < K::NV; ++v) vnew[v][e] = vold[v][e];
                            if (ix >= nx) continue;
                            const bool xp = ix < npml || ix >= nx - npml;
                            const bool top = a < npml && sh.topabsorb;
                            const bool zp = top || a >= nz - npml;
                            const long long px = ix < npml ? (long long)ix + (long long)a * 2 * npml
                                                           : (long long)npml + nx - 1 - ix + (long long)a * 2 * npml;
                            const long long pz = top ? (long long)a * nx + ix : (long long)(npml + nz - 1 - a) * nx + ix;
                            if constexpr (PUNCH) {
                                if (!vact) {
                                    if (xp) {
                                        pwr[0][px] = psx[0][e];
                                        if constexpr (PSV) pwr[1][px] = psx[1][e];
                                    }
                                    if (zp) {
                                        if constexpr (PSV) { pwr[5][pz] = psz[0][e]; pwr[4][pz] = psz[1][e]; }
                                        else pwr[2][pz] = psz[0][e];
                                    }
                                    continue;
                                }
                            }
                            if constexpr (PSV) {
                                const C dxTxx = dA[e], dxTxz = dB[e], dzTxz = dC[e], dzTzz = dD[e];
                                const C bu = mv[0][e], bw = mv[1][e];
                                C u = vold[0][e], w = vold[1][e];
                                // x chain, PD/fd/cu_fd.cu:455-474
                                if (xp) {
                                    const C pa = fmaC<C>(cxc(0, 0, ix), psx[0][e], cxc(1, 0, ix) * dxTxx);
                                    pwr[0][px] = pa;
                                    u = fmaC<C>(bu, fmaC<C>(dxTxx, cxc(2, 0, ix), pa), u);
                                    const C pb = fmaC<C>(cxc(0, 1, ix), psx[1][e], cxc(1, 1, ix) * dxTxz);
                                    pwr[1][px] = pb;
                                    w = fmaC<C>(bw, fmaC<C>(dxTxz, cxc(2, 1, ix), pb), w);
                                } else if (a != 0) {
                                    u = fmaC<C>(bu, dxTxx, u);
                                    w = fmaC<C>(bw, dxTxz, w);
                                }
                                // z chain, :476-499
                                if (zp) {
                                    const int zb = 4 * nx;
                                    const C pa = fmaC<C>(__ldg(cp + (zb + nz + a)), psz[0][e], __ldg(cp + (B + zb + nz + a)) * dzTxz);
                                    const C pb = fmaC<C>(__ldg(cp + (zb + a)), psz[1][e], __ldg(cp + (B + zb + a)) * dzTzz);
                                    pwr[5][pz] = pa;
                                    pwr[4][pz] = pb;
                                    u = fmaC<C>(bu, fmaC<C>(dzTxz, __ldg(cp + (2 * B + zb + nz + a)), pa), u);
                                    w = fmaC<C>(bw, fmaC<C>(dzTzz, __ldg(cp + (2 * B + zb + a)), pb), w);
                                } else if (a == 0) {
                                    u = fmaC<C>(bu, dxTxx + dzTxz, u);
                                    w = (C)0;
                                } else {
                                    u = fmaC<C>(bu, dzTxz, u);
                                    w = fmaC<C>(bw, dzTzz, w);
                                }
                                vnew[0][e] = u;
                                vnew[1][e] = w;
                            } else {
                                const C dxT = dA[e], dzT = dC[e];
                                const C bv = mv[0][e];
                                C v = vold[0][e];
                                if (xp) {
                                    const C pa = fmaC<C>(cxc(0, 0, ix), psx[0][e], cxc(1, 0, ix) * dxT);
                                    pwr[0][px] = pa;
                                    v = fmaC<C>(bv, fmaC<C>(dxT, cxc(2, 0, ix), pa), v);
                                } else {
                                    v = fmaC<C>(bv, dxT, v);
                                }
                                if (zp) {
                                    const int zb = 2 * nx;
                                    const C pa = fmaC<C>(__ldg(cp + (zb + a)), psz[0][e], __ldg(cp + (B + zb + a)) * dzT);
                                    pwr[2][pz] = pa;
                                    v = fmaC<C>(bv, fmaC<C>(dzT, __ldg(cp + (2 * B + zb + a)), pa), v);
                                } else {
                                    v = fmaC<C>(bv, dzT, v);
                                }
                                vnew[0][e] = v;
                            }
                        }
                    }
                    if constexpr (PUNCH) {
                        if (!vact)
#pragma unroll
                            for (int v = 0; v < K::NV; ++v)
#pragma unroll
                                for (int e = 0; e < 4; ++e) vnew[v][e] = vold[v][e];
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
            }  // per-lane iteration
            // release the ring slots this iteration was the last reader of
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&empty_uw[(uw_base + i) % K::NUW]);
                if (i == I.niter - 1) {
                    mbar_arrive(&empty_uw[(uw_base + i + 1) % K::NUW]);
                    mbar_arrive(&empty_uw[(uw_base + i + 2) % K::NUW]);
                }
                mbar_arrive(&empty_pw[gflat % K::NPW]);
            }
        }
        uw_base += I.niter + 2;
    }
}

template <class S, class C, int WAVE, bool BATCH, bool PUNCH, bool TABLE = false, bool FASTF = false>
int launch_fused_impl(const Shot<S, C> &s, const Shot<S, C> *shots, const WorkItem *items, const int *item_off,
                      int nblocks, int par, int it, int rec_index, int *err_flag, cudaStream_t st)
{
    using K = Cfg<S, C, WAVE, TABLE>;
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
    const cudaError_t e = cudaLaunchKernelEx(&cfg, fused_step<S, C, WAVE, BATCH, PUNCH, TABLE, FASTF>, s, shots, items,
                                             item_off, par, it, rec_index, err_flag);
    return e == cudaSuccess ? FD23_OK : FD23_ERR_CUDA;
}

// the FP32 instantiation with the fast iterations (single shot, plain)
template <int WAVE>
int prepare_fast()
{
    return cudaFuncSetAttribute(fused_step<float, float, WAVE, false, false, false, true>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)Cfg<float, float, WAVE>::SMEM) == cudaSuccess
               ? FD23_OK
               : FD23_ERR_CUDA;
}

template <class S, class C, int WAVE, bool PUNCH, bool TABLE = false>
int prepare_one()
{
    using K = Cfg<S, C, WAVE, TABLE>;
    const bool ok = cudaFuncSetAttribute(fused_step<S, C, WAVE, false, PUNCH, TABLE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)K::SMEM) == cudaSuccess &&
                    cudaFuncSetAttribute(fused_step<S, C, WAVE, true, PUNCH, TABLE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)K::SMEM) == cudaSuccess;
    return ok ? FD23_OK : FD23_ERR_CUDA;
}

}  // namespace

}  // namespace fd23
