// C ABI of the fd23 engine (include/fd23.h): solver lifecycle, uploads into
// the padded HBM layout, the time loop and state transfer.  No call exits
// the process; every failure returns a status.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cudaTypedefs.h>

#include "fd23_solver.h"

using namespace fd23;

namespace fd23 {
Layout make_layout(int nx, int nz, int cover_x, int cover_z)
{
    Layout L;
    L.nx = nx;
    L.nz = nz;
    const int cols = kXPad + std::max(cover_x, nx) + 8;
    L.pitch = (cols + 31) / 32 * 32;
    L.rows = kZPad + std::max(cover_z, nz) + 8;
    L.origin = (long long)kZPad * L.pitch + kXPad;
    return L;
}
}  // namespace fd23

namespace {

// float -> bfloat16, round to nearest even (NaN kept quiet)
uint16_t f32_to_bf16(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
float bf16_to_f32(uint16_t h)
{
    uint32_t u = (uint32_t)h << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
uint16_t f32_to_f16(float f)
{
    _Float16 h = (_Float16)f;
    uint16_t u;
    std::memcpy(&u, &h, 2);
    return u;
}
float f16_to_f32(uint16_t u)
{
    _Float16 h;
    std::memcpy(&h, &u, 2);
    return (float)h;
}

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

}  // namespace

namespace fd23 {

int dev_alloc(void **p, size_t bytes)
{
    if (cudaMalloc(p, bytes) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return FD23_ERR_NOMEM;
    }
    return FD23_OK;
}

size_t storage_size(int prec) { return prec == FD23_F64 ? 8 : (prec == FD23_F32 ? 4 : 2); }
size_t compute_size(int prec) { return prec == FD23_F64 ? 8 : 4; }

// convert a double array to the storage type into dst (bytes = n*es)
void to_storage(int prec, const double *src, size_t n, unsigned char *dst)
{
    switch (prec) {
        case FD23_F64: std::memcpy(dst, src, n * 8); break;
        case FD23_F32:
            for (size_t i = 0; i < n; ++i) reinterpret_cast<float *>(dst)[i] = (float)src[i];
            break;
        case FD23_BF16:
            for (size_t i = 0; i < n; ++i) reinterpret_cast<uint16_t *>(dst)[i] = f32_to_bf16((float)src[i]);
            break;
        default:
            for (size_t i = 0; i < n; ++i) reinterpret_cast<uint16_t *>(dst)[i] = f32_to_f16((float)src[i]);
    }
}
void to_compute(int prec, const double *src, size_t n, unsigned char *dst)
{
    if (prec == FD23_F64) std::memcpy(dst, src, n * 8);
    else
        for (size_t i = 0; i < n; ++i) reinterpret_cast<float *>(dst)[i] = (float)src[i];
}
// storage element -> compute element
void storage_to_compute(int prec, const unsigned char *src, size_t n, unsigned char *dst)
{
    switch (prec) {
        case FD23_F64: std::memcpy(dst, src, n * 8); break;
        case FD23_F32: std::memcpy(dst, src, n * 4); break;
        case FD23_BF16:
            for (size_t i = 0; i < n; ++i)
                reinterpret_cast<float *>(dst)[i] = bf16_to_f32(reinterpret_cast<const uint16_t *>(src)[i]);
            break;
        default:
            for (size_t i = 0; i < n; ++i)
                reinterpret_cast<float *>(dst)[i] = f16_to_f32(reinterpret_cast<const uint16_t *>(src)[i]);
    }
}
void compute_to_storage(int prec, const unsigned char *src, size_t n, unsigned char *dst)
{
    switch (prec) {
        case FD23_F64: std::memcpy(dst, src, n * 8); break;
        case FD23_F32: std::memcpy(dst, src, n * 4); break;
        case FD23_BF16:
            for (size_t i = 0; i < n; ++i)
                reinterpret_cast<uint16_t *>(dst)[i] = f32_to_bf16(reinterpret_cast<const float *>(src)[i]);
            break;
        default:
            for (size_t i = 0; i < n; ++i)
                reinterpret_cast<uint16_t *>(dst)[i] = f32_to_f16(reinterpret_cast<const float *>(src)[i]);
    }
}

// upload an nx*nz array (already in element format, es bytes each) into the padded layout
int upload_grid(fd23_solver *s, void *dptr, const unsigned char *host, size_t es)
{
    const Layout &L = s->L;
    CK(cudaMemcpy2DAsync((unsigned char *)dptr + (size_t)L.origin * es, (size_t)L.pitch * es, host,
                         (size_t)L.nx * es, (size_t)L.nx * es, (size_t)L.nz, cudaMemcpyHostToDevice,
                         s->stream));
    return FD23_OK;
}
int download_grid(fd23_solver *s, const void *dptr, unsigned char *host, size_t es)
{
    const Layout &L = s->L;
    CK(cudaMemcpy2DAsync(host, (size_t)L.nx * es, (const unsigned char *)dptr + (size_t)L.origin * es,
                         (size_t)L.pitch * es, (size_t)L.nx * es, (size_t)L.nz, cudaMemcpyDeviceToHost,
                         s->stream));
    return FD23_OK;
}

// Two time steps (it, it+1) in one launch of the two-step sweep.  The
// pending record row (the previous launch's last step) is gathered on the
// way, step it is recorded inside the launch, step it+1 becomes pending.
int step2_impl(fd23_solver *s, int rec_now, int rec_next)
{
    Shot<float, float> sh = make_shot<float, float>(s);
    sh.cta0 = 0;
    sh.ncta = s->nblocks2;
    const int rec_mid = rec_now ? s->nrec_steps++ : -1;
    const int rc = launch_step_fused2<float>(sh, s->f2_width, s->d_items2, s->d_item_off2, s->nblocks2, s->par,
                                             s->it, s->pending_rec, rec_mid, s->err_flag, s->stream);
    if (rc) return rc;
    s->pending_rec = -1;
    s->par = 1 - s->par;
    s->it += 2;
    if (rec_next) s->pending_rec = s->nrec_steps++;
    return FD23_OK;
}

// One time step.  Without a box the fused sweep gathers the previous step's
// receivers on its way; with a box the step is
//   ring(U,W) | residual stress (+ add-ring g) | sweep | sub-ring r |
//   receivers + residual velocity
// (PD/main.cpp:153-199 order; the exchanges that read only fields the next
// update leaves unchanged run earlier, with the same values).
template <class S, class C>
int step_impl(fd23_solver *s, int rec_now, int more)
{
    Shot<S, C> sh = make_shot<S, C>(s);
    const bool box = s->box_on;
    int rc = FD23_OK;
    // incident field of this step and the next (a merged box launch reads both)
    if (box && (rc = wait_incident(s, s->it + 1))) return rc;
    if (box && !s->box_pre_ahead && (rc = launch_box_pre<S, C>(sh, s->fused ? s->par : 0, s->fused, s->stream)))
        return rc;
    s->box_pre_ahead = false;
    if (s->fused) {
        const WorkItem *items = s->d_items;
        const int *off = s->d_item_off;
        int nblocks = s->nblocks;
        int slot = -1;
        if (s->d_punch && s->punch_phase > 0) {
            if ((rc = phase_plan(s, &slot))) return rc;
            items = s->phase[slot].items;
            off = s->phase[slot].off;
            nblocks = s->phase[slot].nblocks;
            sh.ncta = nblocks;
        }
        rc = launch_step_fused<S, C>(sh, s->d.wave, items, off, nblocks, s->par, s->it, s->pending_rec,
                                     s->err_flag, s->stream, s->tune.fast);
        if (rc) return rc;
        if (slot >= 0) CK(cudaEventRecord(s->phase[slot].done, s->stream));
        s->pending_rec = -1;
        s->par = 1 - s->par;
        if (rec_now && !box) s->pending_rec = s->nrec_steps++;
    } else {
        rc = launch_step_twopass<S, C>(sh, s->d.wave, s->it, s->stream);
        if (rc) return rc;
        if (rec_now && !box && (rc = launch_record<S, C>(sh, 0, s->nrec_steps++, s->stream))) return rc;
    }
    if (box) {
        const int ri = rec_now ? s->nrec_steps++ : -1;
        // the fused sweep with another step to come: this step's end and the
        // next step's start as one launch where the box allows it
        rc = FD23_ERR_UNSUPPORTED;
        if (s->fused && more) rc = launch_box_mid<S, C>(sh, s->par, ri, s->stream);
        if (rc == FD23_OK) s->box_pre_ahead = true;
        else if (rc != FD23_ERR_UNSUPPORTED) return rc;
        else if ((rc = launch_box_post<S, C>(sh, s->fused ? s->par : 0, s->fused, ri, s->stream))) return rc;
    }
    s->it++;
    return FD23_OK;
}

template <class S, class C>
int flush_records(fd23_solver *s)
{
    if (s->pending_rec < 0) return FD23_OK;
    Shot<S, C> sh = make_shot<S, C>(s);
    const int rc = launch_record<S, C>(sh, s->par, s->pending_rec, s->stream);
    s->pending_rec = -1;
    return rc;
}

int dispatch_step(fd23_solver *s, int rec_now, int more)
{
    switch (s->d.prec) {
        case FD23_F64: return step_impl<double, double>(s, rec_now, more);
        case FD23_BF16: return step_impl<__nv_bfloat16, float>(s, rec_now, more);
        case FD23_F16: return step_impl<__half, float>(s, rec_now, more);
        default: return step_impl<float, float>(s, rec_now, more);
    }
}
int dispatch_persist(fd23_solver *s, int nsteps, int itrecord, int any_rec)
{
    switch (s->d.prec) {
        case FD23_F64:
            return launch_persist<double, double>(make_shot<double, double>(s), s->d.wave, s->it, nsteps, itrecord,
                                                  s->nrec_steps, any_rec, s->d_bar, s->err_flag, s->stream);
        case FD23_BF16:
            return launch_persist<__nv_bfloat16, float>(make_shot<__nv_bfloat16, float>(s), s->d.wave, s->it, nsteps,
                                                        itrecord, s->nrec_steps, any_rec, s->d_bar, s->err_flag,
                                                        s->stream);
        case FD23_F16:
            return launch_persist<__half, float>(make_shot<__half, float>(s), s->d.wave, s->it, nsteps, itrecord,
                                                 s->nrec_steps, any_rec, s->d_bar, s->err_flag, s->stream);
        default:
            return launch_persist<float, float>(make_shot<float, float>(s), s->d.wave, s->it, nsteps, itrecord,
                                                s->nrec_steps, any_rec, s->d_bar, s->err_flag, s->stream);
    }
}
int dispatch_flush(fd23_solver *s)
{
    switch (s->d.prec) {
        case FD23_F64: return flush_records<double, double>(s);
        case FD23_BF16: return flush_records<__nv_bfloat16, float>(s);
        case FD23_F16: return flush_records<__half, float>(s);
        default: return flush_records<float, float>(s);
    }
}

// Tensor maps of the fused sweep's copies: 3-D views [field][row][column] of
// the wavefield block of each buffer set and of the material block, with the
// box shapes the sweep copies (fused_boxes).  Coordinates of a copy are
// padded-array positions, so every box the sweep asks for lies inside.
// the driver's cuTensorMapEncodeTiled (null when unavailable)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q;
        void *fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn) {
            cudaGetLastError();
            return nullptr;
        }
        encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }
    return encode;
}

// Tensor maps of the two-step sweep (FP32 wavefields and material): the same
// views as encode_maps with its boxes (fused2_boxes).
int encode_maps2(fd23_solver *s)
{
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return FD23_ERR_CUDA;
    const Fused2Boxes bx = fused2_boxes(false, s->f2_width);
    const Layout &L = s->L;
    auto make = [&](TmaDesc &m, void *base, int nfields, int w, int nf, size_t es,
                    CUtensorMapDataType dt) -> int {
        const cuuint64_t dims[3] = {(cuuint64_t)L.pitch, (cuuint64_t)L.rows, (cuuint64_t)nfields};
        const cuuint64_t strides[2] = {(cuuint64_t)L.pitch * es, (cuuint64_t)L.elems() * es};
        const cuuint32_t box[3] = {(cuuint32_t)w, 4u, (cuuint32_t)nf};
        const cuuint32_t estr[3] = {1u, 1u, 1u};
        const CUresult r = encode(reinterpret_cast<CUtensorMap *>(&m), dt, 3, base, dims, strides, box, estr,
                                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                  CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        return r == CUDA_SUCCESS ? FD23_OK : FD23_ERR_CUDA;
    };
    // U, W rows of bx.uww columns (more than a box dimension's 256 for the
    // wide strips): a 4-D view [field][row][column / 8][8] whose box
    // {8, uww / 8, 4, 1} lands as [4][uww] in shared memory
    auto make_groups = [&](TmaDesc &m, void *base, int nfields, int w, int nf) -> int {
        const cuuint64_t dims[4] = {8u, (cuuint64_t)L.pitch / 8, (cuuint64_t)L.rows, (cuuint64_t)nfields};
        const cuuint64_t strides[3] = {32u, (cuuint64_t)L.pitch * 4, (cuuint64_t)L.elems() * 4};
        const cuuint32_t box[4] = {8u, (cuuint32_t)(w / 8), 4u, (cuuint32_t)nf};
        const cuuint32_t estr[4] = {1u, 1u, 1u, 1u};
        const CUresult r = encode(reinterpret_cast<CUtensorMap *>(&m), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims,
                                  strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                  CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        return r == CUDA_SUCCESS ? FD23_OK : FD23_ERR_CUDA;
    };
    if (L.pitch % 8 != 0 || bx.uww % 8 != 0) return FD23_ERR_UNSUPPORTED;
    ShotMaps2 h{};
    int rc = FD23_OK;
    for (int b = 0; b < 2 && !rc; ++b) {
        rc = make_groups(h.uw[b], s->fld_block[b], s->nfld, bx.uww, 1);
        if (!rc) rc = make(h.t[b], s->fld_block[b], s->nfld, bx.pww, 3, 4, CU_TENSOR_MAP_DATA_TYPE_FLOAT32);
    }
    if (!rc) rc = make(h.ms, s->mat_block, s->nmat, bx.mww, 3, 4, CU_TENSOR_MAP_DATA_TYPE_FLOAT32);
    if (!rc) rc = make(h.mv, s->mat_block, s->nmat, bx.mww, 2, 4, CU_TENSOR_MAP_DATA_TYPE_FLOAT32);
    if (rc) return rc;
    if (!s->d_maps2 && (rc = dev_alloc((void **)&s->d_maps2, sizeof(ShotMaps2)))) return rc;
    CK(cudaMemcpy(s->d_maps2, &h, sizeof(ShotMaps2), cudaMemcpyHostToDevice));
    return FD23_OK;
}

int encode_maps(fd23_solver *s)
{
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return FD23_ERR_CUDA;
    const FusedBoxes bx = fused_boxes(s->d.wave, s->d.prec);
    CUtensorMapDataType dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    if (s->d.prec == FD23_F64) dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    if (s->d.prec == FD23_BF16) dt = CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    if (s->d.prec == FD23_F16) dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    const Layout &L = s->L;
    auto make = [&](TmaDesc &m, void *base, int nfields, int w, int nf) -> int {
        const cuuint64_t dims[3] = {(cuuint64_t)L.pitch, (cuuint64_t)L.rows, (cuuint64_t)nfields};
        const cuuint64_t strides[2] = {(cuuint64_t)L.pitch * s->es, (cuuint64_t)L.elems() * s->es};
        const cuuint32_t box[3] = {(cuuint32_t)w, 4u, (cuuint32_t)nf};
        const cuuint32_t estr[3] = {1u, 1u, 1u};
        const CUresult r = encode(reinterpret_cast<CUtensorMap *>(&m), dt, 3, base, dims, strides, box, estr,
                                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                  CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        return r == CUDA_SUCCESS ? FD23_OK : FD23_ERR_CUDA;
    };
    ShotMaps h{};
    int rc = FD23_OK;
    for (int b = 0; b < 2 && !rc; ++b) {
        rc = make(h.uw[b], s->fld_block[b], s->nfld, bx.uww, bx.nv);
        if (!rc) rc = make(h.t[b], s->fld_block[b], s->nfld, bx.pww, bx.nt);
    }
    if (!rc) rc = make(h.ms, s->mat_block, s->nmat, bx.pww, bx.nms);
    if (!rc) rc = make(h.mv, s->mat_block, s->nmat, bx.pww, bx.nmv);
    if (!rc && s->d_midx) {
        // material-table indices: bytes, [row][column] of the padded layout
        const cuuint64_t dims[2] = {(cuuint64_t)L.pitch, (cuuint64_t)L.rows};
        const cuuint64_t strides[1] = {(cuuint64_t)L.pitch};
        const cuuint32_t box[2] = {(cuuint32_t)kIdxBoxW, 8u};
        const cuuint32_t estr[2] = {1u, 1u};
        const CUresult r = encode(reinterpret_cast<CUtensorMap *>(&h.idx), CU_TENSOR_MAP_DATA_TYPE_UINT8, 2,
                                  s->d_midx, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        rc = r == CUDA_SUCCESS ? FD23_OK : FD23_ERR_CUDA;
    }
    if (rc) return rc;
    if (!s->d_maps && (rc = dev_alloc((void **)&s->d_maps, sizeof(ShotMaps)))) return rc;
    CK(cudaMemcpy(s->d_maps, &h, sizeof(ShotMaps), cudaMemcpyHostToDevice));
    return FD23_OK;
}

// CTAs per SM the fused sweep can keep resident (shared memory bound, at most
// the 3 its register budget is built for)
int fused_per_sm(int device, int wave, int prec, bool batch)
{
    // registers and shared memory both bound the residency: ask the runtime
    // (after fused_prepare has raised the dynamic shared-memory limit)
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != device) {
        cudaGetLastError();
        if (cudaSetDevice(device) != cudaSuccess) {
            cudaGetLastError();
            return 1;
        }
    }
    return std::max(1, std::min(3, fused_occupancy(wave, prec, batch)));
}

int upload_plan(const WorkPlan &plan, WorkItem **d_items, int **d_off)
{
    cudaFree(*d_items);
    cudaFree(*d_off);
    *d_items = nullptr;
    *d_off = nullptr;
    int rc = dev_alloc((void **)d_items, plan.items.size() * sizeof(WorkItem));
    if (rc) return rc;
    if ((rc = dev_alloc((void **)d_off, plan.off.size() * sizeof(int)))) return rc;
    CK(cudaMemcpy(*d_items, plan.items.data(), plan.items.size() * sizeof(WorkItem), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(*d_off, plan.off.data(), plan.off.size() * sizeof(int), cudaMemcpyHostToDevice));
    return FD23_OK;
}

// Work list of one solver (fd23_plan.cpp); the relative block costs
// (FD23_COST_XPML, FD23_COST_ZPML, default 4 / 3) were measured on GB300.
int build_worklist(fd23_solver *s)
{
    const FusedGeom g = fused_geom(s->d.wave, s->d.prec);
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->d.device));
    TuneParams tp = s->tune;
    tp.per_sm = std::min(tp.per_sm, fused_per_sm(s->d.device, s->d.wave, s->d.prec));
    WorkPlan plan;
    const std::vector<ShotGeom> geo{ShotGeom{s->d.nx, s->d.nz, s->d.npml, s->d.topabsorb}};
    int rc = plan_work(geo, g.tile_x, sms, tp, plan);
    if (rc) return rc;
    if ((rc = upload_plan(plan, &s->d_items, &s->d_item_off))) return rc;
    s->nblocks = plan.nblocks;
    ++s->punch_ver;  // phase plans follow the tuning
    return FD23_OK;
}

// Work plan of the two-step sweep: strips of kFused2TileX output columns,
// one CTA per SM (its shared memory allows one).
int build_worklist2(fd23_solver *s)
{
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->d.device));
    TuneParams tp = s->tune;
    tp.per_sm = fused2_per_sm(s->f2_width);
    // strip-major: measured faster for this sweep (C1: 5.44e10 cell-updates/s
    // against 5.00e10 with the banded cut); strips from column 0
    tp.bands = 0;
    tp.shift = 0;
    WorkPlan plan;
    const std::vector<ShotGeom> geo{ShotGeom{s->d.nx, s->d.nz, s->d.npml, s->d.topabsorb}};
    int rc = plan_work(geo, fused2_tile_x(s->f2_width), sms, tp, plan);
    if (rc) return rc;
    cudaFree(s->d_items2);
    cudaFree(s->d_item_off2);
    s->d_items2 = nullptr;
    s->d_item_off2 = nullptr;
    if ((rc = upload_plan(plan, &s->d_items2, &s->d_item_off2))) return rc;
    s->nblocks2 = plan.nblocks;
    s->h_items2 = plan.items;
    s->h_item_off2 = plan.off;
    s->rec2_dirty = true;
    return FD23_OK;
}

// Receivers of every work item of the two-step plan (the cells it owns:
// columns [x0, x0+fused2_tile_x), rows [z0, z1)), velocity fields first, then
// stresses, each sorted by row: entries (field, ix, iz, receiver).
int build_rec2(fd23_solver *s)
{
    const int ni = (int)s->h_items2.size();
    const int tx = fused2_tile_x(s->f2_width);
    std::vector<int4> list;
    std::vector<int> off;
    off.reserve(2 * (size_t)ni + 1);
    for (int k = 0; k < ni; ++k) {
        const WorkItem &w = s->h_items2[k];
        for (int part = 0; part < 2; ++part) {
            off.push_back((int)list.size());
            const size_t first = list.size();
            for (int c = part == 0 ? 0 : 2; c < (part == 0 ? 2 : s->nfld); ++c)
                for (int r = 0; r < s->nrec[c] && r < (int)s->h_rx[c].size(); ++r) {
                    const int ix = s->h_rx[c][r], iz = s->h_rz[c][r];
                    if (ix >= w.x0 && ix < w.x0 + tx && iz >= w.z0 && iz < w.z1)
                        list.push_back(make_int4(c, ix, iz, r));
                }
            std::stable_sort(list.begin() + first, list.end(),
                             [](const int4 &a, const int4 &b) { return a.z < b.z; });
        }
    }
    off.push_back((int)list.size());
    cudaFree(s->d_rec2);
    cudaFree(s->d_rec2_off);
    s->d_rec2 = nullptr;
    s->d_rec2_off = nullptr;
    int rc = dev_alloc((void **)&s->d_rec2, std::max<size_t>(1, list.size()) * sizeof(int4));
    if (rc) return rc;
    if ((rc = dev_alloc((void **)&s->d_rec2_off, off.size() * sizeof(int)))) return rc;
    if (!list.empty()) CK(cudaMemcpy(s->d_rec2, list.data(), list.size() * sizeof(int4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->d_rec2_off, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice));
    s->rec2_dirty = false;
    return FD23_OK;
}

int upload_cpml(fd23_solver *s, const std::vector<double> &bck)
{
    std::vector<unsigned char> tmp(bck.size() * s->cs);
    to_compute(s->d.prec, bck.data(), bck.size(), tmp.data());
    CK(cudaMemcpyAsync(s->cpml, tmp.data(), tmp.size(), cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FD23_OK;
}

int zero_state(fd23_solver *s)
{
    const size_t gbytes = s->L.elems() * s->es;
    for (int b = 0; b < 2; ++b) {
        for (int f = 0; f < s->nfld; ++f) CK(cudaMemsetAsync(s->fld[b][f], 0, gbytes, s->stream));
        for (int p = 0; p < s->npsi; ++p)
            CK(cudaMemsetAsync(s->psi[b][p], 0, s->psi_elems[p] * s->cs, s->stream));
    }
    CK(cudaMemsetAsync(s->err_flag, 0, sizeof(int), s->stream));
    if (s->box_on)
        for (int f = 0; f < 5; ++f)
            CK(cudaMemsetAsync(s->box_r[f], 0, (size_t)s->box_bx * s->box_bz * s->cs, s->stream));
    s->it = 0;
    s->par = 0;
    s->nrec_steps = 0;
    s->pending_rec = -1;
    return FD23_OK;
}

void free_box(fd23_solver *s)
{
    for (int f = 0; f < 5; ++f) {
        cudaFree(s->box_r[f]);
        cudaFree(s->box_mat[f]);
        s->box_r[f] = s->box_mat[f] = nullptr;
    }
    cudaFree(s->box_cells);
    s->box_cells = nullptr;
    s->box_on = false;
    s->box_inc_n = 0;
}

void free_all(fd23_solver *s)
{
    for (int b = 0; b < 2; ++b) {
        cudaFree(s->fld_block[b]);
        for (int p = 0; p < 8; ++p) cudaFree(s->psi[b][p]);
    }
    cudaFree(s->mat_block);
    cudaFree(s->d_maps);
    cudaFree(s->d_punch);
    for (auto &ph : s->phase) {
        cudaFree(ph.items);
        cudaFree(ph.off);
        cudaFreeHost(ph.host);
        if (ph.done) cudaEventDestroy(ph.done);
    }
    cudaFree(s->d_midx);
    cudaFree(s->d_mtab);
    cudaFree(s->cpml);
    cudaFree(s->err_flag);
    cudaFree(s->d_bar);
    cudaFree(s->norm_buf);
    cudaFree(s->d_terms);
    cudaFree(s->d_tamp);
    for (int c = 0; c < 5; ++c) {
        cudaFree(s->d_rec[c]);
        cudaFree(s->d_seis[c]);
    }
    free_box(s);
    if (s->copy_stream) cudaStreamSynchronize(s->copy_stream);
    cudaFree(s->box_inc);
    for (cudaEvent_t e : s->inc_ev) cudaEventDestroy(e);
    if (s->inc_gate) cudaEventDestroy(s->inc_gate);
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    cudaFree(s->d_items);
    cudaFree(s->d_item_off);
    cudaFree(s->d_items2);
    cudaFree(s->d_item_off2);
    cudaFree(s->d_maps2);
    for (int p = 0; p < 8; ++p) cudaFree(s->psi_mid[p]);
    cudaFree(s->d_rec2);
    cudaFree(s->d_rec2_off);
    if (s->stream) cudaStreamDestroy(s->stream);
}

int ensure_record_capacity(fd23_solver *s, int need)
{
    if (need <= s->rec_cap) return FD23_OK;
    int cap = std::max(need, s->rec_cap * 2);
    for (int c = 0; c < 5; ++c) {
        if (s->nrec[c] <= 0) continue;
        void *np = nullptr;
        int rc = dev_alloc(&np, (size_t)cap * s->nrec[c] * s->cs);
        if (rc) return rc;
        if (s->d_seis[c] && s->nrec_steps > 0)
            CK(cudaMemcpyAsync(np, s->d_seis[c], (size_t)s->nrec_steps * s->nrec[c] * s->cs,
                               cudaMemcpyDeviceToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        cudaFree(s->d_seis[c]);
        s->d_seis[c] = np;
    }
    s->rec_cap = cap;
    return FD23_OK;
}

bool scaled_form(const fd23_solver *s) { return s->d.prec == FD23_BF16 || s->d.prec == FD23_F16; }

double pow2_round(double v)
{
    if (!(v > 0) || !std::isfinite(v)) return 1.0;
    return std::ldexp(1.0, (int)std::lround(std::log2(v)));
}
// scale of wavefield f (storage = scale * physical)
double field_scale(const fd23_solver *s, int f)
{
    const bool stress = f >= (s->d.wave == FD23_PSV ? FD23_TXX : FD23_TX);
    return stress ? s->sigma * s->kappa : s->sigma;
}
// memory variable p holds a derivative of a stress (scale sigma*kappa) or of a velocity (sigma)
double psi_scale(const fd23_solver *s, int p)
{
    bool of_stress;
    if (s->d.wave == FD23_PSV) of_stress = (p == 0 || p == 1 || p == 4 || p == 5);  // Txx_x Txz_x Tzz_z Txz_z
    else of_stress = (p == 0 || p == 2);                                            // Tx_x Tz_z
    return of_stress ? s->sigma * s->kappa : s->sigma;
}

// sigma: chosen once, when material (kappa) and source are known: the power
// of two that puts the accumulated source stress near 2^8 (room below the
// FP16 maximum, far above its subnormals)
int ensure_sigma(fd23_solver *s);

int upload_source_amps(fd23_solver *s)
{
    if (s->nterms == 0) return FD23_OK;
    const size_t nt = (size_t)s->tamp_nt;
    std::vector<double> a(s->h_tamp);
    for (int k = 0; k < s->nterms; ++k) {
        const double sc = field_scale(s, s->h_tfield[k]);
        for (size_t it = 0; it < nt; ++it) a[k * nt + it] *= sc;
    }
    std::vector<unsigned char> tmp(a.size() * s->cs);
    to_compute(s->d.prec, a.data(), a.size(), tmp.data());
    CK(cudaMemcpy(s->d_tamp, tmp.data(), tmp.size(), cudaMemcpyHostToDevice));
    return FD23_OK;
}

int ensure_sigma(fd23_solver *s)
{
    if (!scaled_form(s) || s->sigma_set || !s->kappa_set) return FD23_OK;
    double peak = 0.0;
    const int nt = s->tamp_nt;
    for (int k = 0; k < s->nterms; ++k) {
        const bool stress = s->h_tfield[k] >= (s->d.wave == FD23_PSV ? FD23_TXX : FD23_TX);
        double run = 0.0, amax = 0.0;
        for (int it = 0; it < nt; ++it) {
            const double a = std::fabs(s->h_tamp[(size_t)k * nt + it]);
            run += a;
            amax = std::max(amax, a);
        }
        peak = std::max(peak, std::max(run, amax) * (stress ? s->kappa : 1.0));
    }
    s->sigma = peak > 0 ? pow2_round(256.0 / peak) : 1.0;
    s->sigma_set = true;
    return upload_source_amps(s);
}

// after a new material: the table follows it; with too many distinct tuples
// it is dropped (as the reference's mktable gives up) and the sweep reads the
// material arrays
int material_done(fd23_solver *s)
{
    s->have_material = true;
    if (!s->table_on) return FD23_OK;
    const int rc = build_material_table(s);
    if (rc == FD23_ERR_UNSUPPORTED) {
        free_material_table(s);
        s->table_on = false;
        return s->fused ? encode_maps(s) : FD23_OK;
    }
    return rc;
}
// the solver's stream waits for the asynchronous incident chunks up to the one
// holding step `upto`
int wait_incident(fd23_solver *s, int upto)
{
    if (s->inc_chunk <= 0 || s->box_inc_n <= 0) return FD23_OK;
    upto = std::min(std::max(upto, s->box_inc_it0), s->box_inc_it0 + s->box_inc_n - 1);
    const int need = (upto - s->box_inc_it0) / s->inc_chunk;
    for (; s->inc_waited <= need; ++s->inc_waited)
        CK(cudaStreamWaitEvent(s->stream, s->inc_ev[s->inc_waited], 0));
    return FD23_OK;
}

}  // namespace fd23

extern "C" {

int fd23_version(void) { return 1; }

const char *fd23_strerror(int st)
{
    switch (st) {
        case FD23_OK: return "ok";
        case FD23_ERR_ARG: return "invalid argument";
        case FD23_ERR_CUDA: return "CUDA runtime error";
        case FD23_ERR_UNSTABLE: return "model fails the CFL stability check (stab > 1)";
        case FD23_ERR_ORDER: return "call made before what it depends on";
        case FD23_ERR_NOMEM: return "device allocation failed";
        case FD23_ERR_NONFINITE: return "wavefield holds NaN or Inf";
        case FD23_ERR_TIMEOUT: return "a bounded device-side wait gave up";
        case FD23_ERR_UNSUPPORTED: return "unsupported configuration";
        default: return "unknown status";
    }
}

int fd23_create(const fd23_desc *desc, fd23_solver **out)
{
    if (!desc || !out) return FD23_ERR_ARG;
    *out = nullptr;
    const fd23_desc &d = *desc;
    if (d.wave != FD23_PSV && d.wave != FD23_SH) return FD23_ERR_ARG;
    if (d.prec < FD23_F32 || d.prec > FD23_F16) return FD23_ERR_ARG;
    if (d.nx < 2 || d.nz < 2 || d.npml < 0 || 2 * d.npml > d.nx || 2 * d.npml > d.nz) return FD23_ERR_ARG;
    if ((long long)d.nx * d.nz > (1LL << 31)) return FD23_ERR_ARG;
    if (!(d.h > 0) || !(d.dt > 0)) return FD23_ERR_ARG;
    if (d.kernel < FD23_KERNEL_AUTO || d.kernel > FD23_KERNEL_FUSED2) return FD23_ERR_ARG;
    if (d.kernel == FD23_KERNEL_FUSED2 && (d.wave != FD23_PSV || d.prec != FD23_F32)) return FD23_ERR_UNSUPPORTED;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || d.device < 0 || d.device >= ndev) {
        cudaGetLastError();
        return FD23_ERR_CUDA;
    }
    CK(cudaSetDevice(d.device));
    fd23_solver *s = new (std::nothrow) fd23_solver();
    if (!s) return FD23_ERR_NOMEM;
    s->d = d;
    s->nfld = d.wave == FD23_PSV ? 5 : 3;
    s->nmat = d.wave == FD23_PSV ? 5 : 3;
    s->npsi = d.wave == FD23_PSV ? 8 : 4;
    s->es = storage_size(d.prec);
    s->cs = compute_size(d.prec);
    s->fused = d.kernel == FD23_KERNEL_AUTO || d.kernel == FD23_KERNEL_FUSED || d.kernel == FD23_KERNEL_FUSED2;
    s->fused2 = d.kernel == FD23_KERNEL_FUSED2;
    s->persist = d.kernel == FD23_KERNEL_PERSIST;
    if (const char *v = getenv("FD23_COST_XPML")) s->tune.wx = atof(v);
    if (const char *v = getenv("FD23_COST_ZPML")) s->tune.wz = atof(v);
    const FusedGeom g = fused_geom(d.wave, d.prec);
    const int ntx = (d.nx + g.tile_x - 1) / g.tile_x;
    s->L = make_layout(d.nx, d.nz, ntx * g.tile_x, (d.nz + 3) / 4 * 4);
    int rc = FD23_OK;
    auto fail = [&](int r) {
        free_all(s);
        delete s;
        return r;
    };
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(FD23_ERR_CUDA);
    const size_t gbytes = s->L.elems() * s->es;
    for (int b = 0; b < 2; ++b) {
        if ((rc = dev_alloc(&s->fld_block[b], s->nfld * gbytes))) return fail(rc);
        for (int f = 0; f < s->nfld; ++f) s->fld[b][f] = (unsigned char *)s->fld_block[b] + f * gbytes;
    }
    if ((rc = dev_alloc(&s->mat_block, s->nmat * gbytes))) return fail(rc);
    if (cudaMemset(s->mat_block, 0, s->nmat * gbytes) != cudaSuccess) return fail(FD23_ERR_CUDA);
    for (int m = 0; m < s->nmat; ++m) s->mat[m] = (unsigned char *)s->mat_block + m * gbytes;
    const size_t px = 2ull * d.npml * d.nz, pz = 2ull * d.npml * d.nx;
    for (int p = 0; p < s->npsi; ++p) s->psi_elems[p] = (p < s->npsi / 2) ? px : pz;
    for (int b = 0; b < 2; ++b)
        for (int p = 0; p < s->npsi; ++p)
            if ((rc = dev_alloc(&s->psi[b][p], std::max<size_t>(1, s->psi_elems[p]) * s->cs))) return fail(rc);
    std::vector<double> bck;
    build_cpml(d.wave, d.nx, d.nz, d.npml, d.pml_dt, d.pml_r, d.pml_v, d.pml_fc, bck);
    s->cpml_blk = (int)(bck.size() / 3);
    if ((rc = dev_alloc(&s->cpml, bck.size() * s->cs))) return fail(rc);
    if ((rc = upload_cpml(s, bck))) return fail(rc);
    if ((rc = dev_alloc((void **)&s->err_flag, sizeof(int)))) return fail(rc);
    if (s->persist && (rc = dev_alloc((void **)&s->d_bar, 2 * sizeof(unsigned)))) return fail(rc);
    if ((rc = dev_alloc((void **)&s->norm_buf, 2 * sizeof(double)))) return fail(rc);
    if (s->fused) {
        if ((rc = fused_prepare(d.wave, d.prec))) return fail(rc);
        if ((rc = build_worklist(s))) return fail(rc);
        if ((rc = encode_maps(s))) return fail(rc);
    }
    if (s->fused2) {
        for (int p = 0; p < s->npsi; ++p)
            if ((rc = dev_alloc(&s->psi_mid[p], std::max<size_t>(1, s->psi_elems[p]) * s->cs))) return fail(rc);
        s->f2_width = 256;
        if (const char *v = getenv("FD23_FUSED2_WIDTH")) s->f2_width = atoi(v) == 128 ? 128 : 256;
        if ((rc = fused2_prepare(false, s->f2_width))) return fail(rc);
        if ((rc = build_worklist2(s))) return fail(rc);
        if ((rc = encode_maps2(s))) return fail(rc);
    }
    if ((rc = zero_state(s))) return fail(rc);
    if (cudaStreamSynchronize(s->stream) != cudaSuccess) return fail(FD23_ERR_CUDA);
    *out = s;
    return FD23_OK;
}

void fd23_destroy(fd23_solver *s)
{
    if (!s) return;
    cudaSetDevice(s->d.device);
    cudaStreamSynchronize(s->stream);
    free_all(s);
    delete s;
}

int fd23_set_material(fd23_solver *s, const double *matv)
{
    if (!s || !matv) return FD23_ERR_ARG;
    CK(cudaSetDevice(s->d.device));
    const size_t n = (size_t)s->d.nx * s->d.nz;
    const int nms = s->d.wave == FD23_PSV ? 3 : 2;  // stress-update arrays come first
    if (scaled_form(s) && !s->kappa_set) {
        // kappa: power of two that brings the largest stress-update and
        // velocity-update coefficients to the same magnitude
        double ms = 0.0, mv = 0.0;
        for (int m = 0; m < s->nmat; ++m)
            for (size_t k = 0; k < n; ++k) {
                const double v = std::fabs(matv[m * n + k]);
                if (m < nms) ms = std::max(ms, v);
                else mv = std::max(mv, v);
            }
        s->kappa = (ms > 0 && mv > 0) ? pow2_round(std::sqrt(mv / ms)) : 1.0;
        s->kappa_set = true;
        int rc = upload_source_amps(s);
        if (rc) return rc;
    }
    std::vector<unsigned char> tmp(n * s->es);
    std::vector<double> scaled;
    for (int m = 0; m < s->nmat; ++m) {
        const double *src = matv + m * n;
        if (s->kappa != 1.0) {
            const double f = m < nms ? s->kappa : 1.0 / s->kappa;
            scaled.assign(src, src + n);
            for (auto &v : scaled) v *= f;
            src = scaled.data();
        }
        to_storage(s->d.prec, src, n, tmp.data());
        int rc = upload_grid(s, s->mat[m], tmp.data(), s->es);
        if (rc) return rc;
        CK(cudaStreamSynchronize(s->stream));
    }
    return material_done(s);
}

int fd23_set_model(fd23_solver *s, const double *vp, const double *vs, const double *den, double *stab)
{
    if (!s || !vs || !den || (s->d.wave == FD23_PSV && !vp)) return FD23_ERR_ARG;
    const size_t n = (size_t)s->d.nx * s->d.nz;
    // built on the device from vp, vs, den: the host builder's arithmetic
    // (and for the 16-bit forms fd23_set_material's scaling and rounding)
    const double st = material_stab(s->d.wave, vp, vs, n, s->d.h, s->d.dt);
    if (stab) *stab = st;
    if (st > 1.0) return FD23_ERR_UNSTABLE;
    CK(cudaSetDevice(s->d.device));
    const int rc = build_material_device(s, vp, vs, den);
    if (rc) return rc;
    return material_done(s);
}

int fd23_set_cpml(fd23_solver *s, const double *bckp)
{
    if (!s || !bckp) return FD23_ERR_ARG;
    CK(cudaSetDevice(s->d.device));
    std::vector<double> bck(bckp, bckp + 3 * (size_t)s->cpml_blk);
    return upload_cpml(s, bck);
}

int fd23_set_source_terms(fd23_solver *s, int nterms, const int *field, const int *ix, const int *iz,
                          const double *amp, int nt_amp)
{
    if (!s || nterms < 0 || nterms > 16 || (nterms > 0 && (!field || !ix || !iz || !amp || nt_amp <= 0)))
        return FD23_ERR_ARG;
    CK(cudaSetDevice(s->d.device));
    std::vector<int4> t((size_t)std::max(nterms, 1));
    for (int k = 0; k < nterms; ++k) {
        if (field[k] < 0 || field[k] >= s->nfld) return FD23_ERR_ARG;
        if (s->d.wave == FD23_PSV && field[k] < FD23_TXX) return FD23_ERR_ARG;  // stress terms only
        if (ix[k] < 0 || ix[k] >= s->d.nx || iz[k] < 0 || iz[k] >= s->d.nz) return FD23_ERR_ARG;
        t[k] = make_int4(field[k], ix[k], iz[k], 0);
    }
    cudaFree(s->d_terms);
    cudaFree(s->d_tamp);
    s->d_terms = nullptr;
    s->d_tamp = nullptr;
    s->nterms = 0;
    if (nterms == 0) return FD23_OK;
    int rc = dev_alloc((void **)&s->d_terms, t.size() * sizeof(int4));
    if (rc) return rc;
    const size_t na = (size_t)nterms * nt_amp;
    if ((rc = dev_alloc(&s->d_tamp, na * s->cs))) return rc;
    CK(cudaMemcpy(s->d_terms, t.data(), nterms * sizeof(int4), cudaMemcpyHostToDevice));
    s->nterms = nterms;
    s->tamp_nt = nt_amp;
    s->h_tfield.assign(field, field + nterms);
    s->h_tamp.assign(amp, amp + na);
    s->h_tcell.clear();
    for (int k = 0; k < nterms; ++k) s->h_tcell.push_back(make_int2(ix[k], iz[k]));
    ++s->punch_ver;
    return upload_source_amps(s);
}

int fd23_set_source(fd23_solver *s, int kind, int xs, int zs, const double *moment, const double *src,
                    int lsrc, int nt_max)
{
    if (!s || !src || lsrc <= 0 || nt_max <= 0) return FD23_ERR_ARG;
    if (kind != FD23_SRC_EXPLOSION && kind != FD23_SRC_FORCE && kind != FD23_SRC_MOMENT &&
        kind != FD23_SRC_MOMENT_P)
        return FD23_ERR_ARG;
    if (kind == FD23_SRC_FORCE && s->d.wave != FD23_SH) return FD23_ERR_ARG;
    if (kind == FD23_SRC_EXPLOSION && s->d.wave != FD23_PSV) return FD23_ERR_ARG;
    if (kind != FD23_SRC_EXPLOSION && !moment) return FD23_ERR_ARG;
    std::vector<SourceTerm> terms;
    std::vector<double> amp;
    build_source_terms(s->d.wave, kind, xs, zs, moment, s->d.h, s->d.dt, src, lsrc, nt_max, terms, amp);
    std::vector<int> f, x, z;
    for (auto &t : terms) {
        f.push_back(t.field);
        x.push_back(t.ix);
        z.push_back(t.iz);
    }
    return fd23_set_source_terms(s, (int)terms.size(), f.data(), x.data(), z.data(), amp.data(), nt_max);
}

int fd23_set_receivers(fd23_solver *s, int field, const int *rx, const int *rz, int n)
{
    if (!s || n < 0 || (n > 0 && (!rx || !rz))) return FD23_ERR_ARG;
    if (field < 0 || field >= s->nfld) return FD23_ERR_ARG;
    if (s->nrec_steps > 0) return FD23_ERR_ORDER;  // change receivers only before recording
    CK(cudaSetDevice(s->d.device));
    std::vector<long long> off((size_t)std::max(n, 1));
    for (int i = 0; i < n; ++i) {
        if (rx[i] < 0 || rx[i] >= s->d.nx || rz[i] < 0 || rz[i] >= s->d.nz) return FD23_ERR_ARG;
        off[i] = s->L.origin + (long long)rz[i] * s->L.pitch + rx[i];
    }
    s->h_rx[field].assign(rx, rx + n);
    s->h_rz[field].assign(rz, rz + n);
    s->rec2_dirty = true;
    cudaFree(s->d_rec[field]);
    cudaFree(s->d_seis[field]);
    s->d_rec[field] = nullptr;
    s->d_seis[field] = nullptr;
    s->nrec[field] = n;
    s->rec_cap = 0;
    for (int c = 0; c < 5; ++c) {  // record buffers are re-sized together
        cudaFree(s->d_seis[c]);
        s->d_seis[c] = nullptr;
    }
    if (n == 0) return FD23_OK;
    int rc = dev_alloc((void **)&s->d_rec[field], off.size() * sizeof(long long));
    if (rc) return rc;
    CK(cudaMemcpy(s->d_rec[field], off.data(), n * sizeof(long long), cudaMemcpyHostToDevice));
    return FD23_OK;
}

int fd23_receivers_line(int nsta, int ix0, int iz0, int idx, int idz, int *rx, int *rz)
{
    // PD/record/cu_record.cu:12-28: station i at (ix0+i*idx, iz0+i*idz),
    // recorded as the pair (x, z), (x-1, z)
    if (nsta < 0 || !rx || !rz) return FD23_ERR_ARG;
    for (int i = 0; i < nsta; ++i) {
        rx[2 * i] = ix0 + idx * i;
        rz[2 * i] = iz0 + idz * i;
        rx[2 * i + 1] = rx[2 * i] - 1;
        rz[2 * i + 1] = rz[2 * i];
    }
    return 2 * nsta;
}

int fd23_run(fd23_solver *s, int nsteps, int itrecord)
{
    if (!s || nsteps < 0 || itrecord <= 0) return FD23_ERR_ARG;
    if (!s->have_material) return FD23_ERR_ORDER;
    CK(cudaSetDevice(s->d.device));
    int rc0 = ensure_sigma(s);
    if (rc0) return rc0;
    int nrec_new = 0;
    for (int k = 0; k < nsteps; ++k)
        if ((s->it + k) % itrecord == 0) ++nrec_new;
    bool any_rec = false;
    for (int c = 0; c < 5; ++c) any_rec = any_rec || s->nrec[c] > 0;
    if (s->box_on && (s->it < s->box_inc_it0 || s->it + nsteps > s->box_inc_it0 + s->box_inc_n))
        return FD23_ERR_ORDER;  // incident field of some step not loaded
    if (any_rec) {
        int rc = ensure_record_capacity(s, s->nrec_steps + nrec_new);
        if (rc) return rc;
    }
    if (s->persist && !s->box_on) {
        // the whole run in one cooperative launch
        if (nsteps == 0) return FD23_OK;
        const int rc = dispatch_persist(s, nsteps, itrecord, any_rec);
        if (rc) return rc;
        s->it += nsteps;
        if (any_rec) s->nrec_steps += nrec_new;
        return FD23_OK;
    }
    const bool two = s->fused2 && !s->box_on && !s->d_punch && !s->d_midx;
    if (two && any_rec && s->rec2_dirty) {
        int rc = build_rec2(s);
        if (rc) return rc;
    }
    for (int k = 0; k < nsteps;) {
        const int rec_now = any_rec && (s->it % itrecord == 0);
        if (two && nsteps - k >= 2) {
            const int rec_next = any_rec && ((s->it + 1) % itrecord == 0);
            int rc = step2_impl(s, rec_now, rec_next);
            if (rc) return rc;
            k += 2;
            continue;
        }
        int rc = dispatch_step(s, rec_now, k + 1 < nsteps);
        if (rc) {
            s->box_pre_ahead = false;
            return rc;
        }
        ++k;
    }
    return dispatch_flush(s);
}

int fd23_sync(fd23_solver *s)
{
    if (!s) return FD23_ERR_ARG;
    CK(cudaSetDevice(s->d.device));
    CK(cudaStreamSynchronize(s->stream));
    int flag = 0;
    CK(cudaMemcpy(&flag, s->err_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag == 2) return FD23_ERR_UNSUPPORTED;  // shared-memory layout check failed
    return flag ? FD23_ERR_TIMEOUT : FD23_OK;
}

int fd23_get_stream(fd23_solver *s, void **stream)
{
    if (!s || !stream) return FD23_ERR_ARG;
    *stream = (void *)s->stream;
    return FD23_OK;
}

int fd23_get_field_device(fd23_solver *s, int field, void **dev_ptr, size_t *elems)
{
    if (!s || !dev_ptr || !elems || field < 0 || field >= s->nfld) return FD23_ERR_ARG;
    *dev_ptr = s->fld[s->par][field];
    *elems = s->L.elems();
    return FD23_OK;
}

int fd23_get_step(fd23_solver *s, int *it)
{
    if (!s || !it) return FD23_ERR_ARG;
    *it = s->it;
    return FD23_OK;
}

int fd23_get_seismograms(fd23_solver *s, int field, void *out, size_t out_bytes, int *nrec_steps)
{
    if (!s) return FD23_ERR_ARG;
    if (field < 0 || field >= s->nfld) return FD23_ERR_ARG;
    int rc = fd23_sync(s);
    if (rc) return rc;
    if (nrec_steps) *nrec_steps = s->nrec_steps;
    const size_t need = (size_t)s->nrec_steps * s->nrec[field] * s->cs;
    if (!out) return FD23_OK;
    if (out_bytes < need) return FD23_ERR_ARG;
    if (need) CK(cudaMemcpy(out, s->d_seis[field], need, cudaMemcpyDeviceToHost));
    if (field_scale(s, field) != 1.0) {  // stored times an exact power of two
        const float inv = (float)(1.0 / field_scale(s, field));
        float *o = (float *)out;
        for (size_t k = 0; k < need / sizeof(float); ++k) o[k] *= inv;
    }
    return FD23_OK;
}

int fd23_reset(fd23_solver *s)
{
    if (!s) return FD23_ERR_ARG;
    CK(cudaSetDevice(s->d.device));
    int rc = zero_state(s);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s->stream));
    return FD23_OK;
}

size_t fd23_state_bytes(fd23_solver *s)
{
    if (!s) return 0;
    size_t n = (size_t)s->nfld * s->d.nx * s->d.nz;
    for (int p = 0; p < s->npsi; ++p) n += s->psi_elems[p];
    return n * s->cs;
}

int fd23_get_state(fd23_solver *s, void *buf, size_t bytes)
{
    if (!s || !buf || bytes < fd23_state_bytes(s)) return FD23_ERR_ARG;
    int rc = ensure_sigma(s);
    if (rc) return rc;
    rc = fd23_sync(s);
    if (rc) return rc;
    const size_t n = (size_t)s->d.nx * s->d.nz;
    unsigned char *o = (unsigned char *)buf;
    std::vector<unsigned char> tmp(n * s->es);
    for (int f = 0; f < s->nfld; ++f) {
        // reference order P-SV: U W Txx Txz Tzz; SH: V Tx Tz (same as storage order)
        if ((rc = download_grid(s, s->fld[s->par][f], tmp.data(), s->es))) return rc;
        CK(cudaStreamSynchronize(s->stream));
        storage_to_compute(s->d.prec, tmp.data(), n, o);
        if (scaled_form(s)) {
            const float inv = (float)(1.0 / field_scale(s, f));
            for (size_t k = 0; k < n; ++k) ((float *)o)[k] *= inv;
        }
        o += n * s->cs;
    }
    for (int p = 0; p < s->npsi; ++p) {
        const size_t b = s->psi_elems[p] * s->cs;
        if (b) CK(cudaMemcpy(o, s->psi[s->par][p], b, cudaMemcpyDeviceToHost));
        if (scaled_form(s)) {
            const float inv = (float)(1.0 / psi_scale(s, p));
            for (size_t k = 0; k < s->psi_elems[p]; ++k) ((float *)o)[k] *= inv;
        }
        o += b;
    }
    return FD23_OK;
}

int fd23_set_state(fd23_solver *s, const void *buf, size_t bytes, int it0)
{
    if (!s || !buf || bytes < fd23_state_bytes(s) || it0 < 0) return FD23_ERR_ARG;
    CK(cudaSetDevice(s->d.device));
    int rc = zero_state(s);
    if (rc) return rc;
    if ((rc = ensure_sigma(s))) return rc;
    const size_t n = (size_t)s->d.nx * s->d.nz;
    const unsigned char *in = (const unsigned char *)buf;
    std::vector<unsigned char> tmp(n * s->es);
    std::vector<float> sc;
    for (int f = 0; f < s->nfld; ++f) {
        if (scaled_form(s)) {
            const float m = (float)field_scale(s, f);
            sc.assign((const float *)in, (const float *)in + n);
            for (auto &v : sc) v *= m;
            compute_to_storage(s->d.prec, (const unsigned char *)sc.data(), n, tmp.data());
        } else
        compute_to_storage(s->d.prec, in, n, tmp.data());
        if ((rc = upload_grid(s, s->fld[0][f], tmp.data(), s->es))) return rc;
        CK(cudaStreamSynchronize(s->stream));
        in += n * s->cs;
    }
    for (int p = 0; p < s->npsi; ++p) {
        const size_t b = s->psi_elems[p] * s->cs;
        if (b && scaled_form(s)) {
            const float m = (float)psi_scale(s, p);
            sc.assign((const float *)in, (const float *)in + s->psi_elems[p]);
            for (auto &v : sc) v *= m;
            CK(cudaMemcpy(s->psi[0][p], sc.data(), b, cudaMemcpyHostToDevice));
        } else if (b) {
            CK(cudaMemcpy(s->psi[0][p], in, b, cudaMemcpyHostToDevice));
        }
        in += b;
    }
    s->it = it0;
    s->par = 0;
    // the fused sweep may leave steady tiles alone: both sets hold the state
    return mirror_sets(s, s->stream);
}

int fd23_field_norm2(fd23_solver *s, double *norm2)
{
    if (!s || !norm2) return FD23_ERR_ARG;
    CK(cudaSetDevice(s->d.device));
    int rc = FD23_OK;
    switch (s->d.prec) {
        case FD23_F64: rc = launch_norm2<double, double>(make_shot<double, double>(s), s->par, s->nfld, (long long)s->L.elems(), s->norm_buf, s->stream); break;
        case FD23_BF16: rc = launch_norm2<__nv_bfloat16, float>(make_shot<__nv_bfloat16, float>(s), s->par, s->nfld, (long long)s->L.elems(), s->norm_buf, s->stream); break;
        case FD23_F16: rc = launch_norm2<__half, float>(make_shot<__half, float>(s), s->par, s->nfld, (long long)s->L.elems(), s->norm_buf, s->stream); break;
        default: rc = launch_norm2<float, float>(make_shot<float, float>(s), s->par, s->nfld, (long long)s->L.elems(), s->norm_buf, s->stream);
    }
    if (rc) return rc;
    double h[2];
    CK(cudaMemcpyAsync(h, s->norm_buf, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    *norm2 = h[0];
    return h[1] != 0.0 ? FD23_ERR_NONFINITE : FD23_OK;
}

int fd23_debug_expire_wait(fd23_solver *s)
{
    if (!s) return FD23_ERR_ARG;
    CK(cudaSetDevice(s->d.device));
    return launch_wait_probe(s->err_flag, s->stream);
}

int fd23_debug_persist_barrier(fd23_solver *s)
{
    if (!s) return FD23_ERR_ARG;
    if (!s->persist || !s->have_material) return FD23_ERR_ORDER;
    CK(cudaSetDevice(s->d.device));
    switch (s->d.prec) {
        case FD23_F64:
            return launch_persist<double, double>(make_shot<double, double>(s), s->d.wave, s->it, 1, 1, 0, 0,
                                                  s->d_bar, s->err_flag, s->stream, true);
        case FD23_BF16:
            return launch_persist<__nv_bfloat16, float>(make_shot<__nv_bfloat16, float>(s), s->d.wave, s->it, 1, 1, 0,
                                                        0, s->d_bar, s->err_flag, s->stream, true);
        case FD23_F16:
            return launch_persist<__half, float>(make_shot<__half, float>(s), s->d.wave, s->it, 1, 1, 0, 0, s->d_bar,
                                                 s->err_flag, s->stream, true);
        default:
            return launch_persist<float, float>(make_shot<float, float>(s), s->d.wave, s->it, 1, 1, 0, 0, s->d_bar,
                                                s->err_flag, s->stream, true);
    }
}

// ---- hybrid box ----
int fd23_set_box(fd23_solver *s, int x0, int z0, int bx, int bz, const double *bmat)
{
    if (!s) return FD23_ERR_ARG;
    CK(cudaSetDevice(s->d.device));
    CK(cudaStreamSynchronize(s->stream));
    if (bx == 0 && bz == 0) {
        free_box(s);
        return FD23_OK;
    }
    if (s->d.wave != FD23_PSV || scaled_form(s) || s->d_punch || s->table_on) return FD23_ERR_UNSUPPORTED;
    if (bx < kBoxMin || bz < kBoxMin || x0 < 0 || z0 < 0 || x0 + bx > s->d.nx || z0 + bz > s->d.nz)
        return FD23_ERR_ARG;
    if (!bmat && !s->have_material) return FD23_ERR_ORDER;
    int rc = box_alloc(s, x0, z0, bx, bz);
    if (rc) return rc;
    const size_t nb = (size_t)bx * bz, bytes = nb * s->cs;
    if (bmat) {
        std::vector<unsigned char> tmp(bytes);
        for (int m = 0; m < 5; ++m) {
            to_compute(s->d.prec, bmat + m * nb, nb, tmp.data());
            CK(cudaMemcpy(s->box_mat[m], tmp.data(), bytes, cudaMemcpyHostToDevice));
        }
    } else {
        // the box cut of the grid material (storage type = compute type here)
        for (int m = 0; m < 5; ++m)
            CK(cudaMemcpy2DAsync(s->box_mat[m], (size_t)bx * s->cs,
                                 (const unsigned char *)s->mat[m] +
                                     (size_t)(s->L.origin + (long long)z0 * s->L.pitch + x0) * s->es,
                                 (size_t)s->L.pitch * s->es, (size_t)bx * s->es, (size_t)bz,
                                 cudaMemcpyDeviceToDevice, s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));
    return FD23_OK;
}

int fd23_set_model_box(fd23_solver *s, const double *vp, const double *vs, const double *den, int x0, int z0,
                       int bx, int bz, double src_vp, double src_vs, double src_den, double *stab, int *replaced,
                       double *bmat)
{
    if (!s || !vp || !vs || !den) return FD23_ERR_ARG;
    if (s->d.wave != FD23_PSV || scaled_form(s) || s->d_punch || s->table_on) return FD23_ERR_UNSUPPORTED;
    if (bx < kBoxMin || bz < kBoxMin || x0 < 0 || z0 < 0 || x0 + bx > s->d.nx || z0 + bz > s->d.nz)
        return FD23_ERR_ARG;
    const double st = material_stab(s->d.wave, vp, vs, (size_t)s->d.nx * s->d.nz, s->d.h, s->d.dt);
    if (stab) *stab = st;
    if (st > 1.0) return FD23_ERR_UNSTABLE;
    CK(cudaSetDevice(s->d.device));
    CK(cudaStreamSynchronize(s->stream));
    int rc = box_alloc(s, x0, z0, bx, bz);
    if (!rc)
        rc = build_material_box_device(s, vp, vs, den, x0, z0, bx, bz, src_vp, src_vs, src_den, replaced, bmat);
    if (rc) {
        free_box(s);
        return rc;
    }
    return material_done(s);
}

}  // extern "C"

namespace fd23 {

// The box's arrays (residual r zeroed; material arrays allocated, not filled)
// and its ring list; the box is then on
int box_alloc(fd23_solver *s, int x0, int z0, int bx, int bz)
{
    free_box(s);
    const size_t nb = (size_t)bx * bz, bytes = nb * s->cs;
    int rc = FD23_OK;
    for (int f = 0; f < 5; ++f) {
        if ((rc = dev_alloc(&s->box_r[f], bytes)) || (rc = dev_alloc(&s->box_mat[f], bytes))) {
            free_box(s);
            return rc;
        }
        CK(cudaMemsetAsync(s->box_r[f], 0, bytes, s->stream));
    }
    // ring cells in incident-field order; the closed-form position used by
    // the sweep must agree with the enumeration
    std::vector<int2> cells;
    for (int pass = 0; pass < 2; ++pass) {
        const int lo = pass ? 4 : 0, hx = pass ? bx - 4 : bx, hz = pass ? bz - 4 : bz;
        for (int j = lo; j < hz; ++j)
            for (int i = lo; i < hx; ++i)
                if (!(i > lo + 3 && i < hx - 4 && j > lo + 3 && j < hz - 4)) cells.push_back(make_int2(i, j));
    }
    for (size_t q = 0; q < cells.size(); ++q)
        if (box_ring_index(cells[q].x, cells[q].y, bx, bz) != (int)q) {
            free_box(s);
            return FD23_ERR_UNSUPPORTED;
        }
    if ((rc = dev_alloc((void **)&s->box_cells, cells.size() * sizeof(int2)))) {
        free_box(s);
        return rc;
    }
    CK(cudaMemcpy(s->box_cells, cells.data(), cells.size() * sizeof(int2), cudaMemcpyHostToDevice));
    CK(cudaStreamSynchronize(s->stream));
    s->box_x0 = x0;
    s->box_z0 = z0;
    s->box_bx = bx;
    s->box_bz = bz;
    s->box_nsub = box_nsub(bx, bz);
    s->box_nring = (int)cells.size();
    s->box_on = true;
    s->box_inc_n = 0;
    return FD23_OK;
}

}  // namespace fd23

extern "C" {

int fd23_set_box_incident(fd23_solver *s, const void *inc, int it0, int nsteps)
{
    if (!s || it0 < 0 || nsteps < 0 || (nsteps > 0 && !inc)) return FD23_ERR_ARG;
    if (!s->box_on) return FD23_ERR_ORDER;
    CK(cudaSetDevice(s->d.device));
    if (s->copy_stream) CK(cudaStreamSynchronize(s->copy_stream));  // an earlier asynchronous upload
    s->inc_chunk = 0;
    const size_t bytes = (size_t)nsteps * 5 * s->box_nring * s->cs;
    if (bytes > s->box_inc_bytes) {
        CK(cudaStreamSynchronize(s->stream));
        cudaFree(s->box_inc);
        s->box_inc = nullptr;
        s->box_inc_bytes = 0;
        s->box_inc_n = 0;
        int rc = dev_alloc(&s->box_inc, bytes);
        if (rc) return rc;
        s->box_inc_bytes = bytes;
    }
    if (bytes) {
        CK(cudaMemcpyAsync(s->box_inc, inc, bytes, cudaMemcpyHostToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    s->box_inc_it0 = it0;
    s->box_inc_n = nsteps;
    return FD23_OK;
}

int fd23_set_box_incident_async(fd23_solver *s, const void *inc, int it0, int nsteps)
{
    if (!s || it0 < 0 || nsteps < 0 || (nsteps > 0 && !inc)) return FD23_ERR_ARG;
    if (!s->box_on) return FD23_ERR_ORDER;
    CK(cudaSetDevice(s->d.device));
    if (!s->copy_stream) CK(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
    if (!s->inc_gate) CK(cudaEventCreateWithFlags(&s->inc_gate, cudaEventDisableTiming));
    CK(cudaStreamSynchronize(s->copy_stream));  // an earlier asynchronous upload
    s->inc_chunk = 0;
    const size_t step_bytes = (size_t)5 * s->box_nring * s->cs;
    const size_t bytes = (size_t)nsteps * step_bytes;
    if (bytes > s->box_inc_bytes) {
        CK(cudaStreamSynchronize(s->stream));
        cudaFree(s->box_inc);
        s->box_inc = nullptr;
        s->box_inc_bytes = 0;
        s->box_inc_n = 0;
        int rc = dev_alloc(&s->box_inc, bytes);
        if (rc) return rc;
        s->box_inc_bytes = bytes;
    } else {
        // work already queued on the solver's stream may read the old field
        CK(cudaEventRecord(s->inc_gate, s->stream));
        CK(cudaStreamWaitEvent(s->copy_stream, s->inc_gate, 0));
    }
    // chunks of 64 steps, each followed by its event
    const int chunk = 64;
    const int nch = (nsteps + chunk - 1) / chunk;
    while ((int)s->inc_ev.size() < nch) {
        cudaEvent_t e = nullptr;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        s->inc_ev.push_back(e);
    }
    for (int c = 0; c < nch; ++c) {
        const size_t off = (size_t)c * chunk * step_bytes;
        const size_t len = (size_t)std::min(chunk, nsteps - c * chunk) * step_bytes;
        CK(cudaMemcpyAsync((unsigned char *)s->box_inc + off, (const unsigned char *)inc + off, len,
                           cudaMemcpyHostToDevice, s->copy_stream));
        CK(cudaEventRecord(s->inc_ev[c], s->copy_stream));
    }
    s->box_inc_it0 = it0;
    s->box_inc_n = nsteps;
    s->inc_chunk = nsteps > 0 ? chunk : 0;
    s->inc_waited = 0;
    return FD23_OK;
}


size_t fd23_box_state_bytes(fd23_solver *s)
{
    return (s && s->box_on) ? 5 * (size_t)s->box_bx * s->box_bz * s->cs : 0;
}

int fd23_get_box_state(fd23_solver *s, void *buf, size_t bytes)
{
    if (!s || !buf) return FD23_ERR_ARG;
    if (!s->box_on) return FD23_ERR_ORDER;
    if (bytes < fd23_box_state_bytes(s)) return FD23_ERR_ARG;
    int rc = fd23_sync(s);
    if (rc) return rc;
    const size_t b = (size_t)s->box_bx * s->box_bz * s->cs;
    for (int f = 0; f < 5; ++f) CK(cudaMemcpy((unsigned char *)buf + f * b, s->box_r[f], b, cudaMemcpyDeviceToHost));
    return FD23_OK;
}

int fd23_set_box_state(fd23_solver *s, const void *buf, size_t bytes)
{
    if (!s || !buf) return FD23_ERR_ARG;
    if (!s->box_on) return FD23_ERR_ORDER;
    if (bytes < fd23_box_state_bytes(s)) return FD23_ERR_ARG;
    CK(cudaSetDevice(s->d.device));
    CK(cudaStreamSynchronize(s->stream));
    const size_t b = (size_t)s->box_bx * s->box_bz * s->cs;
    for (int f = 0; f < 5; ++f)
        CK(cudaMemcpy(s->box_r[f], (const unsigned char *)buf + f * b, b, cudaMemcpyHostToDevice));
    return FD23_OK;
}

int fd23_box_ring_size(int bx, int bz, int *nsub, int *nadd)
{
    if (bx < kBoxMin || bz < kBoxMin) return FD23_ERR_ARG;
    if (nsub) *nsub = box_nsub(bx, bz);
    if (nadd) *nadd = box_nadd(bx, bz);
    return box_nsub(bx, bz) + box_nadd(bx, bz);
}

int fd23_box_ring_index(int bx, int bz, int bi, int bj)
{
    if (bx < kBoxMin || bz < kBoxMin) return FD23_ERR_ARG;
    return box_ring_index(bi, bj, bx, bz);
}

int fd23_box_ring_cells(int x0, int z0, int bx, int bz, int *ix, int *iz)
{
    if (bx < kBoxMin || bz < kBoxMin || !ix || !iz) return FD23_ERR_ARG;
    for (int j = 0; j < bz; ++j)
        for (int i = 0; i < bx; ++i) {
            const int q = box_ring_index(i, j, bx, bz);
            if (q < 0) continue;
            ix[q] = x0 + i;
            iz[q] = z0 + j;
        }
    return box_nsub(bx, bz) + box_nadd(bx, bz);
}

int fd23_box_incident_from_displacement(int bx, int bz, double dt, const double *bmat, const double *u_old,
                                        const double *w_old, const double *u_new, const double *w_new,
                                        double *out)
{
    if (bx < kBoxMin || bz < kBoxMin || !(dt > 0) || !bmat || !u_old || !w_old || !u_new || !w_new || !out)
        return FD23_ERR_ARG;
    return box_incident_from_displacement(bx, bz, dt, bmat, u_old, w_old, u_new, w_new, out);
}

int fd23_box_material(int nx, int nz, double *mat, int x0, int z0, int bx, int bz, double src_vp,
                      double src_vs, double src_den, double dt, double h, double *bmat)
{
    if (nx < 2 || nz < 2 || !mat || !bmat || bx < 1 || bz < 1 || x0 < 0 || z0 < 0 || x0 + bx > nx ||
        z0 + bz > nz || !(src_den > 0) || !(dt > 0) || !(h > 0))
        return FD23_ERR_ARG;
    return box_material(nx, nz, mat, x0, z0, bx, bz, src_vp, src_vs, src_den, dt, h, bmat);
}

// ---- host-only helpers (no GPU needed) ----
int fd23_build_material(int wave, int nx, int nz, double h, double dt, const double *vp, const double *vs,
                        const double *den, double *out, double *stab)
{
    if (nx < 2 || nz < 2 || !vs || !den || !out || (wave == FD23_PSV && !vp)) return FD23_ERR_ARG;
    return wave == FD23_PSV ? build_psv_material(nx, nz, h, dt, vp, vs, den, out, stab)
                            : build_sh_material(nx, nz, h, dt, vs, den, out, stab);
}

int fd23_build_cpml(int wave, int nx, int nz, int npml, double pml_dt, double pml_r, double pml_v,
                    double pml_fc, double *out, size_t out_elems)
{
    std::vector<double> bck;
    build_cpml(wave, nx, nz, npml, pml_dt, pml_r, pml_v, pml_fc, bck);
    if (!out || out_elems < bck.size()) return FD23_ERR_ARG;
    std::copy(bck.begin(), bck.end(), out);
    return (int)bck.size();
}

int fd23_build_source_terms(int wave, int kind, int xs, int zs, const double *moment, double h, double dt,
                            const double *src, int lsrc, int nt, int *field, int *ix, int *iz, double *amp,
                            int max_terms)
{
    if (!src || lsrc <= 0 || nt <= 0 || !field || !ix || !iz || !amp) return FD23_ERR_ARG;
    std::vector<SourceTerm> terms;
    std::vector<double> a;
    build_source_terms(wave, kind, xs, zs, moment, h, dt, src, lsrc, nt, terms, a);
    if ((int)terms.size() > max_terms) return FD23_ERR_ARG;
    for (size_t k = 0; k < terms.size(); ++k) {
        field[k] = terms[k].field;
        ix[k] = terms[k].ix;
        iz[k] = terms[k].iz;
    }
    std::copy(a.begin(), a.end(), amp);
    return (int)terms.size();
}

int fd23_wavelet_gaussian(double dt, int alpha, double *out, int cap) { return wavelet_gaussian(dt, alpha, out, cap); }
int fd23_wavelet_trapezoid(double dt, double t1, double t2, double t3, double *out, int cap)
{
    return wavelet_trapezoid(dt, t1, t2, t3, out, cap);
}
int fd23_wavelet_ricker(double dt, double f0, double t0, double *out, int cap)
{
    return wavelet_ricker(dt, f0, t0, out, cap);
}
void fd23_moment_psv(double strike, double dip, double rake, double azimuth, double out3[3])
{
    moment_psv(strike, dip, rake, azimuth, out3);
}
void fd23_moment_sh(double strike, double dip, double rake, double azimuth, double out2[2])
{
    moment_sh(strike, dip, rake, azimuth, out2);
}

}  // extern "C"
