// The solver object behind the C ABI and the helpers the API and the batch
// code share (fd23_api.cpp, fd23_batch.cpp).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "fd23_internal.h"
#include "fd23_kernels.h"

#define CK(call)                                      \
    do {                                              \
        if ((call) != cudaSuccess) {                  \
            cudaGetLastError();                       \
            return FD23_ERR_CUDA;                     \
        }                                             \
    } while (0)

struct fd23_solver {
    fd23_desc d{};
    int nfld = 0, nmat = 0, npsi = 0;
    size_t es = 4, cs = 4;  // storage / compute element size
    fd23::Layout L;
    cudaStream_t stream = nullptr;
    int fused = 1;
    bool persist = false;     // FD23_KERNEL_PERSIST: a run is one cooperative launch
    unsigned *d_bar = nullptr;  // its grid barrier (count, generation)
    void *fld[2][5] = {};   // wavefields; those of one buffer set are one allocation
    void *mat[5] = {};      // material arrays, one allocation
    void *fld_block[2] = {};
    void *mat_block = nullptr;
    fd23::ShotMaps *d_maps = nullptr;  // tensor maps of the fused sweep
    void *psi[2][8] = {};
    size_t psi_elems[8] = {};
    void *cpml = nullptr;
    int cpml_blk = 0;
    bool have_material = false;
    int *err_flag = nullptr;
    double *norm_buf = nullptr;
    // 16-bit storage forms keep values in range with exact power-of-two scales:
    // stored velocity = sigma * v, stored stress = sigma * kappa * T; the
    // stress-update material is stored times kappa, the velocity-update
    // material divided by kappa.  Both stay 1 for F32 / F64.
    double kappa = 1.0, sigma = 1.0;
    bool kappa_set = false, sigma_set = false;
    std::vector<int> h_tfield;      // source terms as given (for re-scaling)
    std::vector<double> h_tamp;
    // source
    int nterms = 0;
    int4 *d_terms = nullptr;
    void *d_tamp = nullptr;
    int tamp_nt = 0;
    // receivers, one list per wavefield
    int nrec[5] = {};
    long long *d_rec[5] = {};
    void *d_seis[5] = {};
    int rec_cap = 0;      // record rows allocated
    int nrec_steps = 0;   // record rows filled (or pending)
    int pending_rec = -1; // record row to gather from the current buffer set
    // time
    int it = 0;
    int par = 0;
    // fused work list
    fd23::WorkItem *d_items = nullptr;
    int *d_item_off = nullptr;
    int nblocks = 0;
    // work plan of the fused sweep and the parameters it was built with
    fd23::TuneParams tune;
    // hybrid box: residual field, box material, ring cells, incident field
    // of steps [box_inc_it0, box_inc_it0 + box_inc_n)
    // material table (device): indices (padded layout, bytes) and the table
    // [nmat][kTabEntries] of storage values; null when off
    unsigned char *d_midx = nullptr;
    void *d_mtab = nullptr;
    bool table_on = false;
    int table_n = 0;
    // usepunch tile step windows (device, [nbz][nbx] int2), null when off,
    // and their host copy
    int2 *d_punch = nullptr;
    int punch_nbx = 0, punch_nbz = 0;
    std::vector<int2> h_punch;
    // With windows the fused sweep runs on phase plans: work lists over the
    // 4-row blocks live at some step of a phase of punch_phase steps (0: the
    // static plan), built on the host and kept in a ring of device buffers
    // (reused once the event of their last launch has completed).
    struct PhasePlan {
        fd23::WorkItem *items = nullptr;
        int *off = nullptr;
        size_t cap_items = 0, cap_off = 0;
        void *host = nullptr;  // pinned staging of items + offsets
        size_t cap_host = 0;
        int nblocks = 0;
        long long key = -1;
        cudaEvent_t done = nullptr;
    };
    PhasePlan phase[3];
    int punch_phase = 128;
    long long punch_ver = 0;  // bumped when windows, sources or the tuning change
    int phase_next = 0;
    std::vector<int2> h_tcell;  // source-term cells (ix, iz)
    // two-step sweep (FD23_KERNEL_FUSED2): its work plan and tensor maps, the
    // memory variables of the step in between, the per-item receiver lists
    // of that step (rebuilt when receivers change), host copies of the
    // receiver positions
    bool fused2 = false;
    int f2_width = 256;  // strip width of the two-step sweep's CTAs (256 or 128)
    fd23::WorkItem *d_items2 = nullptr;
    int *d_item_off2 = nullptr;
    int nblocks2 = 0;
    std::vector<fd23::WorkItem> h_items2;
    std::vector<int> h_item_off2;
    fd23::ShotMaps2 *d_maps2 = nullptr;
    void *psi_mid[8] = {};
    int4 *d_rec2 = nullptr;
    int *d_rec2_off = nullptr;
    bool rec2_dirty = true;
    std::vector<int> h_rx[5], h_rz[5];
    bool box_on = false;
    int box_x0 = 0, box_z0 = 0, box_bx = 0, box_bz = 0, box_nsub = 0, box_nring = 0;
    void *box_r[5] = {};
    void *box_mat[5] = {};
    int2 *box_cells = nullptr;
    void *box_inc = nullptr;
    size_t box_inc_bytes = 0;
    int box_inc_it0 = 0, box_inc_n = 0;
    // the box's start-of-step work of step `it` already ran (with the end of
    // the step before, launch_box_mid)
    bool box_pre_ahead = false;
    // asynchronous incident upload (fd23_set_box_incident_async): chunk c
    // holds steps box_inc_it0 + c*inc_chunk .. +inc_chunk-1 and is on the
    // device once inc_ev[c] has completed; inc_waited: chunks the solver's
    // stream already waits for
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t inc_gate = nullptr;  // the solver's queued work, before the copies
    std::vector<cudaEvent_t> inc_ev;
    int inc_chunk = 0, inc_waited = 0;
};

namespace fd23 {

int dev_alloc(void **p, size_t bytes);
size_t storage_size(int prec);
size_t compute_size(int prec);
bool scaled_form(const fd23_solver *s);
double field_scale(const fd23_solver *s, int f);
int ensure_sigma(fd23_solver *s);
int ensure_record_capacity(fd23_solver *s, int need);
int dispatch_flush(fd23_solver *s);
int zero_state(fd23_solver *s);
int fused_per_sm(int device, int wave, int prec, bool batch = false);
int upload_plan(const WorkPlan &plan, WorkItem **d_items, int **d_off);
int build_worklist(fd23_solver *s);
int build_worklist2(fd23_solver *s);
int wait_incident(fd23_solver *s, int upto);  // asynchronous incident chunks up to step `upto`
// one step; more != 0: another step follows in the same run
int dispatch_step(fd23_solver *s, int rec_now, int more = 0);
// copies buffer set `par` (wavefields, memory variables) into the other set
int mirror_sets(fd23_solver *s, cudaStream_t st);
// the phase plan of step s->it (fd23_punch.cpp): slot of s->phase to use
int phase_plan(fd23_solver *s, int *slot);
// material table from the device material (fd23_table.cpp): FD23_OK, or
// FD23_ERR_UNSUPPORTED with more distinct tuples than the table holds
int build_material_table(fd23_solver *s);
// one nx x nz array between the host (row-major, es bytes per value) and the
// padded device layout
int upload_grid(fd23_solver *s, void *dptr, const unsigned char *host, size_t es);
int download_grid(fd23_solver *s, const void *dptr, unsigned char *host, size_t es);
void free_material_table(fd23_solver *s);
int encode_maps(fd23_solver *s);
// the material of vp, vs, den built on the device into the storage arrays
// (fd23_matgpu.cu; FP32 and FP64 storage, FD23_ERR_UNSUPPORTED otherwise)
int build_material_device(fd23_solver *s, const double *vp, const double *vs, const double *den);
// the same with the hybrid box homogenised (box_material's rule) and the box
// material stored into the box's arrays (P-SV, FP32 / FP64)
int build_material_box_device(fd23_solver *s, const double *vp, const double *vs, const double *den, int x0,
                              int z0, int bx, int bz, double src_vp, double src_vs, double src_den, int *replaced,
                              double *bmat_out);
int box_alloc(fd23_solver *s, int x0, int z0, int bx, int bz);
// 16-bit forms: the power-of-two scale of a value, the source amplitudes in
// the scaled units (once kappa is known)
double pow2_round(double v);
int upload_source_amps(fd23_solver *s);

template <class S, class C>
Shot<S, C> make_shot(const fd23_solver *s)
{
    Shot<S, C> sh{};
    for (int b = 0; b < 2; ++b)
        for (int f = 0; f < 5; ++f) sh.f[b][f] = (S *)s->fld[b][f];
    for (int m = 0; m < 5; ++m) sh.mat[m] = (const S *)s->mat[m];
    for (int b = 0; b < 2; ++b)
        for (int p = 0; p < 8; ++p) sh.psi[b][p] = (C *)s->psi[b][p];
    sh.cpml = (const C *)s->cpml;
    sh.nx = s->d.nx;
    sh.nz = s->d.nz;
    sh.npml = s->d.npml;
    sh.topabsorb = s->d.topabsorb;
    sh.pitch = s->L.pitch;
    sh.origin = s->L.origin;
    sh.cpml_blk = s->cpml_blk;
    sh.nterms = s->nterms;
    sh.terms = s->d_terms;
    sh.tamp = (const C *)s->d_tamp;
    sh.tamp_nt = s->nterms > 0 ? s->tamp_nt : 0;
    for (int c = 0; c < 5; ++c) {
        sh.nrec[c] = s->nrec[c];
        sh.rec[c] = s->d_rec[c];
        sh.seis[c] = (C *)s->d_seis[c];
    }
    sh.maps = s->d_maps;
    sh.cta0 = 0;
    sh.ncta = s->nblocks > 0 ? s->nblocks : 1;
    sh.punch = Punch{s->d_punch, s->punch_nbx, s->punch_nbz};
    sh.midx = s->d_midx;
    sh.mtab = (const S *)s->d_mtab;
    sh.maps2 = s->d_maps2;
    for (int m = 0; m < 5; ++m) sh.mat16[m] = nullptr;
    for (int p = 0; p < 8; ++p) sh.psim[p] = (C *)s->psi_mid[p];
    sh.rec2 = s->d_rec2;
    sh.rec2_off = s->d_rec2_off;
    sh.box.on = s->box_on ? 1 : 0;
    if (s->box_on) {
        sh.box.x0 = s->box_x0;
        sh.box.z0 = s->box_z0;
        sh.box.bx = s->box_bx;
        sh.box.bz = s->box_bz;
        sh.box.nsub = s->box_nsub;
        sh.box.nring = s->box_nring;
        for (int f = 0; f < 5; ++f) {
            sh.box.r[f] = (C *)s->box_r[f];
            sh.box.rmat[f] = (const C *)s->box_mat[f];
        }
        sh.box.cells = s->box_cells;
        // incident field of the current step
        const bool have = s->box_inc && s->it >= s->box_inc_it0 && s->it < s->box_inc_it0 + s->box_inc_n;
        sh.box.inc = have ? (const C *)((const unsigned char *)s->box_inc +
                                        (size_t)(s->it - s->box_inc_it0) * 5 * s->box_nring * s->cs)
                          : nullptr;
    }
    return sh;
}

}  // namespace fd23
