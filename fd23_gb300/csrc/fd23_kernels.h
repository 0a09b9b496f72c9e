// Launch entry points of the sweep kernels (host side).
#pragma once

#include <cuda_runtime.h>

#include "fd23_internal.h"

namespace fd23 {

// two-pass sweep, fields updated in place in buffer set 0 (cells outside
// their tile's step window return at once, as in the reference)
template <class S, class C>
int launch_step_twopass(const Shot<S, C> &s, int wave, int it, cudaStream_t st);

// steps it0 .. it0+nsteps-1 of the two-pass updates in one cooperative
// launch (small grids; buffer set 0 in place), grid barriers between the
// phases; record rows from rec_row on the steps with it % itrecord == 0
// (any_rec); bar: two zeroed words of device memory, err: the error flag;
// unreachable_barrier: the failure-path check (the first barrier waits for
// one arrival more than the grid has and gives up after a short limit)
template <class S, class C>
int launch_persist(const Shot<S, C> &s, int wave, int it0, int nsteps, int itrecord, int rec_row, int any_rec,
                   unsigned *bar, int *err, cudaStream_t st, bool unreachable_barrier = false);

// receiver gather from buffer set `par` into record row `rec_index`
template <class S, class C>
int launch_record(const Shot<S, C> &s, int par, int rec_index, cudaStream_t st);

// Fused single-pass sweep.  Geometry of its tiles (used to size the padded
// layout and to build the work list):
struct FusedGeom {
    int tile_x;   // output columns per strip
    int rows_per_iter;
};
FusedGeom fused_geom(int wave, int prec);
// copy shapes of the fused sweep (for the tensor maps): stencil-input row
// width, point-wise row width, fields per copy
struct FusedBoxes {
    int uww, pww, nv, nt, nms, nmv;
};
FusedBoxes fused_boxes(int wave, int prec);
int fused_prepare(int wave, int prec);       // once per device before the first launch
size_t fused_smem_bytes(int wave, int prec); // dynamic shared memory of one CTA
int fused_occupancy(int wave, int prec, bool batch);  // resident CTAs per SM (current device)

// One time step of every work item: reads buffer set `par`, writes `1-par`.
// `rec_index` >= 0 gathers the receivers of the previous step from buffer set
// `par` into that record row on the way.  `fast` != 0 selects the FP32
// sweep's instantiation with uniform fast iterations (other storage types and
// the window / table sweeps ignore it).
template <class S, class C>
int launch_step_fused(const Shot<S, C> &s, int wave, const WorkItem *items, const int *item_off,
                      int nblocks, int par, int it, int rec_index, int *err_flag, cudaStream_t st, int fast = 0);

// Hybrid box (P-SV), fd23_box.cu.  Ring exchange on buffer set `par`:
// which = 0 for U, W (start of a step), 1 for the stresses (after the stress
// update and the point source); add ring g = r + s, sub ring r = g - s.
template <class S, class C>
int launch_box_ring(const Shot<S, C> &s, int par, int which, cudaStream_t st);
// start of a step: ring exchange of U, W, then the residual stress update
// (fused != 0: which also stores g = r + s into the add-ring stresses of
// buffer set `par`, the fused sweep's part of the stress exchange)
template <class S, class C>
int launch_box_pre(const Shot<S, C> &s, int par, int fused, cudaStream_t st);
// end of a step: (fused != 0: sub-ring stresses r = g - s from buffer set
// `par`), receivers of buffer set `par` into record row `rec_index` (if >= 0),
// then the residual velocity update
template <class S, class C>
int launch_box_post(const Shot<S, C> &s, int par, int fused, int rec_index, cudaStream_t st);
// fused sweep, boxes of the one-CTA path: launch_box_post of this step and
// launch_box_pre of the next (incident field of step it+1 following that of
// step it) as one launch; FD23_ERR_UNSUPPORTED (nothing launched) for boxes
// too large for it
template <class S, class C>
int launch_box_mid(const Shot<S, C> &s, int par, int rec_index, cudaStream_t st);

// The same sweep over several shots in one launch: `shots` = device array of
// shot descriptors; every CTA's items belong to one shot (a WorkPlan).
// `punch`: some shot carries tile step windows (the sweep with windows
// runs); `table`: the shots carry material tables (all of them)
template <class S, class C>
int launch_step_fused_batch(const Shot<S, C> *shots, int wave, const WorkItem *items, const int *item_off,
                            int nblocks, int par, int it, int rec_index, int *err_flag, bool punch,
                            bool table, cudaStream_t st);

// The sweep with tile step windows (fd23_fused_punch.cu): one shot (`shots`
// null, descriptor `s`) or a shot table; called by the two launchers above.
template <class S, class C>
int launch_step_fused_punch(const Shot<S, C> &s, const Shot<S, C> *shots, int wave, const WorkItem *items,
                            const int *item_off, int nblocks, int par, int it, int rec_index, int *err_flag,
                            cudaStream_t st);
int fused_prepare_punch(int wave, int prec);

// The sweep with material tables, without / with tile step windows
// (fd23_fused_table.cu, fd23_fused_table_punch.cu); same arguments.
template <class S, class C>
int launch_step_fused_table(const Shot<S, C> &s, const Shot<S, C> *shots, int wave, const WorkItem *items,
                            const int *item_off, int nblocks, int par, int it, int rec_index, int *err_flag,
                            cudaStream_t st);
template <class S, class C>
int launch_step_fused_table_punch(const Shot<S, C> &s, const Shot<S, C> *shots, int wave, const WorkItem *items,
                                  const int *item_off, int nblocks, int par, int it, int rec_index, int *err_flag,
                                  cudaStream_t st);
int fused_prepare_table(int wave, int prec);
int fused_prepare_table_punch(int wave, int prec);

// Two-step fused sweep (fd23_fused2.cu; P-SV, FP32 wavefields): one launch
// advances every cell two full time steps, it and it+1, reading buffer set
// `par` and writing `1-par`; the memory variables of step it+1 go to
// s.psim.  `rec_index` >= 0 gathers the receivers of the previous step from
// buffer set `par` on the way (as the one-step sweep does); `rec_mid` >= 0
// records step it (the step in between) into that record row.  `width`:
// strip width of the CTA's first stress update, 256 (one CTA per SM) or 128
// (two); the output strips are fused2_tile_x(width) columns wide.
// half_material: the material is read from FP16 copies (s.maps2 views them).
template <class M>
int launch_step_fused2(const Shot<float, float> &s, int width, const WorkItem *items, const int *item_off,
                       int nblocks, int par, int it, int rec_index, int rec_mid, int *err_flag, cudaStream_t st);
int fused2_prepare(bool half_material, int width);  // once per device before the first launch
int fused2_tile_x(int width);                       // output columns per strip
int fused2_per_sm(int width);                       // CTAs per SM
// copy shapes of the two-step sweep (for its tensor maps)
struct Fused2Boxes {
    int uww, pww, mww;
};
Fused2Boxes fused2_boxes(bool half_material, int width);

// one thread waits on an mbarrier nothing completes, with the sweep's bounded
// wait: sets *err_flag when the wait gives up (about 2 s)
int launch_wait_probe(int *err_flag, cudaStream_t st);

// FP64 sum of squares over the `elems` stored elements of each of the first
// `nfields` wavefields of buffer set `par` (the zero padding included); the
// sum goes to dev_out[0], a NaN/Inf flag to dev_out[1].
template <class S, class C>
int launch_norm2(const Shot<S, C> &s, int par, int nfields, long long elems, double *dev_out,
                 cudaStream_t st);

}  // namespace fd23
