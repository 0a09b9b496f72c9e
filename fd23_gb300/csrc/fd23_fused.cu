// Plain fused sweep: entry points and the instantiations without tile step
// windows (the kernel template is in fd23_fused.cuh).
#include <type_traits>

#include "fd23_fused.cuh"

namespace fd23 {

namespace {

// Failure-path probe: one thread waits, with the sweep's bounded wait, on an
// mbarrier that nothing completes.  The wait gives up after its limit (about
// 2 s), sets the error flag and the kernel returns.
__global__ void wait_probe(int *err_flag)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    mbar_wait_bounded(&bar, 0u, err_flag);
}

}  // namespace

int launch_wait_probe(int *err_flag, cudaStream_t st)
{
    wait_probe<<<1, 32, 0, st>>>(err_flag);
    return cudaPeekAtLastError() == cudaSuccess ? FD23_OK : FD23_ERR_CUDA;
}

template <class S, class C, int WAVE>
FusedBoxes boxes_of()
{
    using K = Cfg<S, C, WAVE>;
    return FusedBoxes{K::UWW, K::PWW, K::NV, K::NT, K::NMS, K::NMV};
}

FusedBoxes fused_boxes(int wave, int prec)
{
    if (wave == FD23_PSV) {
        switch (prec) {
            case FD23_F64: return boxes_of<double, double, FD23_PSV>();
            case FD23_BF16: return boxes_of<__nv_bfloat16, float, FD23_PSV>();
            case FD23_F16: return boxes_of<__half, float, FD23_PSV>();
            default: return boxes_of<float, float, FD23_PSV>();
        }
    }
    switch (prec) {
        case FD23_F64: return boxes_of<double, double, FD23_SH>();
        case FD23_BF16: return boxes_of<__nv_bfloat16, float, FD23_SH>();
        case FD23_F16: return boxes_of<__half, float, FD23_SH>();
        default: return boxes_of<float, float, FD23_SH>();
    }
}

FusedGeom fused_geom(int wave, int prec)
{
    (void)wave;
    (void)prec;
    return FusedGeom{120, 4};  // 128 stress columns, 120 output columns, 4-row blocks
}

template <class S, class C>
int launch_step_fused(const Shot<S, C> &s, int wave, const WorkItem *items, const int *item_off,
                      int nblocks, int par, int it, int rec_index, int *err_flag, cudaStream_t st, int fast)
{
    if (s.midx)
        return s.punch.win ? launch_step_fused_table_punch<S, C>(s, nullptr, wave, items, item_off, nblocks, par, it,
                                                                 rec_index, err_flag, st)
                           : launch_step_fused_table<S, C>(s, nullptr, wave, items, item_off, nblocks, par, it,
                                                           rec_index, err_flag, st);
    if (s.punch.win)
        return launch_step_fused_punch<S, C>(s, nullptr, wave, items, item_off, nblocks, par, it, rec_index,
                                             err_flag, st);
    if constexpr (std::is_same<S, float>::value) {
        if (fast)
            return wave == FD23_PSV
                       ? launch_fused_impl<S, C, FD23_PSV, false, false, false, true>(s, nullptr, items, item_off,
                                                                                    nblocks, par, it, rec_index,
                                                                                    err_flag, st)
                       : launch_fused_impl<S, C, FD23_SH, false, false, false, true>(s, nullptr, items, item_off,
                                                                                   nblocks, par, it, rec_index,
                                                                                   err_flag, st);
    }
    if (wave == FD23_PSV)
        return launch_fused_impl<S, C, FD23_PSV, false, false>(s, nullptr, items, item_off, nblocks, par, it,
                                                               rec_index, err_flag, st);
    return launch_fused_impl<S, C, FD23_SH, false, false>(s, nullptr, items, item_off, nblocks, par, it,
                                                          rec_index, err_flag, st);
}

template <class S, class C>
int launch_step_fused_batch(const Shot<S, C> *shots, int wave, const WorkItem *items, const int *item_off,
                            int nblocks, int par, int it, int rec_index, int *err_flag, bool punch,
                            bool table, cudaStream_t st)
{
    const Shot<S, C> none{};
    if (table)
        return punch ? launch_step_fused_table_punch<S, C>(none, shots, wave, items, item_off, nblocks, par, it,
                                                           rec_index, err_flag, st)
                     : launch_step_fused_table<S, C>(none, shots, wave, items, item_off, nblocks, par, it,
                                                     rec_index, err_flag, st);
    if (punch)
        return launch_step_fused_punch<S, C>(none, shots, wave, items, item_off, nblocks, par, it, rec_index,
                                             err_flag, st);
    if (wave == FD23_PSV)
        return launch_fused_impl<S, C, FD23_PSV, true, false>(none, shots, items, item_off, nblocks, par, it,
                                                              rec_index, err_flag, st);
    return launch_fused_impl<S, C, FD23_SH, true, false>(none, shots, items, item_off, nblocks, par, it,
                                                         rec_index, err_flag, st);
}

int fused_prepare(int wave, int prec)
{
    // opt in to the large dynamic shared memory on the current device
    int rc;
    if (wave == FD23_PSV) {
        switch (prec) {
            case FD23_F64: rc = prepare_one<double, double, FD23_PSV, false>(); break;
            case FD23_BF16: rc = prepare_one<__nv_bfloat16, float, FD23_PSV, false>(); break;
            case FD23_F16: rc = prepare_one<__half, float, FD23_PSV, false>(); break;
            default: rc = prepare_one<float, float, FD23_PSV, false>();
        }
    } else {
        switch (prec) {
            case FD23_F64: rc = prepare_one<double, double, FD23_SH, false>(); break;
            case FD23_BF16: rc = prepare_one<__nv_bfloat16, float, FD23_SH, false>(); break;
            case FD23_F16: rc = prepare_one<__half, float, FD23_SH, false>(); break;
            default: rc = prepare_one<float, float, FD23_SH, false>();
        }
    }
    if (!rc && prec == FD23_F32) rc = wave == FD23_PSV ? prepare_fast<FD23_PSV>() : prepare_fast<FD23_SH>();
    if (!rc) rc = fused_prepare_punch(wave, prec);
    if (!rc) rc = fused_prepare_table(wave, prec);
    if (!rc) rc = fused_prepare_table_punch(wave, prec);
    return rc;
}

template <class S, class C, int WAVE>
int occupancy_one(bool batch)
{
    using K = Cfg<S, C, WAVE>;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &n, batch ? fused_step<S, C, WAVE, true, false, false> : fused_step<S, C, WAVE, false, false, false>,
            K::NTH, K::SMEM) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return n > 0 ? n : 1;
}

int fused_occupancy(int wave, int prec, bool batch)
{
    if (wave == FD23_PSV) {
        switch (prec) {
            case FD23_F64: return occupancy_one<double, double, FD23_PSV>(batch);
            case FD23_BF16: return occupancy_one<__nv_bfloat16, float, FD23_PSV>(batch);
            case FD23_F16: return occupancy_one<__half, float, FD23_PSV>(batch);
            default: return occupancy_one<float, float, FD23_PSV>(batch);
        }
    }
    switch (prec) {
        case FD23_F64: return occupancy_one<double, double, FD23_SH>(batch);
        case FD23_BF16: return occupancy_one<__nv_bfloat16, float, FD23_SH>(batch);
        case FD23_F16: return occupancy_one<__half, float, FD23_SH>(batch);
        default: return occupancy_one<float, float, FD23_SH>(batch);
    }
}

size_t fused_smem_bytes(int wave, int prec)
{
    if (wave == FD23_PSV) {
        switch (prec) {
            case FD23_F64: return Cfg<double, double, FD23_PSV>::SMEM;
            case FD23_BF16: return Cfg<__nv_bfloat16, float, FD23_PSV>::SMEM;
            case FD23_F16: return Cfg<__half, float, FD23_PSV>::SMEM;
            default: return Cfg<float, float, FD23_PSV>::SMEM;
        }
    }
    switch (prec) {
        case FD23_F64: return Cfg<double, double, FD23_SH>::SMEM;
        case FD23_BF16: return Cfg<__nv_bfloat16, float, FD23_SH>::SMEM;
        case FD23_F16: return Cfg<__half, float, FD23_SH>::SMEM;
        default: return Cfg<float, float, FD23_SH>::SMEM;
    }
}

#define FD23_INST(S, C)                                                                                  \
    template int launch_step_fused<S, C>(const Shot<S, C> &, int, const WorkItem *, const int *,       \
                                         int, int, int, int, int *, cudaStream_t, int);                \
    template int launch_step_fused_batch<S, C>(const Shot<S, C> *, int, const WorkItem *, const int *, \
                                               int, int, int, int, int *, bool, bool, cudaStream_t);
FD23_INST(float, float)
FD23_INST(double, double)
FD23_INST(__nv_bfloat16, float)
FD23_INST(__half, float)
#undef FD23_INST

}  // namespace fd23
