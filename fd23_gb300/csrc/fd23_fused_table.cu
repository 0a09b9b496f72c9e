// Fused sweep with material tables (mktable), without tile step windows: entry points and
// instantiations of the kernel template of fd23_fused.cuh with TABLE = true,
// PUNCH = false, in a translation unit of their own so that the variants
// compile in parallel.
#include "fd23_fused.cuh"

namespace fd23 {

template <class S, class C>
int launch_step_fused_table(const Shot<S, C> &s, const Shot<S, C> *shots, int wave, const WorkItem *items, const int *item_off,
       int nblocks, int par, int it, int rec_index, int *err_flag, cudaStream_t st)
{
    if (shots) {
        if (wave == FD23_PSV)
            return launch_fused_impl<S, C, FD23_PSV, true, false, true>(s, shots, items, item_off, nblocks, par, it,
                                                                   rec_index, err_flag, st);
        return launch_fused_impl<S, C, FD23_SH, true, false, true>(s, shots, items, item_off, nblocks, par, it,
                                                              rec_index, err_flag, st);
    }
    if (wave == FD23_PSV)
        return launch_fused_impl<S, C, FD23_PSV, false, false, true>(s, nullptr, items, item_off, nblocks, par, it,
                                                                rec_index, err_flag, st);
    return launch_fused_impl<S, C, FD23_SH, false, false, true>(s, nullptr, items, item_off, nblocks, par, it,
                                                           rec_index, err_flag, st);
}

int fused_prepare_table(int wave, int prec)
{
    if (wave == FD23_PSV) {
        switch (prec) {
            case FD23_F64: return prepare_one<double, double, FD23_PSV, false, true>();
            case FD23_BF16: return prepare_one<__nv_bfloat16, float, FD23_PSV, false, true>();
            case FD23_F16: return prepare_one<__half, float, FD23_PSV, false, true>();
            default: return prepare_one<float, float, FD23_PSV, false, true>();
        }
    }
    switch (prec) {
        case FD23_F64: return prepare_one<double, double, FD23_SH, false, true>();
        case FD23_BF16: return prepare_one<__nv_bfloat16, float, FD23_SH, false, true>();
        case FD23_F16: return prepare_one<__half, float, FD23_SH, false, true>();
        default: return prepare_one<float, float, FD23_SH, false, true>();
    }
}

#define FD23_INST(S, C)                                                                                          \
    template int launch_step_fused_table<S, C>(const Shot<S, C> &, const Shot<S, C> *, int, const WorkItem *, const int *, int, int, \
                          int, int, int *, cudaStream_t);
FD23_INST(float, float)
FD23_INST(double, double)
FD23_INST(__nv_bfloat16, float)
FD23_INST(__half, float)
#undef FD23_INST

}  // namespace fd23
