// Allocation-free variant of the FP64 energy watchdog (fd23_field_norm2).
//
// Some callers cannot allocate device memory: programs whose device memory
// belongs to another allocator (a framework's caching allocator, a memory
// pool sized at start-up, an embedding host that forbids cudaMalloc outside
// its own arena).  For them this entry point takes the arrays to reduce as
// caller-owned device pointers, writes its results to caller-owned host
// memory, and keeps its partial sums in a fixed file-scope device array
// instead of allocating: it calls no cudaMalloc, cudaFree or allocating
// library routine.
//
// The call waits for its stream to finish (it reads the sum back to the
// host), so it cannot run on a stream that is being captured into a graph:
// on a capturing stream it returns FD23_ERR_UNSUPPORTED at once, without
// touching the stream, and the capture stays valid.
//
// Limits and sharing:
//   * at most FD23_NOALLOC_MAX_FIELDS (8) arrays per call; more is rejected
//     with FD23_ERR_ARG;
//   * every array must be device memory of the current device (checked with
//     cudaPointerGetAttributes, which allocates nothing), and the stream must
//     belong to that device;
//   * the scratch (FD23_NOALLOC_BLOCKS partial sums and flags, 16 KiB) is held
//     by every GPU that loads the library until the process exits;
//   * every call shares that one scratch array and leaves its contents
//     behind; each call overwrites every slot it reads, so nothing has to
//     start at zero, but calls that overlap on the GPU (different streams or
//     host threads at the same time) race on it and must be serialized by the
//     caller;
//   * the first call on a device resolves the scratch's device address for
//     that device (cudaGetSymbolAddress).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/fd23.h"

namespace {

constexpr int kMaxFields = 8;     // FD23_NOALLOC_MAX_FIELDS
constexpr int kBlocks = 1024;     // FD23_NOALLOC_BLOCKS (partials per call)
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

// [0, kBlocks): per-block FP64 sums; [kBlocks, 2*kBlocks): per-block NaN/Inf
// flags; [2*kBlocks, 2*kBlocks+2): the final sum and flag
static __device__ __align__(256) double g_noalloc_scratch[2 * kBlocks + 2];

struct FieldPtrs {
    const void *p[kMaxFields];
};

template <class S>
__device__ __forceinline__ double as_double(S v) { return (double)v; }
template <>
__device__ __forceinline__ double as_double<__nv_bfloat16>(__nv_bfloat16 v) { return (double)__bfloat162float(v); }
template <>
__device__ __forceinline__ double as_double<__half>(__half v) { return (double)__half2float(v); }

// every block writes its own partial slot (no accumulation, no clearing)
template <class S>
__global__ void __launch_bounds__(kThreads) partial_sums(FieldPtrs f, int nfields, long long n,
                                                         double *scratch)
{
    __shared__ double ssum[kThreads / 32];
    __shared__ int sbad[kThreads / 32];
    double acc = 0.0;
    int bad = 0;
    for (int k = 0; k < nfields; ++k) {
        const S *a = static_cast<const S *>(f.p[k]);
        for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n;
             i += (long long)gridDim.x * kThreads) {
            const double v = as_double<S>(a[i]);
            if (!isfinite(v)) bad = 1;
            else acc += v * v;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        acc += __shfl_down_sync(0xffffffffu, acc, o);
        bad |= __shfl_down_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) {
        ssum[threadIdx.x >> 5] = acc;
        sbad[threadIdx.x >> 5] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        int b = 0;
        for (int w = 0; w < kThreads / 32; ++w) {
            t += ssum[w];
            b |= sbad[w];
        }
        scratch[blockIdx.x] = t;
        scratch[kBlocks + blockIdx.x] = b ? 1.0 : 0.0;
    }
}

// one block sums the partials in a fixed order (deterministic result)
__global__ void __launch_bounds__(kBlocks) final_sum(double *scratch)
{
    __shared__ double s[kBlocks];
    __shared__ double fb[kBlocks];
    s[threadIdx.x] = scratch[threadIdx.x];
    fb[threadIdx.x] = scratch[kBlocks + threadIdx.x];
    __syncthreads();
    for (int w = kBlocks / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            s[threadIdx.x] += s[threadIdx.x + w];
            fb[threadIdx.x] = fmax(fb[threadIdx.x], fb[threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        scratch[2 * kBlocks] = s[0];
        scratch[2 * kBlocks + 1] = fb[0];
    }
}

std::mutex g_mu;
double *g_scratch_ptr[kMaxDevices] = {};

// set-up, once per device, with that device current
int scratch_for_current_device(double **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return FD23_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return FD23_ERR_CUDA;
        }
        g_scratch_ptr[dev] = static_cast<double *>(p);
    }
    *out = g_scratch_ptr[dev];
    return FD23_OK;
}

// FD23_OK when every pointer is device (or managed) memory of device `dev`
int check_pointers(const FieldPtrs &fp, int nfields, int dev)
{
    for (int k = 0; k < nfields; ++k) {
        if (!fp.p[k]) continue;  // n == 0: nothing is read
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, fp.p[k]) != cudaSuccess) {
            cudaGetLastError();
            return FD23_ERR_ARG;
        }
        if ((a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) || a.device != dev)
            return FD23_ERR_ARG;
    }
    return FD23_OK;
}

}  // namespace

extern "C" int fd23_sum_squares_noalloc(int prec, const void *const *fields, int nfields, size_t n,
                                        void *stream, double *sum, int *nonfinite)
{
    if (!fields || !sum || !nonfinite || nfields <= 0 || prec < FD23_F32 || prec > FD23_F16)
        return FD23_ERR_ARG;
    if (nfields > kMaxFields) return FD23_ERR_ARG;  // beyond the fixed scratch
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the call ends with a stream synchronize, which a capturing stream
    // refuses (and the refusal would invalidate the capture): decline first
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
        cudaGetLastError();
        return FD23_ERR_UNSUPPORTED;
    }
    if (cap != cudaStreamCaptureStatusNone) return FD23_ERR_UNSUPPORTED;
    FieldPtrs fp{};
    for (int k = 0; k < nfields; ++k) {
        if (!fields[k] && n > 0) return FD23_ERR_ARG;
        fp.p[k] = n > 0 ? fields[k] : nullptr;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return FD23_ERR_CUDA;
    }
    int rc = check_pointers(fp, nfields, dev);
    if (rc) return rc;
    if (st) {
        int sdev = -1;
        if (cudaStreamGetDevice(st, &sdev) != cudaSuccess) {
            cudaGetLastError();
            return FD23_ERR_ARG;
        }
        if (sdev != dev) return FD23_ERR_ARG;
    }
    double *scratch = nullptr;
    if ((rc = scratch_for_current_device(&scratch))) return rc;
    const long long nn = (long long)n;
    switch (prec) {
        case FD23_F64: partial_sums<double><<<kBlocks, kThreads, 0, st>>>(fp, nfields, nn, scratch); break;
        case FD23_BF16: partial_sums<__nv_bfloat16><<<kBlocks, kThreads, 0, st>>>(fp, nfields, nn, scratch); break;
        case FD23_F16: partial_sums<__half><<<kBlocks, kThreads, 0, st>>>(fp, nfields, nn, scratch); break;
        default: partial_sums<float><<<kBlocks, kThreads, 0, st>>>(fp, nfields, nn, scratch);
    }
    // a rejected launch must not let the previous call's result through
    if (cudaGetLastError() != cudaSuccess) return FD23_ERR_CUDA;
    final_sum<<<1, kBlocks, 0, st>>>(scratch);
    if (cudaGetLastError() != cudaSuccess) return FD23_ERR_CUDA;
    double h[2];
    if (cudaMemcpyAsync(h, scratch + 2 * kBlocks, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return FD23_ERR_CUDA;
    }
    *sum = h[0];
    *nonfinite = h[1] != 0.0;
    return FD23_OK;
}
