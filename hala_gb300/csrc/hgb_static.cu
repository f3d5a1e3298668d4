// Dot product that allocates nothing: its scratch is a file-scope device array.
//
// Who needs it: a caller that may not allocate device memory at the point it needs a reduction:
// code that runs while another component owns the allocator (a pool that must not grow), code
// inside a stream callback or a host function node where cudaMalloc is not allowed, or a host
// integration that forbids creating a context object (hgb_ctx_create allocates its scratch with
// cudaMalloc).  hgb_dot_f64_noalloc takes only the inputs, a device result pointer and a stream.
//
// The scratch (one partial sum per block of kSpan entries plus an arrival counter) lives in
// g_noalloc_scratch below, which every GPU that loads libhgb holds until the process exits.
// Host code cannot use the array's name as a device address (in host code it names a host-side
// stand-in), so the first call on each device looks the address up with cudaGetSymbolAddress,
// with that device current, and passes it to the kernel.  That first call also clears the
// counter; make it before any stream capture.  All calls share the array: two calls whose
// kernels overlap on the GPU (different streams, or concurrent host threads) race on it and
// must be ordered by the caller.
#include "hgb_internal.cuh"

#include <mutex>

namespace hgb {

constexpr int kNoAllocSpan = 2048;          // entries reduced by one block
constexpr int kNoAllocMaxParts = 16384;     // partial sums the scratch holds
constexpr long kNoAllocMaxN = (long)kNoAllocSpan * kNoAllocMaxParts;   // 33,554,432 entries

// [0, kNoAllocMaxParts): partial sums; [kNoAllocMaxParts]: arrival counter (as unsigned)
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxParts + 2];

__global__ void dot_noalloc_kernel(long n, const double *__restrict__ x, const double *__restrict__ y,
                                   double *scratch, double *out) {
    double acc[1] = {0.0};
    const long base = (long)blockIdx.x * kNoAllocSpan;
    const long end = min(base + (long)kNoAllocSpan, n);
    for (long i = base + threadIdx.x; i < end; i += blockDim.x) acc[0] += x[i] * y[i];
    unsigned *counter = reinterpret_cast<unsigned *>(scratch + kNoAllocMaxParts);
    grid_sum<1>(acc, scratch, counter, [&](double (&s)[1]) { *out = s[0]; });
}

struct NoAllocDevice {
    bool ready = false;
    double *scratch = nullptr;
};
static NoAllocDevice g_dev[64];
static std::mutex g_mu;

// Once per device, with that device current: the device address of the array, counter cleared.
static int noalloc_setup(int dev, double **scratch) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (dev < 0 || dev >= 64) return fail(HGB_ERR_ARG, "dot_f64_noalloc: device %d", dev);
    NoAllocDevice &d = g_dev[dev];
    if (!d.ready) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        e = cudaMemset((double *)p + kNoAllocMaxParts, 0, 2 * sizeof(double));
        if (e != cudaSuccess) return cuda_fail(e, "dot_f64_noalloc setup");
        d.scratch = (double *)p;
        d.ready = true;
    }
    *scratch = d.scratch;
    return HGB_OK;
}

}  // namespace hgb

using namespace hgb;

extern "C" int hgb_dot_f64_noalloc(int n, const double *x, const double *y, double *result_device, void *stream) {
    if (n < 0 || !result_device || (n > 0 && (!x || !y))) return fail(HGB_ERR_ARG, "dot_f64_noalloc: bad arguments");
    if ((long)n > kNoAllocMaxN)
        return fail(HGB_ERR_ARG, "dot_f64_noalloc: n = %d exceeds the static scratch limit of %ld entries", n,
                    kNoAllocMaxN);
    int dev = 0;
    HGB_CUDA(cudaGetDevice(&dev));
    double *scratch = nullptr;
    HGB_TRY(noalloc_setup(dev, &scratch));
    const int blocks = n > 0 ? (int)((n + kNoAllocSpan - 1) / kNoAllocSpan) : 1;
    dot_noalloc_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(n, x, y, scratch, result_device);
    return launch_check("dot_noalloc_kernel");
}
