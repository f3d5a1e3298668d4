// Dot product that allocates nothing: its scratch is a file-scope device array.
//
// Who needs it: a caller that may not allocate device memory at the point it needs a reduction:
// code that runs while another component owns the allocator (a memory pool that must not grow, a
// budget fixed at start-up), or a host integration that may not create a context object
// (hgb_ctx_create allocates its scratch with cudaMalloc).  hgb_dot_f64_noalloc takes only the
// inputs, a device result pointer and a stream, and calls no cudaMalloc, cudaFree or allocating
// library routine.  It does call the CUDA runtime (a device query, a symbol lookup and a kernel
// launch), so it must not be called from a stream callback or a host function node, where CUDA
// API calls are not allowed.
//
// The scratch (one partial sum per block of kNoAllocSpan entries plus an arrival counter) lives
// in g_noalloc_scratch below, which every GPU that loads libhgb holds until the process exits.
// Device memory of a static __device__ array starts at zero when the module loads, and the last
// block of every launch sets the counter back to zero, so no call clears it.  Host code cannot use
// the array's name as a device address (in host code it names a host-side stand-in), so the first
// call on each device, with that device current, looks the address up with cudaGetSymbolAddress
// and passes it to the kernel; that first call should come before any stream capture.  The address
// is kept per device and per CUDA context, so a new context on the device (after
// cudaDeviceReset, or a driver-API context made current) is looked up again.  All calls share the
// array: two calls whose kernels overlap on the GPU (different streams, or concurrent host
// threads) race on it and must be ordered by the caller.
#include "hgb_internal.cuh"

#include <cuda.h>

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
    void *context = nullptr;   // CUDA context the address was looked up in
    double *scratch = nullptr;
};
static NoAllocDevice g_dev[64];
static std::mutex g_mu;

// The current CUDA context, through the driver entry point the runtime exposes (libhgb does not
// link the driver library); null when the lookup is unavailable.
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
static void *current_context() {
    static CtxGetCurrentFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        cudaGetLastError();
        return (CtxGetCurrentFn)p;
    }();
    CUcontext ctx = nullptr;
    if (fn && fn(&ctx) == CUDA_SUCCESS) return (void *)ctx;
    return nullptr;
}

// Set-up, once per device and context, with that device current: the device address of the array.
static int noalloc_setup(int dev, double **scratch) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (dev < 0 || dev >= 64) return fail(HGB_ERR_ARG, "dot_f64_noalloc: device %d", dev);
    NoAllocDevice &d = g_dev[dev];
    void *ctx = current_context();
    if (!d.scratch || !ctx || ctx != d.context) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        d.scratch = (double *)p;
        d.context = ctx;
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
