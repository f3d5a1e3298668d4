// Internal declarations shared by the libhgb translation units (not installed).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include "hgb.h"

namespace hgb {

// ------------------------------------------------------------------------- errors ---------
void set_error(int code, const char *fmt, ...);
int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

#define HGB_CUDA(...)                                                    \
    do {                                                                 \
        cudaError_t e_ = (__VA_ARGS__);                                  \
        if (e_ != cudaSuccess) return ::hgb::cuda_fail(e_, #__VA_ARGS__);\
    } while (0)

#define HGB_TRY(...)                                                     \
    do {                                                                 \
        int s_ = (__VA_ARGS__);                                          \
        if (s_ != HGB_OK) return s_;                                     \
    } while (0)

// Device error word bits (written by kernels, read by the host after a launch sequence).
enum : int { DEV_ERR_TIMEOUT = 1, DEV_ERR_CSR = 2, DEV_ERR_ZERO_PIVOT = 4 };

int dev_error_to_status(int word);

// Maximum number of CTAs a reduction kernel launches; bounds the partial-sum scratch.
constexpr int kMaxReduceBlocks = 2048;
constexpr int kReduceSlots = 4;   // values reduced together in one pass
// the context's partials (1 MB, a size that measured faster than one just above it: the mixed
// 128^3 solve took 5 ms longer with 1 MB + 16 KB): the grid reductions' slots below
// kSpmvPartsOffset (a pass of up to 64 values runs on at most kSpmvPartsOffset / 64 CTAs), then
// kMaxReduceBlocks per-CTA <x, y> parts of a fused SpMV whose consumer sums them
constexpr long kSpmvPartsOffset = (long)kMaxReduceBlocks * 48;
constexpr long kPartialsDoubles = (long)kMaxReduceBlocks * 64;

// Scalars kept on the device by the fused solvers (one set per context).
struct SolverScalars {
    double zr, pap, rr, nzr;     // CG recurrences
    double tol2;                 // stopping threshold on ||r||^2
    double r0;                   // first residual norm of the current inner solve
    double rel;                  // inner relative tolerance (IR); 0 = absolute test only
    int it, done, max_iter, pad;
    // reliable-update PCG: largest ||r||^2 since the last update, the update threshold (delta^2),
    // 0 while an update is due in the current iteration, updates so far
    double rmax2, delta2;
    int ru_skip, updates;
    double last2;                // ||r||^2 after the previous update
    int restart, pad2;           // 1: the next direction update restarts (beta = 0)
};

}  // namespace hgb

struct hgb_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 0;
    // scratch: reduction partials, counter, results, device error word, solver scalars
    double *partials = nullptr;            // kPartialsDoubles: grid reductions, then the SpMV's per-CTA parts
    unsigned *counter = nullptr;           // reduction arrival counter (self-resetting)
    double *result = nullptr;              // 8 result slots
    int *err = nullptr;                    // device error word
    hgb::SolverScalars *scal = nullptr;    // fused-solver scalars
    double *host_result = nullptr;         // pinned staging for host-returned scalars (64 doubles)
    unsigned error_epoch = 0;              // bumped whenever a device-side failure is collected
    void *arena = nullptr;                 // grow-only staging for host-buffer (mixed) solves
    size_t arena_bytes = 0;
    cudaStream_t worker = nullptr;         // capturable stream used when the caller's is the NULL stream
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    cudaMemPool_t pool = nullptr;          // solver workspaces: stream-ordered, memory kept between solves
    int spmv_mode = HGB_SPMV_FUSED;        // arithmetic of the 'N' products (hgb_ctx_set_spmv_mode)
    cudaStream_t copy = nullptr;           // host-to-device transfers of the host-buffer entries
};

namespace hgb {

// Solver workspaces come from the context's memory pool in stream order: after the first solve of
// a size the pool holds the memory, so a solve allocates without a device-wide cudaMalloc and frees
// without the synchronising cudaFree.
template <typename T>
inline cudaError_t ws_alloc(hgb_ctx *c, T **p, size_t count) {
    return cudaMallocFromPoolAsync((void **)p, sizeof(T) * (count ? count : 1), c->pool, c->stream);
}
inline void ws_free(hgb_ctx *c, void *p) {
    if (p) cudaFreeAsync(p, c->stream);
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

// read and clear the device error word (synchronises the stream)
int collect_dev_error(hgb_ctx *ctx);

// host -> device in chunks (one cudaMemcpyAsync per chunk) on stream s; a pageable source is staged
// by the driver chunk by chunk, so the first chunks move while later ones are still being read
int h2d_chunked(hgb_ctx *ctx, cudaStream_t s, void *dst, const void *src, size_t bytes);

// Graph capture is not possible on the legacy NULL stream.  For the duration of a fused solve the
// context's work moves to its private non-blocking stream, ordered after the caller's prior work
// and before the caller's later work by events.
struct CaptureStream {
    hgb_ctx *c;
    cudaStream_t saved;
    bool swapped = false;
    explicit CaptureStream(hgb_ctx *ctx) : c(ctx), saved(ctx->stream) {
        if (saved == nullptr || saved == cudaStreamLegacy) {
            cudaEventRecord(c->ev_in, saved);
            cudaStreamWaitEvent(c->worker, c->ev_in, 0);
            c->stream = c->worker;
            swapped = true;
        }
    }
    ~CaptureStream() {
        if (swapped) {
            cudaEventRecord(c->ev_out, c->worker);
            cudaStreamWaitEvent(saved, c->ev_out, 0);
            c->stream = saved;
        }
    }
};

inline int reduce_grid(const hgb_ctx *ctx, long n, int per_block) {
    long b = (n + per_block - 1) / per_block;
    long cap = (long)ctx->num_sms * 4;
    if (cap > kMaxReduceBlocks) cap = kMaxReduceBlocks;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

inline int launch_check(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, what);
    return HGB_OK;
}

// ------------------------------------------------------- device-side primitives ---------

// Values not yet produced by a sync-free solve hold a signalling-NaN pattern that IEEE
// arithmetic never generates; a computed value equal to it is replaced by the canonical NaN.
template <typename T> struct Pending;
template <> struct Pending<double> {
    static constexpr unsigned long long bits = 0x7FF4DEADBEEF0001ull;
    __device__ static bool is(double v) { return (unsigned long long)__double_as_longlong(v) == bits; }
    __device__ static double value() { return __longlong_as_double((long long)bits); }
    __device__ static double canon(double v) {
        return is(v) ? __longlong_as_double(0x7FF8000000000000ll) : v;
    }
};
template <> struct Pending<float> {
    static constexpr unsigned bits = 0x7FA5A5A5u;
    __device__ static bool is(float v) { return (unsigned)__float_as_uint(v) == bits; }
    __device__ static float value() { return __uint_as_float(bits); }
    __device__ static float canon(float v) { return is(v) ? __uint_as_float(0x7FC00000u) : v; }
};

__device__ __forceinline__ double ld_relaxed(const double *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return __longlong_as_double((long long)v);
}
__device__ __forceinline__ float ld_relaxed(const float *p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return __uint_as_float(v);
}
__device__ __forceinline__ int ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(double *p, double v) {
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(__double_as_longlong(v)) : "memory");
}
__device__ __forceinline__ void st_relaxed(float *p, float v) {
    asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(__float_as_uint(v)) : "memory");
}
__device__ __forceinline__ void st_release(int *p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Poll budget of the sync-free waits: about a second of polling on GB300 before giving up.
constexpr int kSpinLimit = 1 << 22;

// Wait until *p no longer holds the pending pattern; bounded.  On timeout the error word gets
// DEV_ERR_TIMEOUT and NaN is returned so that dependents terminate too.  A wait also gives up as
// soon as another wait has timed out (checked every 4096 polls), so a launch whose inputs can
// never arrive ends after one poll budget instead of one budget per waiting row.
template <typename T>
__device__ __forceinline__ T wait_value(const T *p, int *err, int limit = kSpinLimit) {
    T v = ld_relaxed(p);
    int spins = 0;
    while (Pending<T>::is(v)) {
        ++spins;
        if (spins > limit || ((spins & 4095) == 0 && (*(volatile int *)err & DEV_ERR_TIMEOUT))) {
            atomicOr(err, DEV_ERR_TIMEOUT);
            return Pending<T>::canon(Pending<T>::value());
        }
        v = ld_relaxed(p);
    }
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of NV doubles (blockDim.x multiple of 32, <= 1024).  Result valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
    __shared__ double sh[32][NV];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = warp_sum(v[k]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) sh[wid][k] = v[k];
    __syncthreads();
    int nw = blockDim.x >> 5;
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double t = lane < nw ? sh[lane][k] : 0.0;
            v[k] = warp_sum(t);
        }
    }
}

// Deterministic grid reduction: every CTA stores its partial sums; the last CTA to arrive adds
// them in CTA order and runs fin(sums) in thread 0.  Returns true in the finishing thread.
// The arrival counter resets itself, so back-to-back launches (and graph replays) need no memset.
template <int NV, typename Fin>
__device__ __forceinline__ void grid_sum(double (&v)[NV], double *partials, unsigned *counter,
                                         Fin fin) {
    block_sum<NV>(v);
    __shared__ bool last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) partials[blockIdx.x * NV + k] = v[k];
        __threadfence();
        unsigned t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) acc[k] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
#pragma unroll
        for (int k = 0; k < NV; k++) acc[k] += __ldcg(partials + b * NV + k);
    block_sum<NV>(acc);
    if (threadIdx.x == 0) {
        *counter = 0u;
        fin(acc);
    }
}

}  // namespace hgb
