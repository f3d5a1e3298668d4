// Library core: error reporting, the engine context, BLAS-1, tall-skinny gemv, diagonal index.
#include "hgb_internal.cuh"
#include "hgb_kernels.cuh"
#include "hgb_complex.cuh"

#include <algorithm>
#include <cstring>
#include <mutex>

namespace hgb {

static thread_local std::string g_last_error;

void set_error(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = std::string(hgb_status_string(code)) + ": " + buf;
}

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = std::string(hgb_status_string(code)) + ": " + buf;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    return fail(e == cudaErrorMemoryAllocation ? HGB_ERR_ALLOC : HGB_ERR_CUDA, "%s: %s", what,
                cudaGetErrorString(e));
}

int h2d_chunked(hgb_ctx *c, cudaStream_t s, void *dst, const void *src, size_t bytes) {
    (void)c;
    constexpr size_t kChunk = (size_t)16 << 20;
    for (size_t o = 0; o < bytes; o += kChunk) {
        const size_t b = std::min(kChunk, bytes - o);
        HGB_CUDA(cudaMemcpyAsync((char *)dst + o, (const char *)src + o, b, cudaMemcpyHostToDevice, s));
    }
    return HGB_OK;
}

int dev_error_to_status(int w) {
    if (w & DEV_ERR_TIMEOUT) return HGB_ERR_TIMEOUT;
    if (w & DEV_ERR_CSR) return HGB_ERR_CSR;
    if (w & DEV_ERR_ZERO_PIVOT) return HGB_ERR_ZERO_PIVOT;
    return HGB_OK;
}

int collect_dev_error(hgb_ctx *ctx) {
    int w = 0;
    HGB_CUDA(cudaMemcpyAsync(&w, ctx->err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    HGB_CUDA(cudaStreamSynchronize(ctx->stream));
    if (w) {
        ctx->error_epoch++;
        HGB_CUDA(cudaMemsetAsync(ctx->err, 0, sizeof(int), ctx->stream));
        int st = dev_error_to_status(w);
        return fail(st, "device-side check failed (error word 0x%x)", w);
    }
    return HGB_OK;
}

// ------------------------------------------------------------------ BLAS-1 kernels ------

template <typename T>
__global__ void dot_kernel(long n, const T *__restrict__ x, const T *__restrict__ y,
                           double *partials, unsigned *counter, T *out, int op) {
    // op 0: dot(x, y); op 1: sqrt(dot(x, x))
    double acc[1] = {0.0};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        acc[0] += (double)x[i] * (double)y[i];
    grid_sum<1>(acc, partials, counter, [&](double (&s)[1]) {
        *out = (T)(op == 1 ? sqrt(s[0]) : s[0]);
    });
}

template <typename T>
__global__ void axpy_kernel(long n, T alpha, const T *__restrict__ x, T *__restrict__ y) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        y[i] += alpha * x[i];
}

template <typename T>
__global__ void scal_kernel(long n, T alpha, T *__restrict__ x) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        x[i] *= alpha;
}

// Tall-skinny gemv for the Krylov basis: W is m x k column-major.
// 'T': y[j] = alpha * <W[:,j], x> + beta * y[j] for the KMAX columns j0.. j0+KMAX (one grid
// reduction, double accumulation); wider W takes one launch per group of 64 columns.
template <int KMAX, typename T>
__global__ void gemv_t_kernel(int m, int k, T alpha, const T *__restrict__ W, const T *__restrict__ x, T beta, T *y,
                              double *partials, unsigned *counter) {
    double acc[KMAX];
#pragma unroll
    for (int j = 0; j < KMAX; j++) acc[j] = 0.0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < m; i += (long)gridDim.x * blockDim.x) {
        const double xi = (double)x[i];
#pragma unroll
        for (int j = 0; j < KMAX; j++)
            if (j < k) acc[j] += (double)W[(long)j * m + i] * xi;
    }
    grid_sum<KMAX>(acc, partials, counter, [&](double (&s)[KMAX]) {
        for (int j = 0; j < k; j++) y[j] = (beta == T(0)) ? (T)(alpha * s[j]) : (T)(alpha * s[j] + beta * y[j]);
    });
}

// 'N': y[i] = alpha * sum_j W[i,j] * c[j] + beta * y[i]
template <typename T>
__global__ void gemv_n_kernel(int m, int k, T alpha, const T *__restrict__ W, const T *__restrict__ c, T beta,
                              T *__restrict__ y) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < m; i += (long)gridDim.x * blockDim.x) {
        T s = T(0);
        for (int j = 0; j < k; j++) s += W[(long)j * m + i] * c[j];
        y[i] = (beta == T(0)) ? alpha * s : alpha * s + beta * y[i];
    }
}

// C = diag(x) A (side 'L': row i scaled by x[i]) or A diag(x) (side 'R': column j by x[j]);
// A, C m x k column-major, packed
template <typename T>
__global__ void dgmm_kernel(long m, long k, int left, const T *__restrict__ A, const T *__restrict__ x, T *C) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < m * k; e += (long)gridDim.x * blockDim.x) {
        const long i = e % m, j = e / m;
        C[e] = A[e] * x[left ? i : j];
    }
}

// diag[i] = position of column i in row i (binary search; columns sorted)
__global__ void diag_index_kernel(int n, const int *__restrict__ pntr, const int *__restrict__ indx,
                                  int *__restrict__ diag, int *err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int lo = pntr[i], hi = pntr[i + 1] - 1, pos = -1;
        while (lo <= hi) {
            int mid = (lo + hi) >> 1;
            int c = indx[mid];
            if (c == i) { pos = mid; break; }
            if (c < i) lo = mid + 1; else hi = mid - 1;
        }
        if (pos < 0) atomicOr(err, DEV_ERR_CSR);
        diag[i] = pos;
    }
}

__global__ void wait_timeout_kernel(const double *never, int *err, int limit) {
    if (threadIdx.x == 0 && blockIdx.x == 0) (void)wait_value<double>(never, err, limit);
}

__global__ void fill_pending_f64(long n, double *p) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        p[i] = Pending<double>::value();
}

}  // namespace hgb

namespace hgb {
template <typename T>
static int dot_impl(hgb_ctx *c, int n, const T *x, const T *y, T *result, int on_device, int op) {
    if (!c || n < 0 || !result || (n > 0 && (!x || !y))) return fail(HGB_ERR_ARG, "dot/nrm2: bad arguments");
    DeviceGuard g(c->device);
    T *dst = on_device ? result : (T *)c->result;
    int grid = reduce_grid(c, n, 256 * 4);
    dot_kernel<T><<<grid, 256, 0, c->stream>>>(n, x, y, c->partials, c->counter, dst, op);
    HGB_TRY(launch_check("dot_kernel"));
    if (!on_device) {
        HGB_CUDA(cudaMemcpyAsync(c->host_result, c->result, sizeof(T), cudaMemcpyDeviceToHost, c->stream));
        HGB_CUDA(cudaStreamSynchronize(c->stream));
        memcpy(result, c->host_result, sizeof(T));
    }
    return HGB_OK;
}

template <typename T>
static int axpy_impl(hgb_ctx *c, int n, T a, const T *x, T *y) {
    if (!c || n < 0 || (n > 0 && (!x || !y))) return fail(HGB_ERR_ARG, "axpy: bad arguments");
    if (n == 0) return HGB_OK;
    DeviceGuard g(c->device);
    axpy_kernel<T><<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, a, x, y);
    return launch_check("axpy_kernel");
}

template <typename T>
static int scal_impl(hgb_ctx *c, int n, T a, T *x) {
    if (!c || n < 0 || (n > 0 && !x)) return fail(HGB_ERR_ARG, "scal: bad arguments");
    if (n == 0) return HGB_OK;
    DeviceGuard g(c->device);
    scal_kernel<T><<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, a, x);
    return launch_check("scal_kernel");
}
}  // namespace hgb

using namespace hgb;

// ==================================================================== C ABI ==============
extern "C" {

const char *hgb_status_string(int s) {
    switch (s) {
        case HGB_OK: return "HGB_OK";
        case HGB_ERR_ARG: return "HGB_ERR_ARG";
        case HGB_ERR_CSR: return "HGB_ERR_CSR";
        case HGB_ERR_ZERO_PIVOT: return "HGB_ERR_ZERO_PIVOT";
        case HGB_ERR_TIMEOUT: return "HGB_ERR_TIMEOUT";
        case HGB_ERR_NOT_CONVERGED: return "HGB_ERR_NOT_CONVERGED";
        case HGB_ERR_CUDA: return "HGB_ERR_CUDA";
        case HGB_ERR_ALLOC: return "HGB_ERR_ALLOC";
        case HGB_ERR_UNSUPPORTED: return "HGB_ERR_UNSUPPORTED";
        default: return "HGB_ERR_UNKNOWN";
    }
}

const char *hgb_last_error(void) { return g_last_error.c_str(); }

int hgb_version(void) { return 10000 * 1 + 100 * 1 + 0; }

int hgb_ctx_create(int device, hgb_ctx **out) {
    if (!out) return fail(HGB_ERR_ARG, "hgb_ctx_create: null output");
    *out = nullptr;
    int ndev = 0;
    HGB_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(HGB_ERR_ARG, "device %d out of range [0,%d)", device, ndev);
    DeviceGuard g(device);
    hgb_ctx *c = new hgb_ctx();
    c->device = device;
    cudaError_t e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaMalloc(&c->partials, sizeof(double) * kPartialsDoubles);
    if (e == cudaSuccess) e = cudaMalloc(&c->counter, sizeof(unsigned) * 8);
    if (e == cudaSuccess) e = cudaMalloc(&c->result, sizeof(double) * 8);
    if (e == cudaSuccess) e = cudaMalloc(&c->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&c->scal, sizeof(SolverScalars));
    if (e == cudaSuccess) e = cudaMallocHost(&c->host_result, sizeof(double) * 64);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->worker, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_out, cudaEventDisableTiming);
    if (e == cudaSuccess) {
        cudaMemPoolProps pp = {};
        pp.allocType = cudaMemAllocationTypePinned;
        pp.location.type = cudaMemLocationTypeDevice;
        pp.location.id = device;
        e = cudaMemPoolCreate(&c->pool, &pp);
    }
    if (e == cudaSuccess) {
        uint64_t keep = UINT64_MAX;   // never trim: the next solve of the same size reuses the memory
        e = cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e == cudaSuccess) e = cudaMemset(c->counter, 0, sizeof(unsigned) * 8);
    if (e == cudaSuccess) e = cudaMemset(c->err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(c->scal, 0, sizeof(SolverScalars));
    if (e != cudaSuccess) {
        hgb_ctx_destroy(c);
        return cuda_fail(e, "hgb_ctx_create");
    }
    *out = c;
    return HGB_OK;
}

int hgb_ctx_destroy(hgb_ctx *c) {
    if (!c) return HGB_OK;
    DeviceGuard g(c->device);
    cudaFree(c->partials);
    cudaFree(c->counter);
    cudaFree(c->result);
    cudaFree(c->err);
    cudaFree(c->scal);
    cudaFreeHost(c->host_result);
    cudaFree(c->arena);
    if (c->worker) cudaStreamDestroy(c->worker);
    if (c->copy) cudaStreamDestroy(c->copy);
    if (c->ev_in) cudaEventDestroy(c->ev_in);
    if (c->ev_out) cudaEventDestroy(c->ev_out);
    if (c->pool) cudaMemPoolDestroy(c->pool);   // released once the last stream-ordered free has run
    delete c;
    return HGB_OK;
}

int hgb_ctx_set_stream(hgb_ctx *c, void *stream) {
    if (!c) return fail(HGB_ERR_ARG, "null context");
    c->stream = (cudaStream_t)stream;
    return HGB_OK;
}

int hgb_ctx_set_spmv_mode(hgb_ctx *c, int mode) {
    if (!c) return fail(HGB_ERR_ARG, "set_spmv_mode: null context");
    if (mode != HGB_SPMV_FUSED && mode != HGB_SPMV_EXACT) return fail(HGB_ERR_ARG, "set_spmv_mode: mode %d", mode);
    c->spmv_mode = mode;
    return HGB_OK;
}

int hgb_ctx_get_spmv_mode(hgb_ctx *c, int *mode) {
    if (!c || !mode) return fail(HGB_ERR_ARG, "get_spmv_mode: bad arguments");
    *mode = c->spmv_mode;
    return HGB_OK;
}

int hgb_ctx_synchronize(hgb_ctx *c) {
    if (!c) return fail(HGB_ERR_ARG, "null context");
    DeviceGuard g(c->device);
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    return HGB_OK;
}

// ------------------------------------------------------------------ BLAS-1 --------------

int hgb_dot_f64(hgb_ctx *c, int n, const double *x, const double *y, double *r, int d) { return dot_impl(c, n, x, y, r, d, 0); }
int hgb_dot_f32(hgb_ctx *c, int n, const float *x, const float *y, float *r, int d) { return dot_impl(c, n, x, y, r, d, 0); }
int hgb_nrm2_f64(hgb_ctx *c, int n, const double *x, double *r, int d) { return dot_impl(c, n, x, x, r, d, 1); }
int hgb_nrm2_f32(hgb_ctx *c, int n, const float *x, float *r, int d) { return dot_impl(c, n, x, x, r, d, 1); }

int hgb_axpy_f64(hgb_ctx *c, int n, double a, const double *x, double *y) { return axpy_impl(c, n, a, x, y); }
int hgb_axpy_f32(hgb_ctx *c, int n, float a, const float *x, float *y) { return axpy_impl(c, n, a, x, y); }

int hgb_scal_f64(hgb_ctx *c, int n, double a, double *x) { return scal_impl(c, n, a, x); }
int hgb_scal_f32(hgb_ctx *c, int n, float a, float *x) { return scal_impl(c, n, a, x); }

int hgb_copy_f64(hgb_ctx *c, int n, const double *x, double *y) {
    if (!c || n < 0 || (n > 0 && (!x || !y))) return fail(HGB_ERR_ARG, "copy: bad arguments");
    DeviceGuard g(c->device);
    if (n) HGB_CUDA(cudaMemcpyAsync(y, x, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, c->stream));
    return HGB_OK;
}
int hgb_copy_f32(hgb_ctx *c, int n, const float *x, float *y) {
    if (!c || n < 0 || (n > 0 && (!x || !y))) return fail(HGB_ERR_ARG, "copy: bad arguments");
    DeviceGuard g(c->device);
    if (n) HGB_CUDA(cudaMemcpyAsync(y, x, sizeof(float) * (size_t)n, cudaMemcpyDeviceToDevice, c->stream));
    return HGB_OK;
}

int hgb_dotc_c128(hgb_ctx *c, int n, const void *x, const void *y, double *r, int d) {
    if (!c) return fail(HGB_ERR_ARG, "dotc: null context");
    DeviceGuard g(c->device);
    return zdot<double>(c, 0, n, x, y, r, d);
}
int hgb_dotc_c64(hgb_ctx *c, int n, const void *x, const void *y, float *r, int d) {
    if (!c) return fail(HGB_ERR_ARG, "dotc: null context");
    DeviceGuard g(c->device);
    return zdot<float>(c, 0, n, x, y, r, d);
}
int hgb_dotu_c128(hgb_ctx *c, int n, const void *x, const void *y, double *r, int d) {
    if (!c) return fail(HGB_ERR_ARG, "dotu: null context");
    DeviceGuard g(c->device);
    return zdot<double>(c, 1, n, x, y, r, d);
}
int hgb_dotu_c64(hgb_ctx *c, int n, const void *x, const void *y, float *r, int d) {
    if (!c) return fail(HGB_ERR_ARG, "dotu: null context");
    DeviceGuard g(c->device);
    return zdot<float>(c, 1, n, x, y, r, d);
}
int hgb_nrm2_c128(hgb_ctx *c, int n, const void *x, double *r, int d) {
    if (!c) return fail(HGB_ERR_ARG, "nrm2: null context");
    DeviceGuard g(c->device);
    return zdot<double>(c, 2, n, x, x, r, d);
}
int hgb_axpy_c128(hgb_ctx *c, int n, const double *a, const void *x, void *y) {
    if (!c) return fail(HGB_ERR_ARG, "axpy: null context");
    DeviceGuard g(c->device);
    return zaxpy<double>(c, n, a, x, y);
}
int hgb_scal_c128(hgb_ctx *c, int n, const double *a, void *x) {
    if (!c) return fail(HGB_ERR_ARG, "scal: null context");
    DeviceGuard g(c->device);
    return zscal<double>(c, n, a, x);
}
int hgb_nrm2_c64(hgb_ctx *c, int n, const void *x, float *r, int d) {
    if (!c) return fail(HGB_ERR_ARG, "nrm2: null context");
    DeviceGuard g(c->device);
    return zdot<float>(c, 2, n, x, x, r, d);
}
int hgb_axpy_c64(hgb_ctx *c, int n, const float *a, const void *x, void *y) {
    if (!c) return fail(HGB_ERR_ARG, "axpy: null context");
    DeviceGuard g(c->device);
    return zaxpy<float>(c, n, a, x, y);
}
int hgb_scal_c64(hgb_ctx *c, int n, const float *a, void *x) {
    if (!c) return fail(HGB_ERR_ARG, "scal: null context");
    DeviceGuard g(c->device);
    return zscal<float>(c, n, a, x);
}

int hgb_set_zero(hgb_ctx *c, size_t bytes, void *x) {
    if (!c || (bytes && !x)) return fail(HGB_ERR_ARG, "set_zero: bad arguments");
    DeviceGuard g(c->device);
    if (bytes) HGB_CUDA(cudaMemsetAsync(x, 0, bytes, c->stream));
    return HGB_OK;
}

}  // extern "C"

namespace hgb {
template <typename T>
static int gemv_impl(hgb_ctx *c, char trans, int m, int k, T alpha, const T *W, const T *x, T beta, T *y) {
    if (!c || m < 0 || k < 0) return fail(HGB_ERR_ARG, "gemv: m=%d k=%d", m, k);
    if (m == 0 || k == 0) return HGB_OK;
    DeviceGuard g(c->device);
    if (trans == 'N' || trans == 'n') {
        gemv_n_kernel<T><<<reduce_grid(c, m, 256 * 2), 256, 0, c->stream>>>(m, k, alpha, W, x, beta, y);
        return launch_check("gemv_n_kernel");
    }
    if (trans != 'T' && trans != 't' && trans != 'C' && trans != 'c') return fail(HGB_ERR_ARG, "gemv: trans '%c'", trans);
    const int grid = reduce_grid(c, m, 256 * 8);
    for (int j0 = 0; j0 < k; j0 += 64) {   // groups of up to 64 columns, one grid reduction each
        const int kk = std::min(64, k - j0);
        const T *Wj = W + (long)j0 * m;
        T *yj = y + j0;
        if (kk <= 8) gemv_t_kernel<8, T><<<grid, 256, 0, c->stream>>>(m, kk, alpha, Wj, x, beta, yj, c->partials, c->counter);
        else if (kk <= 16) gemv_t_kernel<16, T><<<grid, 256, 0, c->stream>>>(m, kk, alpha, Wj, x, beta, yj, c->partials, c->counter);
        else if (kk <= 32) gemv_t_kernel<32, T><<<grid, 256, 0, c->stream>>>(m, kk, alpha, Wj, x, beta, yj, c->partials, c->counter);
        else gemv_t_kernel<64, T><<<grid, 256, 0, c->stream>>>(m, kk, alpha, Wj, x, beta, yj, c->partials, c->counter);
        HGB_TRY(launch_check("gemv_t_kernel"));
    }
    return HGB_OK;
}

template <typename T>
static int dgmm_impl(hgb_ctx *c, char side, int m, int k, const T *A, const T *x, T *C) {
    if (!c || m < 0 || k < 0) return fail(HGB_ERR_ARG, "dgmm: m=%d k=%d", m, k);
    if (side != 'L' && side != 'l' && side != 'R' && side != 'r') return fail(HGB_ERR_ARG, "dgmm: side '%c'", side);
    if ((long)m * k == 0) return HGB_OK;
    DeviceGuard g(c->device);
    dgmm_kernel<T><<<reduce_grid(c, (long)m * k, 256 * 4), 256, 0, c->stream>>>(m, k, (side == 'L' || side == 'l') ? 1 : 0,
                                                                                 A, x, C);
    return launch_check("dgmm_kernel");
}
}  // namespace hgb

extern "C" {

int hgb_gemv_f64(hgb_ctx *c, char trans, int m, int k, double alpha, const double *W, const double *x, double beta,
                 double *y) {
    return gemv_impl<double>(c, trans, m, k, alpha, W, x, beta, y);
}
int hgb_gemv_f32(hgb_ctx *c, char trans, int m, int k, float alpha, const float *W, const float *x, float beta,
                 float *y) {
    return gemv_impl<float>(c, trans, m, k, alpha, W, x, beta, y);
}
int hgb_dgmm_f64(hgb_ctx *c, char side, int m, int k, const double *A, const double *x, double *C) {
    return dgmm_impl<double>(c, side, m, k, A, x, C);
}
int hgb_dgmm_f32(hgb_ctx *c, char side, int m, int k, const float *A, const float *x, float *C) {
    return dgmm_impl<float>(c, side, m, k, A, x, C);
}

int hgb_diag_index(hgb_ctx *c, int n, int nnz, const int *pntr, const int *indx, int *diag) {
    if (!c || n <= 0 || nnz < 0 || !pntr || !indx || !diag) return fail(HGB_ERR_ARG, "diag_index: bad arguments");
    DeviceGuard g(c->device);
    diag_index_kernel<<<(n + 255) / 256, 256, 0, c->stream>>>(n, pntr, indx, diag, c->err);
    HGB_TRY(launch_check("diag_index_kernel"));
    return collect_dev_error(c);
}

int hgb_selftest_wait_timeout(hgb_ctx *c, int spin_limit) {
    if (!c || spin_limit <= 0) return fail(HGB_ERR_ARG, "selftest: bad arguments");
    DeviceGuard g(c->device);
    double *slot = c->result + 7;
    fill_pending_f64<<<1, 32, 0, c->stream>>>(1, slot);
    wait_timeout_kernel<<<1, 32, 0, c->stream>>>(slot, c->err, spin_limit);
    HGB_TRY(launch_check("wait_timeout_kernel"));
    return collect_dev_error(c);
}

}  // extern "C"
