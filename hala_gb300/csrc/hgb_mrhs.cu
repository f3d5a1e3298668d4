// Several right-hand sides with one matrix: the SpMM, the ILU(0) apply and the multi-RHS PCG of
// solve_batch_cg / solve_batch_cg_ilu (hex/solvers/hala_solvers_cg_batch.hpp:68-248).
//
// Vectors are n x nrhs column-major, as in the reference.  The SpMM is the reference's
// sparse_gemm_array (sparse/hala_sparse_utils.hpp:127-133), one sparse_gemv_array per column: here
// one kernel reads the matrix once and sums every column in the single-column product's order, so
// each column is bit-identical to hgb_csr_gemv.  The ILU apply runs the single-column sweeps per
// column.  The PCG follows solve_cg_core (hex/solvers/hala_solvers_cg.hpp:92-156) with one scalar
// per column (batch_dot, vdivide, batch_axpy, batch_scal of wax/hala_blas_extensions.hpp) and
// stops when iterations >= max_iter (the reference tests ==) or batch_max_norm2(r) < tol, i.e.
// when the largest column norm is below tol (all columns iterate together).  The column scalars
// stay on the device; the host reads one number per iteration for the stopping test.
#include "hgb_internal.cuh"
#include "hgb_kernels.cuh"

#include <algorithm>
#include <cmath>

namespace hgb {

constexpr int kMrBlock = 256;
constexpr int kMrMaxParts = 512;   // reduction blocks per column

// partial dot products of column c (blockIdx.y), rows split over gridDim.x blocks
template <typename X>
__global__ void mr_dot_partial_kernel(long n, int nparts, const X *__restrict__ x, const X *__restrict__ y,
                                      double *__restrict__ partial) {
    const long off = (long)blockIdx.y * n;
    DotAcc<X> d;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        d.add(x[off + i], y[off + i]);
    double acc[1] = {d.get()};
    block_sum<1>(acc);
    if (threadIdx.x == 0) partial[blockIdx.y * nparts + blockIdx.x] = acc[0];
}

// column sums of the partials in block order (deterministic); out[c] in the solution type
template <typename X>
__global__ void mr_dot_final_kernel(int nparts, const double *__restrict__ partial, X *__restrict__ out) {
    double acc[1] = {0.0};
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc[0] += partial[blockIdx.x * nparts + i];
    block_sum<1>(acc);
    if (threadIdx.x == 0) out[blockIdx.x] = (X)acc[0];
}

// q[c] = num[c] / den[c]  (vdivide)
template <typename X>
__global__ void mr_div_kernel(int nrhs, const X *num, const X *den, X *q) {
    for (int c = threadIdx.x; c < nrhs; c += blockDim.x) q[c] = num[c] / den[c];
}

// y[:, c] += (sign * a[c]) * x[:, c]  (batch_axpy with the constant factor sign = +-1)
template <typename X>
__global__ void mr_axpy_kernel(long n, int nrhs, X sign, const X *__restrict__ a, const X *__restrict__ x,
                               X *__restrict__ y) {
    const long total = n * nrhs;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const X s = sign * a[i / n];
        y[i] = add_rn(y[i], mul_rn(s, x[i]));
    }
}

// p[:, c] = a[c] * p[:, c], then p += z  (batch_scal and axpy(1, z, p))
template <typename X>
__global__ void mr_scal_add_kernel(long n, int nrhs, const X *__restrict__ a, const X *__restrict__ z,
                                   X *__restrict__ p) {
    const long total = n * nrhs;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x)
        p[i] = add_rn(mul_rn(a[i / n], p[i]), z[i]);
}

template <typename X>
__global__ void mr_fill_kernel(int n, X v, X *out) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = v;
}

// *out = sqrt(max_c |norms[c]|)  (batch_max_norm2 from the column dot products)
template <typename X>
__global__ void mr_maxnorm_kernel(int nrhs, const X *norms, double *out) {
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int c = 0; c < nrhs; c++) m = fmax(m, fabs((double)norms[c]));
        *out = sqrt(m);
    }
}

template <typename X>
static int mr_dot(hgb_ctx *c, long n, int nrhs, const X *x, const X *y, X *out, double *partial) {
    const int nparts = (int)std::max<long>(1, std::min<long>(kMrMaxParts, (n + kMrBlock * 8 - 1) / (kMrBlock * 8)));
    mr_dot_partial_kernel<X><<<dim3(nparts, nrhs), kMrBlock, 0, c->stream>>>(n, nparts, x, y, partial);
    mr_dot_final_kernel<X><<<nrhs, kMrBlock, 0, c->stream>>>(nparts, partial, out);
    return launch_check("mr_dot");
}

static int mr_grid(hgb_ctx *c, long total) {
    return (int)std::max<long>(1, std::min<long>((total + kMrBlock - 1) / kMrBlock, (long)c->num_sms * 8));
}

template <typename V>
static int mr_gemm(hgb_csr *A, int nrhs, typename Val<V>::X alpha, const typename Val<V>::X *x, long ldx,
                   typename Val<V>::X beta, typename Val<V>::X *y, long ldy) {
    return spmm_n_launch<V>(csr_ctx(A), csr_rows(A), csr_pntr(A), csr_indx(A), (const V *)csr_vals(A), nrhs, alpha, x,
                            ldx, beta, y, ldy);
}

template <typename X>
static int mr_precond(hgb_ctx *c, hgb_ilu *M, long n, int nrhs, const X *r, X *z) {
    if (!M) {
        HGB_CUDA(cudaMemcpyAsync(z, r, sizeof(X) * n * nrhs, cudaMemcpyDeviceToDevice, c->stream));
        return HGB_OK;
    }
    for (int k = 0; k < nrhs; k++) HGB_TRY(ilu_apply_internal(M, 'N', r + k * n, z + k * n));
    return HGB_OK;
}

template <typename V>
static int mr_cg(hgb_ctx *c, hgb_csr *A, hgb_ilu *M, int nrhs, const typename Val<V>::X *b, typename Val<V>::X *x,
                 double tol, int max_iter, int *iters, double *res) {
    using X = typename Val<V>::X;
    const long n = csr_rows(A), total = n * nrhs;
    X *r = nullptr, *p = nullptr, *ap = nullptr, *z = nullptr, *sc = nullptr;
    double *partial = nullptr, *norm = nullptr;
    auto release = [&]() {
        cudaFreeAsync(r, c->stream);
        cudaFreeAsync(p, c->stream);
        cudaFreeAsync(ap, c->stream);
        cudaFreeAsync(z, c->stream);
        cudaFreeAsync(sc, c->stream);
        cudaFreeAsync(partial, c->stream);
        cudaFreeAsync(norm, c->stream);
    };
    int st = HGB_OK;
    do {
        if (cudaMallocFromPoolAsync((void **)&r, sizeof(X) * total, c->pool, c->stream) != cudaSuccess ||
            cudaMallocFromPoolAsync((void **)&p, sizeof(X) * total, c->pool, c->stream) != cudaSuccess ||
            cudaMallocFromPoolAsync((void **)&ap, sizeof(X) * total, c->pool, c->stream) != cudaSuccess ||
            cudaMallocFromPoolAsync((void **)&z, sizeof(X) * total, c->pool, c->stream) != cudaSuccess ||
            cudaMallocFromPoolAsync((void **)&sc, sizeof(X) * 3 * nrhs, c->pool, c->stream) != cudaSuccess ||
            cudaMallocFromPoolAsync((void **)&partial, sizeof(double) * kMrMaxParts * nrhs, c->pool, c->stream) != cudaSuccess ||
            cudaMallocFromPoolAsync((void **)&norm, sizeof(double), c->pool, c->stream) != cudaSuccess) {
            st = fail(HGB_ERR_ALLOC, "cg_solve_nrhs: device memory for %d columns of %ld rows", nrhs, n);
            break;
        }
        X *zr = sc, *nzr = sc + nrhs, *a = sc + 2 * nrhs;
        const int g = mr_grid(c, total);
        // r = b - A x;  z = M^-1 r;  p = z;  zr = <r, z>
        if ((st = mr_gemm<V>(A, nrhs, X(1), x, n, X(0), p, n))) break;
        if (cudaMemcpyAsync(r, b, sizeof(X) * total, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) {
            st = cuda_fail(cudaGetLastError(), "cg_solve_nrhs");
            break;
        }
        {
            // axpy(-1, p, r) over the whole block of columns
            X *ones = nzr;   // scratch: the factor 1 per column
            mr_fill_kernel<X><<<1, 32, 0, c->stream>>>(nrhs, X(1), ones);
            mr_axpy_kernel<X><<<g, kMrBlock, 0, c->stream>>>(n, nrhs, X(-1), ones, p, r);
        }
        if ((st = mr_precond<X>(c, M, n, nrhs, r, z))) break;
        if (cudaMemcpyAsync(p, z, sizeof(X) * total, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) {
            st = cuda_fail(cudaGetLastError(), "cg_solve_nrhs");
            break;
        }
        if ((st = mr_dot<X>(c, n, nrhs, r, z, zr, partial))) break;
        int it = 1;
        double rn = 0.0;
        for (;;) {
            if ((st = mr_gemm<V>(A, nrhs, X(1), p, n, X(0), ap, n))) break;
            it++;
            if ((st = mr_dot<X>(c, n, nrhs, p, ap, nzr, partial))) break;
            mr_div_kernel<X><<<1, 32, 0, c->stream>>>(nrhs, zr, nzr, a);
            mr_axpy_kernel<X><<<g, kMrBlock, 0, c->stream>>>(n, nrhs, X(1), a, p, x);
            mr_axpy_kernel<X><<<g, kMrBlock, 0, c->stream>>>(n, nrhs, X(-1), a, ap, r);
            if ((st = mr_dot<X>(c, n, nrhs, r, r, nzr, partial))) break;
            mr_maxnorm_kernel<X><<<1, 32, 0, c->stream>>>(nrhs, nzr, norm);
            if ((st = launch_check("cg_solve_nrhs"))) break;
            if (cudaMemcpyAsync(&rn, norm, sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
                cudaStreamSynchronize(c->stream) != cudaSuccess) {
                st = cuda_fail(cudaGetLastError(), "cg_solve_nrhs");
                break;
            }
            if ((st = collect_dev_error(c))) break;
            if (it >= max_iter || rn < tol || std::isnan(rn)) break;
            if ((st = mr_precond<X>(c, M, n, nrhs, r, z))) break;
            if ((st = mr_dot<X>(c, n, nrhs, r, z, nzr, partial))) break;
            mr_div_kernel<X><<<1, 32, 0, c->stream>>>(nrhs, nzr, zr, a);
            mr_scal_add_kernel<X><<<g, kMrBlock, 0, c->stream>>>(n, nrhs, a, z, p);
            if (cudaMemcpyAsync(zr, nzr, sizeof(X) * nrhs, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) {
                st = cuda_fail(cudaGetLastError(), "cg_solve_nrhs");
                break;
            }
        }
        *iters = it;
        *res = rn;
    } while (false);
    release();
    return st;
}

}  // namespace hgb

using namespace hgb;

extern "C" {

int hgb_csr_gemm(hgb_csr *A, int nrhs, double alpha, const void *x, int ldx, double beta, void *y, int ldy) {
    if (!A || nrhs < 0 || (nrhs > 0 && (!x || !y)) || ldx < csr_cols(A) || ldy < csr_rows(A))
        return fail(HGB_ERR_ARG, "csr_gemm: bad arguments");
    DeviceGuard g(csr_ctx(A)->device);
    switch (csr_dtype(A)) {
        case HGB_F64:
            return mr_gemm<double>(A, nrhs, alpha, (const double *)x, ldx, beta, (double *)y, ldy);
        case HGB_F32:
            return mr_gemm<float>(A, nrhs, (float)alpha, (const float *)x, ldx, (float)beta, (float *)y, ldy);
        case HGB_C128:
        case HGB_C64:
            return fail(HGB_ERR_UNSUPPORTED, "csr_gemm: real matrices (complex products go column by column through csr_gemv)");
        default:
            return mr_gemm<uint16_t>(A, nrhs, (float)alpha, (const float *)x, ldx, (float)beta, (float *)y, ldy);
    }
}

int hgb_ilu0_apply_nrhs(hgb_ilu *M, char trans, int nrhs, const void *x, void *r) {
    if (!M || nrhs < 0 || (nrhs > 0 && (!x || !r))) return fail(HGB_ERR_ARG, "ilu0_apply_nrhs: bad arguments");
    const long n = ilu_n(M);
    const size_t xs = ilu_xbytes(M);
    for (int k = 0; k < nrhs; k++)
        HGB_TRY(ilu_apply_internal(M, trans, (const char *)x + k * n * xs, (char *)r + k * n * xs));
    return HGB_OK;
}

int hgb_cg_solve_nrhs(hgb_ctx *c, hgb_csr *A, hgb_ilu *M, int nrhs, const void *B, void *X, double tol, int max_iter,
                      hgb_solve_info *info) {
    if (!c || !A || nrhs < 1 || !B || !X) return fail(HGB_ERR_ARG, "cg_solve_nrhs: bad arguments");
    if (csr_rows(A) != csr_cols(A)) return fail(HGB_ERR_ARG, "cg_solve_nrhs: square matrix required");
    if (max_iter < 1) return fail(HGB_ERR_ARG, "cg_solve_nrhs: max_iter < 1");
    DeviceGuard g(c->device);
    const hgb_dtype dt = csr_dtype(A);
    if (dt == HGB_C128 || dt == HGB_C64) return fail(HGB_ERR_UNSUPPORTED, "cg_solve_nrhs: real matrices");
    if (M) {
        if (ilu_n(M) != csr_rows(A)) return fail(HGB_ERR_ARG, "cg_solve_nrhs: preconditioner size");
        if (!ilu_matches(ilu_store(M), dt)) return fail(HGB_ERR_ARG, "cg_solve_nrhs: preconditioner precision does not match the matrix");
    }
    int it = 0;
    double rn = 0.0;
    int st;
    if (dt == HGB_F64) st = mr_cg<double>(c, A, M, nrhs, (const double *)B, (double *)X, tol, max_iter, &it, &rn);
    else if (dt == HGB_F32) st = mr_cg<float>(c, A, M, nrhs, (const float *)B, (float *)X, tol, max_iter, &it, &rn);
    else st = mr_cg<uint16_t>(c, A, M, nrhs, (const float *)B, (float *)X, tol, max_iter, &it, &rn);
    if (st) return st;
    if (info) {
        info->iterations = it;
        info->outer = 0;
        info->residual = rn;
        info->true_residual = -1.0;
        info->kernel_launches = -1;
    }
    return HGB_OK;
}

}  // extern "C"
