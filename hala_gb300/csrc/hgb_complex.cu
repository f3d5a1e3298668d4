// Complex variants of the path (C128: pairs of doubles, C64: pairs of floats, interleaved real and
// imaginary parts as std::complex / cuDoubleComplex store them).  The reference's templates are
// generic over std::complex<float> and std::complex<double> (sparse/hala_sparse_utils.hpp:104-336,
// hex/solvers/*.hpp) and its own solver tests run all four types (tests/solvers_tests.cpp:15-40).
//
//  - SpMV 'N' (thread per row, column order), 'T' and 'C' (the matrix's cached transpose: one
//    thread per column, entries in ascending original row, 'C' conjugating the values; without a
//    matrix object the scatter uses atomics): the arithmetic of sparse_gemv_array (utils:104-118).
//  - BLAS-1: dotc / dotu, nrm2, axpy, scal (grid reductions accumulate in double).
//  - ILU(0): the row-wise IKJ order of factorize_ilu_array (utils:229-255), rows of one level of
//    the lower pattern factorised in parallel (one launch per level); the apply and the triangular
//    solves sweep level by level in the orders of apply_ilu_array (utils:263-276) and
//    sparse_trsv_array (utils:284-336), 'T' and 'C' through the transposed pattern.
//  - CG and GMRES: the loops of solve_cg_core and solve_gmres (hex/solvers/hala_solvers_cg.hpp:92-156,
//    hala_solvers_gmres.hpp:127-230) driven from the host with device BLAS-1 (host scalars, as the
//    reference's GPU path).  CG's inner products conjugate (hala::dot); GMRES projects with the
//    unconjugated transpose, as the reference's krylov_project does (gemv 'T',
//    hala_solvers_gmres.hpp:47-50,67-72).
// Products and sums are separately rounded (re = ac - bd, im = ad + bc), the reference's std::complex
// multiplication; complex division follows Smith's method (R. L. Smith, CACM 5(8), 1962).  Results
// are compared with the reference within a tolerance (1e-12 relative for C128, 1e-5 for C64), not
// bit for bit: libstdc++'s complex division scales differently.
#include "hgb_internal.cuh"
#include "hgb_kernels.cuh"
#include "hgb_complex.cuh"

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

namespace hgb {

template <typename R> struct alignas(2 * sizeof(R)) Cx {
    R re, im;
};

template <typename R> __host__ __device__ __forceinline__ Cx<R> cx(R re, R im) { return Cx<R>{re, im}; }

__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float rdiv(float a, float b) { return __fdiv_rn(a, b); }

template <typename R> __device__ __forceinline__ Cx<R> zadd(Cx<R> a, Cx<R> b) { return cx(radd(a.re, b.re), radd(a.im, b.im)); }
template <typename R> __device__ __forceinline__ Cx<R> zsub(Cx<R> a, Cx<R> b) { return cx(rsub(a.re, b.re), rsub(a.im, b.im)); }
template <typename R> __device__ __forceinline__ Cx<R> zmul(Cx<R> a, Cx<R> b) {
    return cx(rsub(rmul(a.re, b.re), rmul(a.im, b.im)), radd(rmul(a.re, b.im), rmul(a.im, b.re)));
}
template <typename R> __device__ __forceinline__ Cx<R> zconj(Cx<R> a) { return cx(a.re, -a.im); }
// Smith's division: divide by the larger of |b.re| and |b.im| first
template <typename R> __device__ __forceinline__ Cx<R> zdiv(Cx<R> a, Cx<R> b) {
    if (fabs(b.re) >= fabs(b.im)) {
        if (b.re == R(0) && b.im == R(0)) return cx(rdiv(a.re, b.re), rdiv(a.im, b.re));   // inf / nan as IEEE gives
        const R r = rdiv(b.im, b.re), den = radd(b.re, rmul(b.im, r));
        return cx(rdiv(radd(a.re, rmul(a.im, r)), den), rdiv(rsub(a.im, rmul(a.re, r)), den));
    }
    const R r = rdiv(b.re, b.im), den = radd(rmul(b.re, r), b.im);
    return cx(rdiv(radd(rmul(a.re, r), a.im), den), rdiv(rsub(rmul(a.im, r), a.re), den));
}
template <typename R> __device__ __forceinline__ bool zzero(Cx<R> a) { return a.re == R(0) && a.im == R(0); }

static int zgrid(hgb_ctx *c, long work) {
    return (int)std::max<long>(1, std::min<long>((work + 255) / 256, (long)c->num_sms * 8));
}

// ----------------------------------------------------------------------------- SpMV ------
// y = alpha A x + beta y (beta == 0 does not read y); rows summed in column order
template <typename R>
__global__ void zspmv_n_kernel(int n_rows, const int *__restrict__ pntr, const int *__restrict__ indx,
                               const Cx<R> *__restrict__ vals, Cx<R> alpha, const Cx<R> *__restrict__ x, Cx<R> beta,
                               Cx<R> *__restrict__ y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_rows; i += gridDim.x * blockDim.x) {
        Cx<R> sum = cx<R>(0, 0);
        for (int j = pntr[i]; j < pntr[i + 1]; j++) sum = zadd(sum, zmul(vals[j], x[indx[j]]));
        const Cx<R> a = zmul(alpha, sum);
        y[i] = zzero(beta) ? a : zadd(a, zmul(beta, y[i]));
    }
}

// through the cached transpose: y_c = beta y_c + sum over rows i of column c, ascending, (alpha x_i) v
template <typename R>
__global__ void zspmv_t_cached_kernel(int n_cols, const int *__restrict__ pntrT, const int *__restrict__ rowT,
                                      const int *__restrict__ mapT, const Cx<R> *__restrict__ vals, int conj,
                                      Cx<R> alpha, const Cx<R> *__restrict__ x, Cx<R> beta, Cx<R> *__restrict__ y) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n_cols; c += gridDim.x * blockDim.x) {
        Cx<R> acc = zzero(beta) ? cx<R>(0, 0) : zmul(beta, y[c]);
        for (int p = pntrT[c]; p < pntrT[c + 1]; p++) {
            Cx<R> v = vals[mapT[p]];
            if (conj) v = zconj(v);
            acc = zadd(acc, zmul(zmul(alpha, x[rowT[p]]), v));
        }
        y[c] = acc;
    }
}

template <typename R>
__global__ void zscale_kernel(long n, Cx<R> beta, Cx<R> *y) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        y[i] = zzero(beta) ? cx<R>(0, 0) : zmul(beta, y[i]);
}

template <typename R>
__global__ void zspmv_t_atomic_kernel(int n_rows, const int *__restrict__ pntr, const int *__restrict__ indx,
                                      const Cx<R> *__restrict__ vals, int conj, Cx<R> alpha,
                                      const Cx<R> *__restrict__ x, Cx<R> *y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_rows; i += gridDim.x * blockDim.x) {
        const Cx<R> ax = zmul(alpha, x[i]);
        for (int p = pntr[i]; p < pntr[i + 1]; p++) {
            Cx<R> v = vals[p];
            if (conj) v = zconj(v);
            const Cx<R> t = zmul(ax, v);
            atomicAdd(&y[indx[p]].re, t.re);
            atomicAdd(&y[indx[p]].im, t.im);
        }
    }
}

template <typename R>
int zspmv(hgb_ctx *c, char trans, int n_rows, int n_cols, const int *pntr, const int *indx, const void *vals,
          const R *alpha, const void *x, const R *beta, void *y, const Transpose *T) {
    const Cx<R> a = cx(alpha[0], alpha[1]), b = cx(beta[0], beta[1]);
    const Cx<R> *V = (const Cx<R> *)vals, *X = (const Cx<R> *)x;
    Cx<R> *Y = (Cx<R> *)y;
    if (trans == 'N' || trans == 'n') {
        if (n_rows <= 0) return HGB_OK;
        zspmv_n_kernel<R><<<zgrid(c, n_rows), 256, 0, c->stream>>>(n_rows, pntr, indx, V, a, X, b, Y);
        return launch_check("zspmv_n_kernel");
    }
    const int conj = (trans == 'C' || trans == 'c') ? 1 : 0;
    if (n_cols <= 0) return HGB_OK;
    if (T) {
        zspmv_t_cached_kernel<R><<<zgrid(c, n_cols), 256, 0, c->stream>>>(n_cols, T->pntr, T->row, T->map, V, conj, a, X,
                                                                          b, Y);
        return launch_check("zspmv_t_cached_kernel");
    }
    zscale_kernel<R><<<zgrid(c, n_cols), 256, 0, c->stream>>>(n_cols, b, Y);
    if (n_rows > 0)
        zspmv_t_atomic_kernel<R><<<zgrid(c, n_rows), 256, 0, c->stream>>>(n_rows, pntr, indx, V, conj, a, X, Y);
    return launch_check("zspmv_t_atomic_kernel");
}
template int zspmv<double>(hgb_ctx *, char, int, int, const int *, const int *, const void *, const double *,
                           const void *, const double *, void *, const Transpose *);
template int zspmv<float>(hgb_ctx *, char, int, int, const int *, const int *, const void *, const float *,
                          const void *, const float *, void *, const Transpose *);

// --------------------------------------------------------------------------- BLAS-1 ------
// op 0: sum conj(x_i) y_i; op 1: sum x_i y_i; op 2: sqrt(sum conj(x_i) x_i) (real)
template <typename R>
__global__ void zdot_kernel(long n, const Cx<R> *__restrict__ x, const Cx<R> *__restrict__ y, double *partials,
                            unsigned *counter, R *out, int op) {
    double acc[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double xr = x[i].re, xi = (op == 1) ? (double)x[i].im : -(double)x[i].im;
        const double yr = (op == 2) ? (double)x[i].re : (double)y[i].re;
        const double yi = (op == 2) ? (double)x[i].im : (double)y[i].im;
        acc[0] += xr * yr - xi * yi;
        acc[1] += xr * yi + xi * yr;
    }
    grid_sum<2>(acc, partials, counter, [&](double (&s)[2]) {
        if (op == 2) {
            out[0] = (R)sqrt(s[0]);
        } else {
            out[0] = (R)s[0];
            out[1] = (R)s[1];
        }
    });
}

template <typename R>
__global__ void zaxpy_kernel(long n, Cx<R> a, const Cx<R> *__restrict__ x, Cx<R> *__restrict__ y) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        y[i] = zadd(y[i], zmul(a, x[i]));
}

template <typename R>
__global__ void zscal_kernel(long n, Cx<R> a, Cx<R> *__restrict__ x) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        x[i] = zmul(a, x[i]);
}

template <typename R>
int zdot(hgb_ctx *c, int op, int n, const void *x, const void *y, R *result, int on_device) {
    if (n < 0 || !result || (n > 0 && (!x || !y))) return fail(HGB_ERR_ARG, "complex dot: bad arguments");
    const int nr = (op == 2) ? 1 : 2;
    if (n == 0) {
        if (on_device) HGB_CUDA(cudaMemsetAsync(result, 0, sizeof(R) * nr, c->stream));
        else for (int k = 0; k < nr; k++) result[k] = R(0);
        return HGB_OK;
    }
    R *out = on_device ? result : (R *)c->result;
    zdot_kernel<R><<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, (const Cx<R> *)x, (const Cx<R> *)y, c->partials,
                                                                       c->counter, out, op);
    HGB_TRY(launch_check("zdot_kernel"));
    if (!on_device) {
        HGB_CUDA(cudaMemcpyAsync(c->host_result, out, sizeof(R) * nr, cudaMemcpyDeviceToHost, c->stream));
        HGB_CUDA(cudaStreamSynchronize(c->stream));
        for (int k = 0; k < nr; k++) result[k] = ((R *)c->host_result)[k];
    }
    return HGB_OK;
}

template <typename R>
int zaxpy(hgb_ctx *c, int n, const R *alpha, const void *x, void *y) {
    if (n < 0 || !alpha || (n > 0 && (!x || !y))) return fail(HGB_ERR_ARG, "complex axpy: bad arguments");
    if (n == 0) return HGB_OK;
    zaxpy_kernel<R><<<zgrid(c, n), 256, 0, c->stream>>>(n, cx(alpha[0], alpha[1]), (const Cx<R> *)x, (Cx<R> *)y);
    return launch_check("zaxpy_kernel");
}

template <typename R>
int zscal(hgb_ctx *c, int n, const R *alpha, void *x) {
    if (n < 0 || !alpha || (n > 0 && !x)) return fail(HGB_ERR_ARG, "complex scal: bad arguments");
    if (n == 0) return HGB_OK;
    zscal_kernel<R><<<zgrid(c, n), 256, 0, c->stream>>>(n, cx(alpha[0], alpha[1]), (Cx<R> *)x);
    return launch_check("zscal_kernel");
}

// ------------------------------------------------------------- level-synchronous sweeps ----
// Host-side levels of a triangular dependency graph: rows grouped by level, in solve order.
struct ZLevels {
    int nlev = 0;
    int *perm = nullptr;    // rows, level by level (device)
    std::vector<int> hptr;  // level offsets into perm [nlev + 1]
    void release() {
        cudaFree(perm);
        perm = nullptr;
        nlev = 0;
        hptr.clear();
    }
};

// levels of rows 0..n-1 where row i depends on the columns deps(i) (all earlier in solve order)
template <typename Deps>
static int zlevels(int n, bool forward, Deps deps, ZLevels &Lv) {
    std::vector<int> lev(n, 0);
    int nl = 0;
    for (int k = 0; k < n; k++) {
        const int i = forward ? k : n - 1 - k;
        int l = 0;
        deps(i, [&](int j) { l = std::max(l, lev[j] + 1); });
        lev[i] = l;
        nl = std::max(nl, l + 1);
    }
    std::vector<int> cnt(nl + 1, 0), perm(n);
    for (int i = 0; i < n; i++) cnt[lev[i] + 1]++;
    for (int l = 0; l < nl; l++) cnt[l + 1] += cnt[l];
    std::vector<int> cur(cnt.begin(), cnt.end() - 1);
    for (int k = 0; k < n; k++) {
        const int i = forward ? k : n - 1 - k;
        perm[cur[lev[i]]++] = i;
    }
    Lv.release();
    Lv.nlev = nl;
    Lv.hptr = cnt;
    HGB_CUDA(cudaMalloc(&Lv.perm, sizeof(int) * std::max(n, 1)));
    HGB_CUDA(cudaMemcpy(Lv.perm, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    return HGB_OK;
}

// ILU(0) row i (rows of one level of the lower pattern, in parallel): for each lower entry (i, j) in
// ascending j, a_ij /= a_jj, then a_ik -= a_ij a_jk over the matching columns k > j of row j
template <typename R>
__global__ void zilu_level_kernel(const int *__restrict__ rows, int cnt, const int *__restrict__ pntr,
                                  const int *__restrict__ indx, const int *__restrict__ diag, Cx<R> *f, int *err) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < cnt; t += gridDim.x * blockDim.x) {
        const int i = rows[t];
        for (int q = pntr[i]; q < diag[i]; q++) {
            const int j = indx[q];
            const Cx<R> u = f[diag[j]];
            if (zzero(u)) atomicOr(err, DEV_ERR_ZERO_PIVOT);
            const Cx<R> l = zdiv(f[q], u);
            f[q] = l;
            int jk = diag[j] + 1, ik = q + 1;
            const int je = pntr[j + 1], ie = pntr[i + 1];
            while (jk < je && ik < ie) {
                const int a = indx[jk], b = indx[ik];
                if (a == b) {
                    f[ik] = zsub(f[ik], zmul(l, f[jk]));
                    jk++;
                    ik++;
                } else if (a < b) {
                    jk++;
                } else {
                    ik++;
                }
            }
        }
    }
}

// One level of a triangular sweep on the rows of one level, strict part [a, e) of each row:
// MODE 0 (apply_ilu_array): x_i = (b_i - sum v x) [/ d];  MODE 1 (sparse_trsv_array): the sum
// accumulated first, x_i = (alpha b_i - sum) [/ d].  For the transposed solves the pattern is the
// transpose (values through map, conjugated for 'C').
template <typename R, int MODE>
__global__ void zsweep_level_kernel(const int *__restrict__ rows, int cnt, const int *__restrict__ pntr,
                                    const int *__restrict__ indx, const int *__restrict__ map, const int *__restrict__ diag,
                                    int lower, int unit, int conj, const Cx<R> *__restrict__ vals, Cx<R> alpha,
                                    const Cx<R> *__restrict__ b, Cx<R> *x) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < cnt; t += gridDim.x * blockDim.x) {
        const int i = rows[t];
        const int d = diag[i];
        const int a = lower ? pntr[i] : d + 1, e = lower ? d : pntr[i + 1];
        auto val = [&](int p) {
            Cx<R> v = vals[map ? map[p] : p];
            return conj ? zconj(v) : v;
        };
        Cx<R> acc;
        if (MODE == 0) {
            acc = b[i];
            for (int p = a; p < e; p++) acc = zsub(acc, zmul(val(p), x[indx[p]]));
        } else {
            Cx<R> s = cx<R>(0, 0);
            for (int p = a; p < e; p++) s = zadd(s, zmul(val(p), x[indx[p]]));
            acc = zsub(zmul(alpha, b[i]), s);
        }
        x[i] = unit ? acc : zdiv(acc, val(d));
    }
}

__global__ void zdiag_index_kernel(int n, const int *__restrict__ pntr, const int *__restrict__ indx, int *diag,
                                   int *err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int pos = -1;
        for (int p = pntr[i]; p < pntr[i + 1]; p++)
            if (indx[p] == i) pos = p;
        if (pos < 0) atomicOr(err, DEV_ERR_CSR);
        diag[i] = pos;
    }
}

// A triangular system on a (possibly full) CSR pattern: the lower or upper triangle and its levels,
// plus, built on first transposed use, the transposed pattern and its levels.
struct ZTriangle {
    int n = 0, nnz = 0;
    bool lower = true;
    const int *pntr = nullptr, *indx = nullptr;
    int *diag = nullptr;
    ZLevels lev;
    bool has_T = false;
    Transpose T;
    int *diagT = nullptr;
    ZLevels levT;
    void release() {
        cudaFree(diag);
        lev.release();
        if (has_T) {
            T.release();
            cudaFree(diagT);
            levT.release();
        }
        diag = diagT = nullptr;
        has_T = false;
    }
};

// diag_d: the diagonal index when the caller has it (device), else found here
static int ztri_setup(hgb_ctx *c, int n, int nnz, const int *pntr, const int *indx, const int *diag_d, bool lower,
                      ZTriangle &Z) {
    Z.n = n;
    Z.nnz = nnz;
    Z.lower = lower;
    Z.pntr = pntr;
    Z.indx = indx;
    HGB_CUDA(cudaMalloc(&Z.diag, sizeof(int) * n));
    if (diag_d) {
        HGB_CUDA(cudaMemcpyAsync(Z.diag, diag_d, sizeof(int) * n, cudaMemcpyDeviceToDevice, c->stream));
    } else {
        zdiag_index_kernel<<<zgrid(c, n), 256, 0, c->stream>>>(n, pntr, indx, Z.diag, c->err);
        HGB_TRY(launch_check("zdiag_index_kernel"));
        HGB_TRY(collect_dev_error(c));
    }
    std::vector<int> hp(n + 1), hi(std::max(nnz, 1)), hd(n);
    HGB_CUDA(cudaMemcpyAsync(hp.data(), pntr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaMemcpyAsync(hi.data(), indx, sizeof(int) * nnz, cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaMemcpyAsync(hd.data(), Z.diag, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    return zlevels(n, lower, [&](int i, auto use) {
        const int a = lower ? hp[i] : hd[i] + 1, e = lower ? hd[i] : hp[i + 1];
        for (int p = a; p < e; p++) use(hi[p]);
    }, Z.lev);
}

// the transposed pattern: the transpose of a lower triangle is upper and conversely
static int ztri_setup_T(hgb_ctx *c, ZTriangle &Z) {
    if (Z.has_T) return HGB_OK;
    HGB_TRY(build_transpose(c, Z.n, Z.n, Z.nnz, Z.pntr, Z.indx, Z.T));
    Z.has_T = true;   // release() frees the transpose from here on
    HGB_CUDA(cudaMalloc(&Z.diagT, sizeof(int) * Z.n));
    zdiag_index_kernel<<<zgrid(c, Z.n), 256, 0, c->stream>>>(Z.n, Z.T.pntr, Z.T.row, Z.diagT, c->err);
    HGB_TRY(launch_check("zdiag_index_kernel"));
    HGB_TRY(collect_dev_error(c));
    const int n = Z.n;
    std::vector<int> hp(n + 1), hi(std::max(Z.nnz, 1)), hd(n);
    HGB_CUDA(cudaMemcpyAsync(hp.data(), Z.T.pntr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaMemcpyAsync(hi.data(), Z.T.row, sizeof(int) * Z.nnz, cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaMemcpyAsync(hd.data(), Z.diagT, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    const bool lowT = !Z.lower;
    return zlevels(n, lowT, [&](int i, auto use) {
        const int a = lowT ? hp[i] : hd[i] + 1, e = lowT ? hd[i] : hp[i + 1];
        for (int p = a; p < e; p++) use(hi[p]);
    }, Z.levT);
}

template <typename R, int MODE>
static int zsweep(hgb_ctx *c, ZTriangle &Z, char trans, int unit, const Cx<R> *vals, Cx<R> alpha, const Cx<R> *b,
                  Cx<R> *x) {
    const bool nt = (trans == 'N' || trans == 'n');
    if (!nt) HGB_TRY(ztri_setup_T(c, Z));
    const ZLevels &L = nt ? Z.lev : Z.levT;
    const int *pntr = nt ? Z.pntr : Z.T.pntr, *indx = nt ? Z.indx : Z.T.row, *map = nt ? nullptr : Z.T.map;
    const int *diag = nt ? Z.diag : Z.diagT;
    const int lower = nt ? (Z.lower ? 1 : 0) : (Z.lower ? 0 : 1);
    const int conj = (trans == 'C' || trans == 'c') ? 1 : 0;
    for (int l = 0; l < L.nlev; l++) {
        const int cnt = L.hptr[l + 1] - L.hptr[l];
        zsweep_level_kernel<R, MODE><<<zgrid(c, cnt), 256, 0, c->stream>>>(L.perm + L.hptr[l], cnt, pntr, indx, map,
                                                                           diag, lower, unit, conj, vals, alpha, b, x);
    }
    return launch_check("zsweep_level_kernel");
}

}  // namespace hgb

using namespace hgb;

// ------------------------------------------------------------------------ objects --------
struct hgb_zilu {
    hgb_ctx *ctx = nullptr;
    int n = 0, nnz = 0, rsize = 8;   // rsize: bytes of one real part (8: C128, 4: C64)
    void *f = nullptr;               // the factor
    void *tmp = nullptr;             // the forward sweep's output
    ZTriangle L, U;
};

struct hgb_ztri {
    hgb_ctx *ctx = nullptr;
    int rsize = 8, unit = 0;
    const void *vals = nullptr;
    void *bcopy = nullptr;
    ZTriangle Z;
};

namespace hgb {

int zilu_create(hgb_ctx *c, int n, int nnz, const int *pntr, const int *indx, const void *vals, int rsize,
                hgb_zilu **out, int *zero_pivot) {
    *out = nullptr;
    HGB_TRY(csr_check(c, n, n, nnz, pntr, indx));
    hgb_zilu *M = new hgb_zilu();
    M->ctx = c;
    M->n = n;
    M->nnz = nnz;
    M->rsize = rsize;
    int st = HGB_OK;
    do {
        const size_t es = 2 * (size_t)rsize;
        if (cudaMalloc(&M->f, es * nnz) != cudaSuccess || cudaMalloc(&M->tmp, es * n) != cudaSuccess) {
            st = cuda_fail(cudaGetLastError(), "complex ilu0_create");
            break;
        }
        if (cudaMemcpyAsync(M->f, vals, es * nnz, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) {
            st = cuda_fail(cudaGetLastError(), "complex ilu0_create");
            break;
        }
        if ((st = ztri_setup(c, n, nnz, pntr, indx, nullptr, true, M->L))) break;
        if ((st = ztri_setup(c, n, nnz, pntr, indx, M->L.diag, false, M->U))) break;
        // factorise level by level over the lower pattern's levels
        for (int l = 0; l < M->L.lev.nlev; l++) {
            const int cnt = M->L.lev.hptr[l + 1] - M->L.lev.hptr[l];
            const int *rows = M->L.lev.perm + M->L.lev.hptr[l];
            if (rsize == 8)
                zilu_level_kernel<double><<<zgrid(c, cnt), 256, 0, c->stream>>>(rows, cnt, pntr, indx, M->L.diag,
                                                                                (Cx<double> *)M->f, c->err);
            else
                zilu_level_kernel<float><<<zgrid(c, cnt), 256, 0, c->stream>>>(rows, cnt, pntr, indx, M->L.diag,
                                                                               (Cx<float> *)M->f, c->err);
        }
        if ((st = launch_check("zilu_level_kernel"))) break;
        st = collect_dev_error(c);
        if (st == HGB_ERR_ZERO_PIVOT) {
            *zero_pivot = 1;
            st = HGB_OK;
        }
    } while (0);
    if (st) {
        zilu_destroy(M);
        return st;
    }
    *out = M;
    return HGB_OK;
}

// r = U^-1 L^-1 x ('N', apply_ilu_array's order) or (LU)^-T / (LU)^-H x (U^T first, then L^T)
int zilu_apply(hgb_zilu *M, char trans, const void *x, void *r) {
    hgb_ctx *c = M->ctx;
    const bool nt = (trans == 'N' || trans == 'n');
    if (M->rsize == 8) {
        using C = Cx<double>;
        C *tmp = (C *)M->tmp;
        if (nt) {
            HGB_TRY((zsweep<double, 0>(c, M->L, 'N', 1, (const C *)M->f, cx(1.0, 0.0), (const C *)x, tmp)));
            return zsweep<double, 0>(c, M->U, 'N', 0, (const C *)M->f, cx(1.0, 0.0), tmp, (C *)r);
        }
        HGB_TRY((zsweep<double, 1>(c, M->U, trans, 0, (const C *)M->f, cx(1.0, 0.0), (const C *)x, tmp)));
        return zsweep<double, 1>(c, M->L, trans, 1, (const C *)M->f, cx(1.0, 0.0), tmp, (C *)r);
    }
    using C = Cx<float>;
    C *tmp = (C *)M->tmp;
    if (nt) {
        HGB_TRY((zsweep<float, 0>(c, M->L, 'N', 1, (const C *)M->f, cx(1.0f, 0.0f), (const C *)x, tmp)));
        return zsweep<float, 0>(c, M->U, 'N', 0, (const C *)M->f, cx(1.0f, 0.0f), tmp, (C *)r);
    }
    HGB_TRY((zsweep<float, 1>(c, M->U, trans, 0, (const C *)M->f, cx(1.0f, 0.0f), (const C *)x, tmp)));
    return zsweep<float, 1>(c, M->L, trans, 1, (const C *)M->f, cx(1.0f, 0.0f), tmp, (C *)r);
}

int zilu_export(hgb_zilu *M, void *factor, int *diag) {
    hgb_ctx *c = M->ctx;
    if (factor) HGB_CUDA(cudaMemcpyAsync(factor, M->f, 2 * (size_t)M->rsize * M->nnz, cudaMemcpyDeviceToDevice, c->stream));
    if (diag) HGB_CUDA(cudaMemcpyAsync(diag, M->L.diag, sizeof(int) * M->n, cudaMemcpyDeviceToDevice, c->stream));
    return HGB_OK;
}

int zilu_rsize(const hgb_zilu *M) { return M->rsize; }

void zilu_destroy(hgb_zilu *M) {
    if (!M) return;
    cudaFree(M->f);
    cudaFree(M->tmp);
    M->L.release();
    M->U.release();
    delete M;
}

int ztri_create(hgb_ctx *c, char uplo, char diag, int n, int nnz, const int *pntr, const int *indx, const void *vals,
                int rsize, hgb_ztri **out) {
    *out = nullptr;
    HGB_TRY(csr_check(c, n, n, nnz, pntr, indx));
    hgb_ztri *T = new hgb_ztri();
    T->ctx = c;
    T->rsize = rsize;
    T->unit = (diag == 'U' || diag == 'u') ? 1 : 0;
    T->vals = vals;
    int st = ztri_setup(c, n, nnz, pntr, indx, nullptr, uplo == 'L' || uplo == 'l', T->Z);
    if (st) {
        ztri_destroy(T);
        return st;
    }
    *out = T;
    return HGB_OK;
}

// op(T) x = alpha b, the arithmetic of sparse_trsv_array (sum first, then alpha b - sum, / d)
int ztri_solve(hgb_ztri *T, char trans, const void *alpha, const void *b, void *x) {
    hgb_ctx *c = T->ctx;
    const size_t es = 2 * (size_t)T->rsize;
    const void *src = b;
    if (b == x) {   // the sweep reads b while it writes x
        if (!T->bcopy) HGB_CUDA(cudaMalloc(&T->bcopy, es * T->Z.n));
        HGB_CUDA(cudaMemcpyAsync(T->bcopy, b, es * T->Z.n, cudaMemcpyDeviceToDevice, c->stream));
        src = T->bcopy;
    }
    if (T->rsize == 8) {
        const double *a = (const double *)alpha;
        return zsweep<double, 1>(c, T->Z, trans, T->unit, (const Cx<double> *)T->vals, cx(a[0], a[1]),
                                 (const Cx<double> *)src, (Cx<double> *)x);
    }
    const float *a = (const float *)alpha;
    return zsweep<float, 1>(c, T->Z, trans, T->unit, (const Cx<float> *)T->vals, cx(a[0], a[1]), (const Cx<float> *)src,
                            (Cx<float> *)x);
}

void ztri_destroy(hgb_ztri *T) {
    if (!T) return;
    cudaFree(T->bcopy);
    T->Z.release();
    delete T;
}

// ------------------------------------------------------------------------- solvers -------
// The loop of solve_cg_core (hex/solvers/hala_solvers_cg.hpp:92-156) with the complex inner product
// <u, v> = sum conj(u_i) v_i (the reference's dot on the GPU engine is cublasZdotc /
// cublasCdotc) and host scalars.  M may be null.  info gets the reference's iteration count.
template <typename R>
static int zcg_run(hgb_ctx *c, hgb_csr *A, hgb_zilu *M, const void *b, void *x, double tol, int max_iter,
                   hgb_solve_info *info) {
    using Z = std::complex<R>;
    const int n = csr_rows(A);
    const size_t es = sizeof(Z);
    char *r = nullptr, *p = nullptr, *Ap = nullptr, *z = nullptr;
    int st = HGB_OK, it = 0;
    R rn = 0;
    long long launches = 0;
    auto dotc = [&](const void *u, const void *v, Z &out) {
        R t[2];
        const int e = zdot<R>(c, 0, n, u, v, t, 0);
        out = Z(t[0], t[1]);
        launches++;
        return e;
    };
    auto spmv = [&](const void *in, void *outv, R alpha, R beta) {
        const R a[2] = {alpha, 0}, bb[2] = {beta, 0};
        launches++;
        return zspmv<R>(c, 'N', n, n, csr_pntr(A), csr_indx(A), csr_vals(A), a, in, bb, outv, nullptr);
    };
    auto axpy = [&](Z a, const void *u, void *v) {
        const R t[2] = {a.real(), a.imag()};
        launches++;
        return zaxpy<R>(c, n, t, u, v);
    };
    auto copy = [&](void *dst, const void *src) {
        return cudaMemcpyAsync(dst, src, es * n, cudaMemcpyDeviceToDevice, c->stream) == cudaSuccess
                   ? HGB_OK
                   : cuda_fail(cudaGetLastError(), "complex cg");
    };
    auto precond = [&](const void *in, void *outv) {
        if (!M) return copy(outv, in);
        launches += 2;
        return zilu_apply(M, 'N', in, outv);
    };
    do {
        if (ws_alloc(c, &r, es * n) || ws_alloc(c, &p, es * n) || ws_alloc(c, &Ap, es * n) || ws_alloc(c, &z, es * n)) {
            st = cuda_fail(cudaGetLastError(), "complex cg workspace");
            break;
        }
        if ((st = copy(r, b))) break;
        if ((st = spmv(x, r, -1, 1))) break;   // r = b - A x
        if ((st = precond(r, z))) break;
        if ((st = copy(p, z))) break;
        Z zr, nzr;
        if ((st = dotc(r, z, zr))) break;
        it = 1;
        for (;;) {
            if ((st = spmv(p, Ap, 1, 0))) break;
            it++;
            if ((st = dotc(p, Ap, nzr))) break;
            const Z a = zr / nzr;
            if ((st = axpy(a, p, x))) break;
            if ((st = axpy(-a, Ap, r))) break;
            R nr[1];
            if ((st = zdot<R>(c, 2, n, r, r, nr, 0))) break;
            launches++;
            rn = nr[0];
            if (it >= max_iter || rn < (R)tol || rn != rn) break;
            if ((st = precond(r, z))) break;
            if ((st = dotc(r, z, nzr))) break;
            const Z bt = nzr / zr;
            const R bs[2] = {bt.real(), bt.imag()};
            if ((st = zscal<R>(c, n, bs, p))) break;
            launches++;
            if ((st = axpy(Z(1, 0), z, p))) break;
            zr = nzr;
        }
    } while (0);
    ws_free(c, r);
    ws_free(c, p);
    ws_free(c, Ap);
    ws_free(c, z);
    if (info) {
        info->iterations = it;
        info->outer = 0;
        info->residual = rn;
        info->true_residual = -1;
        info->kernel_launches = launches;
    }
    return st;   // as the reference's solve_cg: the iteration limit is not an error
}

// netlib zrotg (before 3.10) and LAPACK zrot (c real, s complex): [c s; -conj(s) c] [a; b] = [r; 0]
template <typename R>
static void zrotg_h(std::complex<R> &ca, std::complex<R> cb, R &c, std::complex<R> &s) {
    using Z = std::complex<R>;
    if (std::abs(ca) == R(0)) {
        c = 0;
        s = Z(1, 0);
        ca = cb;
        return;
    }
    const R scale = std::abs(ca) + std::abs(cb);
    const R p = std::abs(ca / scale), q = std::abs(cb / scale);
    const R norm = scale * std::sqrt(p * p + q * q);
    const Z alpha = ca / std::abs(ca);
    c = std::abs(ca) / norm;
    s = alpha * std::conj(cb) / norm;
    ca = alpha * norm;
}
template <typename R>
static void zrot_h(std::complex<R> &x, std::complex<R> &y, R c, std::complex<R> s) {
    const std::complex<R> t = c * x + s * y;
    y = c * y - std::conj(s) * x;
    x = t;
}

// The loop of solve_gmres (hex/solvers/hala_solvers_gmres.hpp:127-230), left preconditioned, one
// classical Gram-Schmidt pass, Givens rotations and the packed triangular solve on the host; tol on
// the preconditioned residual estimate, max_iter restarts.  The projection coefficients are W^T r
// without conjugation, as krylov_project computes them (gemv 'T', :47-50 and :67-72): on complex
// data the basis is orthogonal in the bilinear form x^T y, not the Hermitian one, and the estimate
// can differ from the true residual; the reference's own complex tests (real-valued data,
// tests/solvers_tests.hpp:105-137) do not see the difference.
template <typename R>
static int zgmres_run(hgb_ctx *c, hgb_csr *A, hgb_zilu *M, int restart, const void *b, void *x, double tol,
                      int max_iter, hgb_solve_info *info) {
    using Z = std::complex<R>;
    const int n = csr_rows(A);
    const size_t es = sizeof(Z);
    char *t = nullptr, *r = nullptr, *W = nullptr;
    int st = HGB_OK, total = 0, outer = 0;
    R inner_res = 0, outer_res = (R)tol + 1;
    long long launches = 0;
    auto col = [&](int j) { return W + (size_t)j * n * es; };
    auto copy = [&](void *dst, const void *src) {
        return cudaMemcpyAsync(dst, src, es * n, cudaMemcpyDeviceToDevice, c->stream) == cudaSuccess
                   ? HGB_OK
                   : cuda_fail(cudaGetLastError(), "complex gmres");
    };
    auto spmv = [&](const void *in, void *outv, R alpha, R beta) {
        const R a[2] = {alpha, 0}, bb[2] = {beta, 0};
        launches++;
        return zspmv<R>(c, 'N', n, n, csr_pntr(A), csr_indx(A), csr_vals(A), a, in, bb, outv, nullptr);
    };
    auto precond = [&](const void *in, void *outv) {
        if (!M) return copy(outv, in);
        launches += 2;
        return zilu_apply(M, 'N', in, outv);
    };
    auto nrm2 = [&](const void *u, R &out) {
        R v[1];
        const int e = zdot<R>(c, 2, n, u, u, v, 0);
        out = v[0];
        launches++;
        return e;
    };
    auto scal = [&](Z a, void *u) {
        const R v[2] = {a.real(), a.imag()};
        launches++;
        return zscal<R>(c, n, v, u);
    };
    auto axpy = [&](Z a, const void *u, void *v) {
        const R w[2] = {a.real(), a.imag()};
        launches++;
        return zaxpy<R>(c, n, w, u, v);
    };
    do {
        if (ws_alloc(c, &t, es * n) || ws_alloc(c, &r, es * n) || ws_alloc(c, &W, es * (size_t)n * restart)) {
            st = cuda_fail(cudaGetLastError(), "complex gmres workspace");
            break;
        }
        std::vector<Z> H, S, Zc;
        std::vector<R> C;
        while (outer_res > (R)tol && outer < max_iter) {
            H.clear();
            S.clear();
            C.clear();
            Zc.clear();
            if ((st = copy(t, b))) break;
            if ((st = spmv(x, t, -1, 1))) break;
            if ((st = precond(t, r))) break;
            total++;
            if ((st = nrm2(r, inner_res))) break;
            if ((st = scal(Z(R(1) / inner_res, 0), r))) break;
            Zc.push_back(Z(inner_res, 0));
            if ((st = copy(col(0), r))) break;
            int inner = 0;
            while (inner_res > (R)tol && inner < restart) {
                if ((st = spmv(r, t, 1, 0))) break;
                if ((st = precond(t, r))) break;
                total++;
                std::vector<Z> cf(inner + 1);
                for (int j = 0; j <= inner && !st; j++) {   // the projection: cf = W^T r, then r -= W cf
                    R v[2];
                    st = zdot<R>(c, 1, n, col(j), r, v, 0);
                    launches++;
                    cf[j] = Z(v[0], v[1]);
                }
                for (int j = 0; j <= inner && !st; j++) st = axpy(-cf[j], col(j), r);
                if (st) break;
                R nrm;
                if ((st = nrm2(r, nrm))) break;
                if ((st = scal(Z(R(1) / nrm, 0), r))) break;
                for (int i = 0; i < inner; i++) zrot_h(cf[i], cf[i + 1], C[i], S[i]);
                R ic;
                Z is;
                zrotg_h(cf[inner], Z(nrm, 0), ic, is);
                H.insert(H.end(), cf.begin(), cf.end());
                S.push_back(is);
                C.push_back(ic);
                inner_res = std::abs(S.back() * Zc.back());
                inner++;
                if (inner_res > (R)tol && inner < restart) {
                    if ((st = copy(col(inner), r))) break;
                    Zc.push_back(Z(0, 0));
                    zrot_h(Zc[inner - 1], Zc[inner], C.back(), S.back());
                }
            }
            if (st) break;
            if (!H.empty()) {   // tpsv('U', 'N', 'N') on the packed factor, then x += W Z
                const int nz = (int)Zc.size();
                long kk = (long)nz * (nz + 1) / 2 - 1;
                for (int j = nz - 1; j >= 0; j--) {
                    if (Zc[j] != Z(0, 0)) {
                        Zc[j] /= H[kk];
                        const Z tt = Zc[j];
                        long q = kk - 1;
                        for (int i = j - 1; i >= 0; i--, q--) Zc[i] -= tt * H[q];
                    }
                    kk -= j + 1;
                }
                for (int j = 0; j < nz && !st; j++) st = axpy(Zc[j], col(j), x);
                if (st) break;
            }
            outer++;
            outer_res = inner_res;
        }
    } while (0);
    ws_free(c, t);
    ws_free(c, r);
    ws_free(c, W);
    if (info) {
        info->iterations = total;
        info->outer = outer;
        info->residual = outer_res;
        info->true_residual = -1;
        info->kernel_launches = launches;
    }
    return st;   // as the reference's solve_gmres: the restart limit is not an error
}

int zcg_solve(hgb_ctx *c, hgb_csr *A, hgb_zilu *M, const void *b, void *x, double tol, int max_iter,
              hgb_solve_info *info) {
    if (M && zilu_rsize(M) != (csr_dtype(A) == HGB_C128 ? 8 : 4)) return fail(HGB_ERR_ARG, "complex cg: preconditioner precision");
    DeviceGuard g(c->device);
    return csr_dtype(A) == HGB_C128 ? zcg_run<double>(c, A, M, b, x, tol, max_iter, info)
                                    : zcg_run<float>(c, A, M, b, x, tol, max_iter, info);
}

int zgmres_solve(hgb_ctx *c, hgb_csr *A, hgb_zilu *M, int restart, const void *b, void *x, double tol, int max_iter,
                 hgb_solve_info *info) {
    if (M && zilu_rsize(M) != (csr_dtype(A) == HGB_C128 ? 8 : 4)) return fail(HGB_ERR_ARG, "complex gmres: preconditioner precision");
    DeviceGuard g(c->device);
    return csr_dtype(A) == HGB_C128 ? zgmres_run<double>(c, A, M, restart, b, x, tol, max_iter, info)
                                    : zgmres_run<float>(c, A, M, restart, b, x, tol, max_iter, info);
}

template int zdot<double>(hgb_ctx *, int, int, const void *, const void *, double *, int);
template int zdot<float>(hgb_ctx *, int, int, const void *, const void *, float *, int);
template int zaxpy<double>(hgb_ctx *, int, const double *, const void *, void *);
template int zaxpy<float>(hgb_ctx *, int, const float *, const void *, void *);
template int zscal<double>(hgb_ctx *, int, const double *, void *);
template int zscal<float>(hgb_ctx *, int, const float *, void *);

}  // namespace hgb
