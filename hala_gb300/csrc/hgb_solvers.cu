// Fused Krylov solvers over the SpMV / ILU kernels.
//
// CG / PCG follow solve_cg_core (hex/solvers/hala_solvers_cg.hpp:92-156) step for step, but the
// scalars never leave the device: <p,Ap> is reduced in the SpMV epilogue, ||r||^2 in the x/r
// update, and the convergence decision is taken on the device.  One iteration is six launches
// (SpMV+dot, update+norm, L solve, U solve, <r,z>, p update); ITERS_PER_GRAPH iterations are
// captured once into a CUDA graph and replayed, every launch of an iteration after convergence
// being a no-op, so the host synchronises once per graph replay instead of three times per
// iteration as the reference does (cublasDdot / cublasDnrm2 in host pointer mode).
#include "hgb_internal.cuh"
#include "hgb_kernels.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace hgb {

constexpr int kItersPerGraph = 16;

template <typename X>
__global__ void cg_update_kernel(long n, const SolverScalars *__restrict__ s_in, SolverScalars *s,
                                 const X *__restrict__ p, const X *__restrict__ Ap, X *__restrict__ x,
                                 X *__restrict__ r, double *partials, unsigned *counter) {
    if (s_in->done) return;
    // a = <r,z> / <p,Ap>; x += a p; r -= a Ap  (axpy(a,p,x), axpy(-a,Ap,r))
    const X a = (X)(s_in->zr / s_in->pap);
    const X ma = -a;
    double acc[1] = {0.0};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        x[i] = add_rn(x[i], mul_rn(a, p[i]));
        X ri = add_rn(r[i], mul_rn(ma, Ap[i]));
        r[i] = ri;
        acc[0] += (double)ri * (double)ri;
    }
    grid_sum<1>(acc, partials, counter, [&](double (&v)[1]) {
        s->rr = v[0];
        s->it += 1;
        s->done = (s->it >= s->max_iter) || (v[0] < s->tol2) || !(v[0] == v[0]);
    });
}

template <typename X>
__global__ void cg_rz_kernel(long n, SolverScalars *s, const X *__restrict__ r, const X *__restrict__ z,
                             double *partials, unsigned *counter, int init) {
    if (!init && s->done) return;
    double acc[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        acc[0] += (double)r[i] * (double)z[i];
        if (init) acc[1] += (double)r[i] * (double)r[i];
    }
    grid_sum<2>(acc, partials, counter, [&](double (&v)[2]) {
        s->nzr = s->zr;      // previous <r,z>, used by the p update
        s->zr = v[0];
        if (init) {
            s->rr = v[1];
            s->r0 = sqrt(v[1]);
            if (s->rel > 0.0) {
                double t = s->rel * s->r0;
                s->tol2 = fmax(s->tol2, t * t);
            }
        }
    });
}

// p = (zr_new / zr_old) p + z   (scal(a, p); axpy(1, z, p))
template <typename X>
__global__ void cg_p_kernel(long n, const SolverScalars *__restrict__ s, X *__restrict__ p, const X *__restrict__ z) {
    if (s->done) return;
    const X bta = (X)(s->zr / s->nzr);
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        p[i] = add_rn(mul_rn(bta, p[i]), z[i]);
}

__global__ void cg_init_kernel(SolverScalars *s, double tol2, double rel, int max_iter) {
    s->it = 1;
    s->done = 0;
    s->max_iter = max_iter;
    s->tol2 = tol2;
    s->rel = rel;
    s->zr = 0.0;
    s->nzr = 0.0;
    s->pap = 0.0;
    s->rr = 0.0;
}

template <typename X>
__global__ void copy_kernel(long n, const X *__restrict__ a, X *__restrict__ b) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) b[i] = a[i];
}

__global__ void f64_to_f32_kernel(long n, const double *__restrict__ a, float *__restrict__ b) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) b[i] = (float)a[i];
}

__global__ void add_f32_to_f64_kernel(long n, const float *__restrict__ d, double *__restrict__ x) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) x[i] += (double)d[i];
}

__global__ void zero_f32_kernel(long n, float *d) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) d[i] = 0.0f;
}

// r = b - A x in FP64 and ||r||^2 -> result slot (the refinement residual)
__global__ void residual_norm_kernel(long n, const double *__restrict__ r, double *partials, unsigned *counter,
                                     double *out) {
    double acc[1] = {0.0};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        acc[0] += r[i] * r[i];
    grid_sum<1>(acc, partials, counter, [&](double (&v)[1]) { *out = v[0]; });
}

static inline int ew_grid(hgb_ctx *c, long n) {
    return std::max(1, (int)std::min<long>((n + 255) / 256, (long)c->num_sms * 4));
}

// Workspace of one fused CG run (X = vector type).
template <typename X>
struct CgWork {
    X *r = nullptr, *z = nullptr, *p = nullptr, *Ap = nullptr;
    int alloc(long n, bool need_z) {
        size_t b = sizeof(X) * (size_t)n;
        if (cudaMalloc(&r, b) || cudaMalloc(&p, b) || cudaMalloc(&Ap, b) || (need_z && cudaMalloc(&z, b)))
            return cuda_fail(cudaErrorMemoryAllocation, "cg workspace");
        return HGB_OK;
    }
    void release() {
        cudaFree(r);
        cudaFree(z);
        cudaFree(p);
        cudaFree(Ap);
    }
};

template <typename V, typename X>
static int spmv_A(hgb_ctx *c, hgb_csr *A, X alpha, const X *x, X beta, X *y, double *dot, const int *skip,
                  bool trans = false) {
    if (trans) return spmv_t_fused_launch<V>(A, alpha, x, beta, y, x, dot, skip);
    return spmv_n_launch<V>(c, csr_rows(A), csr_pntr(A), csr_indx(A), (const V *)csr_vals(A), alpha, x, beta, y, dot,
                            skip);
}
template <>
int spmv_A<uint16_t, float>(hgb_ctx *c, hgb_csr *A, float alpha, const float *x, float beta, float *y, double *dot,
                           const int *skip, bool trans) {
    if (trans) return fail(HGB_ERR_UNSUPPORTED, "transposed product of a bf16 matrix");
    return spmv_n_launch<uint16_t>(c, csr_rows(A), csr_pntr(A), csr_indx(A), (const uint16_t *)csr_vals(A), alpha, x,
                                   beta, y, dot, skip);
}

// One CG iteration: the launches captured into the graph.
template <typename V, typename X>
static int cg_iteration(hgb_ctx *c, hgb_csr *A, hgb_ilu *M, CgWork<X> &w, X *x, long n, bool trans) {
    SolverScalars *s = c->scal;
    const int *done = &s->done;
    HGB_TRY(spmv_A<V, X>(c, A, X(1), w.p, X(0), w.Ap, &s->pap, done, trans));
    cg_update_kernel<X><<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, s, s, w.p, w.Ap, x, w.r, c->partials, c->counter);
    X *z = M ? w.z : w.r;
    if (M) HGB_TRY(ilu_apply_internal(M, trans ? 'T' : 'N', w.r, w.z, done));
    cg_rz_kernel<X><<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, s, w.r, z, c->partials, c->counter, 0);
    cg_p_kernel<X><<<ew_grid(c, n), 256, 0, c->stream>>>(n, s, w.p, z);
    return launch_check("cg iteration");
}

// Runs CG on (A, M) for b -> x (x holds the initial guess).  zero_x0: skip r = b - A x.
// kernels per captured CG iteration: SpMV+dot, update+norm, [L solve, U solve], <r,z>, p update
static int cg_launches_per_iter(bool precond) { return precond ? 6 : 4; }

template <typename V, typename X>
static int cg_run(hgb_ctx *c, hgb_csr *A, hgb_ilu *M, const X *b, X *x, double tol2, double rel, int max_iter,
                  bool zero_x0, int *iters, double *rr_out, long long *launches, bool trans = false) {
    const long n = csr_rows(A);
    CaptureStream cs(c);
    CgWork<X> w;
    int st = w.alloc(n, M != nullptr);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    SolverScalars hs{};
    do {
        if (st) break;
        SolverScalars *s = c->scal;
        cg_init_kernel<<<1, 1, 0, c->stream>>>(s, tol2, rel, max_iter);
        *launches += 1 + (zero_x0 ? 0 : 1) + (M ? 2 : 0) + 2;   // init, SpMV, L/U solves, copy, <r,z>
        // r = b - A x  (r = b; r += -1 * A x)
        if (cudaMemcpyAsync(w.r, b, sizeof(X) * n, cudaMemcpyDeviceToDevice, c->stream)) { st = cuda_fail(cudaGetLastError(), "cg"); break; }
        if (trans && (st = csr_ensure_transpose(A))) break;
        if (!zero_x0 && (st = spmv_A<V, X>(c, A, X(-1), x, X(1), w.r, nullptr, nullptr, trans))) break;
        X *z = M ? w.z : w.r;
        if (M && (st = ilu_apply_internal(M, trans ? 'T' : 'N', w.r, w.z, nullptr))) break;
        copy_kernel<X><<<ew_grid(c, n), 256, 0, c->stream>>>(n, z, w.p);
        cg_rz_kernel<X><<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, s, w.r, z, c->partials, c->counter, 1);
        if ((st = launch_check("cg init"))) break;
        // capture ITERS_PER_GRAPH iterations
        cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
        if (cudaStreamBeginCapture(c->stream, mode)) { st = cuda_fail(cudaGetLastError(), "begin capture"); break; }
        for (int k = 0; k < kItersPerGraph && !st; k++) st = cg_iteration<V, X>(c, A, M, w, x, n, trans);
        cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
        if (st) break;
        if (ce != cudaSuccess) { st = cuda_fail(ce, "end capture"); break; }
        if (cudaGraphInstantiate(&exec, graph, 0)) { st = cuda_fail(cudaGetLastError(), "graph instantiate"); break; }
        for (;;) {
            if (cudaGraphLaunch(exec, c->stream)) { st = cuda_fail(cudaGetLastError(), "graph launch"); break; }
            *launches += (long long)kItersPerGraph * cg_launches_per_iter(M != nullptr);
            if (cudaMemcpyAsync(c->host_result, s, sizeof(SolverScalars), cudaMemcpyDeviceToHost, c->stream)) { st = cuda_fail(cudaGetLastError(), "cg"); break; }
            if (cudaStreamSynchronize(c->stream)) { st = cuda_fail(cudaGetLastError(), "cg sync"); break; }
            memcpy(&hs, c->host_result, sizeof(SolverScalars));
            if (hs.done) break;
        }
    } while (0);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    w.release();
    if (st) return st;
    HGB_TRY(collect_dev_error(c));
    *iters = hs.it;
    *rr_out = hs.rr;
    return HGB_OK;
}

static int true_residual(hgb_ctx *c, hgb_csr *A64, const double *b, const double *x, double *r, double *res,
                         long long *launches, bool trans = false) {
    *launches += 2;
    const long n = csr_rows(A64);
    HGB_CUDA(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
    if (trans) HGB_TRY(csr_ensure_transpose(A64));
    HGB_TRY(spmv_A<double, double>(c, A64, -1.0, x, 1.0, r, nullptr, nullptr, trans));
    residual_norm_kernel<<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, r, c->partials, c->counter, c->result);
    HGB_TRY(launch_check("residual_norm_kernel"));
    HGB_CUDA(cudaMemcpyAsync(c->host_result, c->result, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    *res = sqrt(c->host_result[0]);
    return HGB_OK;
}

}  // namespace hgb

using namespace hgb;

extern "C" {

int hgb_cg_solve(hgb_ctx *c, hgb_csr *A, hgb_ilu *M, const void *b, void *x, double tol, int max_iter,
                 hgb_solve_info *info) {
    return hgb_cg_solve_op(c, A, M, 'N', b, x, tol, max_iter, info);
}

int hgb_cg_solve_op(hgb_ctx *c, hgb_csr *A, hgb_ilu *M, char trans, const void *b, void *x, double tol, int max_iter,
                    hgb_solve_info *info) {
    if (!c || !A || !b || !x) return fail(HGB_ERR_ARG, "cg_solve: bad arguments");
    const bool tr = (trans == 'T' || trans == 't' || trans == 'C' || trans == 'c');
    if (!tr && trans != 'N' && trans != 'n') return fail(HGB_ERR_ARG, "cg_solve: trans '%c'", trans);
    if (csr_rows(A) != csr_cols(A)) return fail(HGB_ERR_ARG, "cg_solve: square matrix required");
    if (max_iter < 1) return fail(HGB_ERR_ARG, "cg_solve: max_iter < 1");
    DeviceGuard g(c->device);
    hgb_dtype dt = csr_dtype(A);
    if (M) {
        if (ilu_n(M) != csr_rows(A)) return fail(HGB_ERR_ARG, "cg_solve: preconditioner size");
        bool ok = (dt == HGB_F64) ? (ilu_store(M) == HGB_F64) : (ilu_store(M) != HGB_F64);
        if (!ok) return fail(HGB_ERR_ARG, "cg_solve: preconditioner precision does not match the matrix");
    }
    int it = 0;
    double rr = 0.0;
    double tol2 = tol * tol;
    long long launches = 0;
    int st;
    if (dt == HGB_F64) st = cg_run<double, double>(c, A, M, (const double *)b, (double *)x, tol2, 0.0, max_iter, false, &it, &rr, &launches, tr);
    else if (dt == HGB_F32) st = cg_run<float, float>(c, A, M, (const float *)b, (float *)x, tol2, 0.0, max_iter, false, &it, &rr, &launches, tr);
    else st = cg_run<uint16_t, float>(c, A, M, (const float *)b, (float *)x, tol2, 0.0, max_iter, false, &it, &rr, &launches, tr);
    if (st) return st;
    if (info) {
        info->iterations = it;
        info->outer = 0;
        info->residual = sqrt(rr);
        info->true_residual = -1.0;
        info->kernel_launches = launches;
    }
    return HGB_OK;
}

int hgb_ir_pcg_solve(hgb_ctx *c, hgb_csr *A64, hgb_csr *Ai, hgb_ilu *Mi, const double *b, double *x, double tol,
                     double inner_rtol, int max_inner, int max_outer, hgb_solve_info *info) {
    return hgb_ir_pcg_solve_op(c, A64, Ai, Mi, 'N', b, x, tol, inner_rtol, max_inner, max_outer, info);
}

int hgb_ir_pcg_solve_op(hgb_ctx *c, hgb_csr *A64, hgb_csr *Ai, hgb_ilu *Mi, char trans, const double *b, double *x,
                        double tol, double inner_rtol, int max_inner, int max_outer, hgb_solve_info *info) {
    if (!c || !A64 || !Ai || !b || !x) return fail(HGB_ERR_ARG, "ir_pcg: bad arguments");
    const bool tr = (trans == 'T' || trans == 't' || trans == 'C' || trans == 'c');
    if (!tr && trans != 'N' && trans != 'n') return fail(HGB_ERR_ARG, "ir_pcg: trans '%c'", trans);
    if (tr && csr_dtype(Ai) == HGB_BF16) return fail(HGB_ERR_UNSUPPORTED, "ir_pcg: transposed solve with a bf16 matrix");
    if (csr_dtype(A64) != HGB_F64) return fail(HGB_ERR_ARG, "ir_pcg: the outer matrix must be F64");
    if (csr_dtype(Ai) == HGB_F64) return fail(HGB_ERR_ARG, "ir_pcg: the inner matrix must be F32 or BF16");
    if (Mi && ilu_store(Mi) == HGB_F64) return fail(HGB_ERR_ARG, "ir_pcg: the inner preconditioner must store F32 or BF16");
    const long n = csr_rows(A64);
    if (csr_rows(Ai) != n || csr_cols(A64) != n) return fail(HGB_ERR_ARG, "ir_pcg: sizes");
    if (max_inner < 1 || max_outer < 0 || !(inner_rtol > 0.0)) return fail(HGB_ERR_ARG, "ir_pcg: limits");
    DeviceGuard g(c->device);
    double *r64 = nullptr;
    float *r32 = nullptr, *d32 = nullptr;
    int st = HGB_OK;
    int total = 0, outer = 0;
    double res = 0.0;
    long long launches = 0;
    do {
        if (cudaMalloc(&r64, sizeof(double) * n) || cudaMalloc(&r32, sizeof(float) * n) || cudaMalloc(&d32, sizeof(float) * n)) {
            st = cuda_fail(cudaErrorMemoryAllocation, "ir_pcg workspace");
            break;
        }
        for (;;) {
            if ((st = true_residual(c, A64, b, x, r64, &res, &launches, tr))) break;
            if (res < tol || outer >= max_outer || !(res == res)) break;
            f64_to_f32_kernel<<<ew_grid(c, n), 256, 0, c->stream>>>(n, r64, r32);
            zero_f32_kernel<<<ew_grid(c, n), 256, 0, c->stream>>>(n, d32);
            int it = 0;
            double rr = 0.0;
            launches += 3;   // residual cast, zero, update
            // reduce this sweep's residual only as far as the target needs (with a factor 2 of
            // margin), never by less than inner_rtol: the last sweep stops early
            const double rel = std::min(0.5, std::max(inner_rtol, 0.5 * tol / res));
            if (csr_dtype(Ai) == HGB_F32)
                st = cg_run<float, float>(c, Ai, Mi, r32, d32, 0.0, rel, max_inner, true, &it, &rr, &launches, tr);
            else
                st = cg_run<uint16_t, float>(c, Ai, Mi, r32, d32, 0.0, rel, max_inner, true, &it, &rr, &launches);
            if (st) break;
            total += it;
            add_f32_to_f64_kernel<<<ew_grid(c, n), 256, 0, c->stream>>>(n, d32, x);
            if ((st = launch_check("ir update"))) break;
            outer++;
        }
    } while (0);
    cudaFree(r64);
    cudaFree(r32);
    cudaFree(d32);
    if (st) return st;
    if (info) {
        info->iterations = total;
        info->outer = outer;
        info->residual = res;
        info->true_residual = res;
        info->kernel_launches = launches;
    }
    if (!(res < tol)) return fail(HGB_ERR_NOT_CONVERGED, "ir_pcg: ||b-Ax|| = %g after %d sweeps (tol %g)", res, outer, tol);
    return HGB_OK;
}

}  // extern "C"

// ===================================================================== GMRES ===========
namespace hgb {

// r -= W c (k columns) and ||r||^2 -> out   (krylov_project's gemv 'N' fused with norm2)
__global__ void cgs_update_kernel(long n, int k, const double *__restrict__ W, const double *__restrict__ cf,
                                  double *__restrict__ r, double *partials, unsigned *counter, double *out) {
    double acc[1] = {0.0};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double ri = r[i];
        for (int j = 0; j < k; j++) ri = __dadd_rn(ri, __dmul_rn(-cf[j], W[(long)j * n + i]));
        r[i] = ri;
        acc[0] += ri * ri;
    }
    grid_sum<1>(acc, partials, counter, [&](double (&v)[1]) { *out = v[0]; });
}

__global__ void scale_copy_kernel(long n, double a, double *__restrict__ r, double *__restrict__ wcol) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double v = r[i] * a;
        r[i] = v;
        if (wcol) wcol[i] = v;
    }
}

static void rotg(double &a, double &b, double &c, double &s) {
    double roe = (std::fabs(a) > std::fabs(b)) ? a : b;
    double scale = std::fabs(a) + std::fabs(b), r, z;
    if (scale == 0.0) { c = 1.0; s = 0.0; r = 0.0; z = 0.0; }
    else {
        r = scale * std::sqrt((a / scale) * (a / scale) + (b / scale) * (b / scale));
        if (roe < 0.0) r = -r;
        c = a / r;
        s = b / r;
        z = 1.0;
        if (std::fabs(a) > std::fabs(b)) z = s;
        if (std::fabs(b) >= std::fabs(a) && c != 0.0) z = 1.0 / c;
    }
    a = r;
    b = z;
}

static void rot(double &x, double &y, double c, double s) {
    double t = c * x + s * y;
    y = c * y - s * x;
    x = t;
}

}  // namespace hgb

extern "C" int hgb_gmres_solve(hgb_ctx *c, hgb_csr *A, hgb_ilu *M, int restart, const void *bv, void *xv, double tol,
                               int max_iter, hgb_solve_info *info) {
    if (!c || !A || !bv || !xv || restart < 1 || restart > 64) return fail(HGB_ERR_ARG, "gmres: bad arguments (restart 1..64)");
    if (csr_dtype(A) != HGB_F64) return fail(HGB_ERR_UNSUPPORTED, "gmres: F64 only");
    if (M && ilu_store(M) != HGB_F64) return fail(HGB_ERR_ARG, "gmres: preconditioner must be F64");
    const long n = csr_rows(A);
    const double *b = (const double *)bv;
    double *x = (double *)xv;
    DeviceGuard g(c->device);
    double *t = nullptr, *r = nullptr, *W = nullptr, *dc = nullptr;
    int st = HGB_OK;
    int total = 0, outer = 0;
    long long launches = 0;
    double inner_res = 0.0, outer_res = tol + 1.0;
    std::vector<double> H, S, C, Z, cf(restart + 2);
    double *hbuf = c->host_result;   // pinned, >= 8 doubles; coefficients go through dc
    std::vector<double> hcf(restart + 2);
    do {
        if (cudaMalloc(&t, sizeof(double) * n) || cudaMalloc(&r, sizeof(double) * n) ||
            cudaMalloc(&W, sizeof(double) * n * restart) || cudaMalloc(&dc, sizeof(double) * (restart + 2))) {
            st = cuda_fail(cudaErrorMemoryAllocation, "gmres workspace");
            break;
        }
        auto precon = [&](const double *in, double *out) -> int {
            if (M) return ilu_apply_internal(M, 'N', in, out, nullptr);
            return cudaMemcpyAsync(out, in, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream) ? HGB_ERR_CUDA : HGB_OK;
        };
        auto norm_sync = [&](const double *v, double *out) -> int {
            residual_norm_kernel<<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, v, c->partials, c->counter, c->result);
            HGB_CUDA(cudaMemcpyAsync(hbuf, c->result, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
            HGB_CUDA(cudaStreamSynchronize(c->stream));
            *out = std::sqrt(hbuf[0]);
            return HGB_OK;
        };
        while (outer_res > tol && outer < max_iter) {
            H.clear(); S.clear(); C.clear(); Z.clear();
            // t = b - A x ; r = P^-1 t
            if (cudaMemcpyAsync(t, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream)) { st = HGB_ERR_CUDA; break; }
            if ((st = spmv_A<double, double>(c, A, -1.0, x, 1.0, t, nullptr, nullptr))) break;
            if ((st = precon(t, r))) break;
            total++;
            launches += 1 + (M ? 2 : 0) + 2;
            if ((st = norm_sync(r, &inner_res))) break;
            scale_copy_kernel<<<ew_grid(c, n), 256, 0, c->stream>>>(n, 1.0 / inner_res, r, W);
            Z.push_back(inner_res);
            int k = 0;
            while (inner_res > tol && k < restart) {
                if ((st = spmv_A<double, double>(c, A, 1.0, r, 0.0, t, nullptr, nullptr))) break;
                if ((st = precon(t, r))) break;
                total++;
                launches += 1 + (M ? 2 : 0) + 3;
                // krylov_project: cf = W^T r (k+1 columns) ; r -= W cf ; nrm = ||r||
                if ((st = hgb_gemv_f64(c, 'T', (int)n, k + 1, 1.0, W, r, 0.0, dc))) break;
                cgs_update_kernel<<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, k + 1, W, dc, r, c->partials,
                                                                                    c->counter, dc + restart + 1);
                if ((st = launch_check("cgs_update_kernel"))) break;
                if (cudaMemcpyAsync(hcf.data(), dc, sizeof(double) * (restart + 2), cudaMemcpyDeviceToHost, c->stream) ||
                    cudaStreamSynchronize(c->stream)) { st = cuda_fail(cudaGetLastError(), "gmres"); break; }
                double nrm = std::sqrt(hcf[restart + 1]);
                for (int j = 0; j <= k; j++) cf[j] = hcf[j];
                for (int i = 0; i < k; i++) rot(cf[i], cf[i + 1], C[i], S[i]);
                double beta = nrm, ic, is;
                rotg(cf[k], beta, ic, is);
                H.insert(H.end(), cf.begin(), cf.begin() + k + 1);
                S.push_back(is);
                C.push_back(ic);
                inner_res = std::fabs(S.back() * Z.back());
                k++;
                bool expand = (inner_res > tol) && (k < restart);
                scale_copy_kernel<<<ew_grid(c, n), 256, 0, c->stream>>>(n, 1.0 / nrm, r, expand ? W + (long)k * n : nullptr);
                if (expand) {
                    Z.push_back(0.0);
                    rot(Z[k - 1], Z[k], C.back(), S.back());
                }
            }
            if (st) break;
            if (!H.empty()) {
                // tpsv('U','N','N', nz, H, Z), column-oriented back substitution (packed upper)
                int nz = (int)Z.size();
                long kk = (long)nz * (nz + 1) / 2 - 1;
                for (int j = nz - 1; j >= 0; j--) {
                    if (Z[j] != 0.0) {
                        Z[j] /= H[kk];
                        double tt = Z[j];
                        long q = kk - 1;
                        for (int i = j - 1; i >= 0; i--, q--) Z[i] -= tt * H[q];
                    }
                    kk -= j + 1;
                }
                if (cudaMemcpyAsync(dc, Z.data(), sizeof(double) * nz, cudaMemcpyHostToDevice, c->stream)) { st = HGB_ERR_CUDA; break; }
                if ((st = hgb_gemv_f64(c, 'N', (int)n, nz, 1.0, W, dc, 1.0, x))) break;
                launches += 1;
                if (cudaStreamSynchronize(c->stream)) { st = cuda_fail(cudaGetLastError(), "gmres"); break; }
            }
            outer++;
            outer_res = inner_res;
        }
    } while (0);
    cudaFree(t);
    cudaFree(r);
    cudaFree(W);
    cudaFree(dc);
    if (st) return st;
    HGB_TRY(collect_dev_error(c));
    if (info) {
        info->iterations = total;
        info->outer = outer;
        info->residual = inner_res;
        info->true_residual = -1.0;
        info->kernel_launches = launches;
    }
    return HGB_OK;
}

// ========================================================== host-buffer (mixed) solve ====
extern "C" int hgb_mixed_cg_solve(hgb_ctx *c, int n, int nnz, const int *pntr_h, const int *indx_h, const double *vals_h,
                                  hgb_ilu *M, const double *b_h, double *x_h, double tol, int max_iter,
                                  hgb_solve_info *info) {
    if (!c || n <= 0 || nnz < 0 || !pntr_h || !indx_h || !vals_h || !b_h || !x_h) return fail(HGB_ERR_ARG, "mixed_cg: bad arguments");
    DeviceGuard g(c->device);
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    size_t op = 0, oi = op + al(sizeof(int) * (n + 1)), ov = oi + al(sizeof(int) * (size_t)nnz);
    size_t ob = ov + al(sizeof(double) * (size_t)nnz), ox = ob + al(sizeof(double) * n), total = ox + al(sizeof(double) * n);
    if (c->arena_bytes < total) {
        cudaFree(c->arena);
        c->arena = nullptr;
        c->arena_bytes = 0;
        HGB_CUDA(cudaMalloc(&c->arena, total));
        c->arena_bytes = total;
    }
    char *base = (char *)c->arena;
    int *dp = (int *)(base + op), *di = (int *)(base + oi);
    double *dv = (double *)(base + ov), *db = (double *)(base + ob), *dx = (double *)(base + ox);
    HGB_CUDA(cudaMemcpyAsync(dp, pntr_h, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, c->stream));
    HGB_CUDA(cudaMemcpyAsync(di, indx_h, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, c->stream));
    HGB_CUDA(cudaMemcpyAsync(dv, vals_h, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, c->stream));
    HGB_CUDA(cudaMemcpyAsync(db, b_h, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    HGB_CUDA(cudaMemcpyAsync(dx, x_h, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    hgb_csr *A = nullptr;
    HGB_TRY(hgb_csr_create(c, n, n, nnz, dp, di, dv, HGB_F64, &A));
    int st = hgb_cg_solve(c, A, M, db, dx, tol, max_iter, info);
    hgb_csr_destroy(A);
    if (st) return st;
    HGB_CUDA(cudaMemcpyAsync(x_h, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    return HGB_OK;
}

namespace hgb {
__global__ void f64_to_inner_kernel(long n, const double *__restrict__ a, float *f32, uint16_t *b16) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        float v = (float)a[i];
        if (f32) f32[i] = v;
        if (b16) {
            uint32_t u = __float_as_uint(v);
            b16[i] = ((u & 0x7fffffffu) > 0x7f800000u) ? (uint16_t)((u >> 16) | 0x40u)
                                                      : (uint16_t)((u + 0x7fffu + ((u >> 16) & 1u)) >> 16);
        }
    }
}
}  // namespace hgb

extern "C" int hgb_mixed_ir_pcg_solve(hgb_ctx *c, int n, int nnz, const int *pntr_h, const int *indx_h,
                                      const double *vals_h, hgb_ilu *Mi, const double *b_h, double *x_h,
                                      double tol, double inner_rtol, int max_inner, int max_outer,
                                      hgb_solve_info *info) {
    if (!c || n <= 0 || nnz < 0 || !pntr_h || !indx_h || !vals_h || !b_h || !x_h || !Mi)
        return fail(HGB_ERR_ARG, "mixed_ir_pcg: bad arguments");
    if (ilu_store(Mi) == HGB_F64) return fail(HGB_ERR_ARG, "mixed_ir_pcg: the preconditioner must store F32 or BF16");
    DeviceGuard g(c->device);
    const bool bf16 = ilu_store(Mi) == HGB_BF16;
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    size_t op = 0, oi = op + al(sizeof(int) * (n + 1)), ov = oi + al(sizeof(int) * (size_t)nnz);
    size_t ow = ov + al(sizeof(double) * (size_t)nnz), ob = ow + al(sizeof(float) * (size_t)nnz);
    size_t ox = ob + al(sizeof(double) * n), total = ox + al(sizeof(double) * n);
    if (c->arena_bytes < total) {
        cudaFree(c->arena);
        c->arena = nullptr;
        c->arena_bytes = 0;
        HGB_CUDA(cudaMalloc(&c->arena, total));
        c->arena_bytes = total;
    }
    char *base = (char *)c->arena;
    int *dp = (int *)(base + op), *di = (int *)(base + oi);
    double *dv = (double *)(base + ov), *db = (double *)(base + ob), *dx = (double *)(base + ox);
    void *dw = base + ow;
    HGB_CUDA(cudaMemcpyAsync(dp, pntr_h, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, c->stream));
    HGB_CUDA(cudaMemcpyAsync(di, indx_h, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, c->stream));
    HGB_CUDA(cudaMemcpyAsync(dv, vals_h, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, c->stream));
    HGB_CUDA(cudaMemcpyAsync(db, b_h, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    HGB_CUDA(cudaMemcpyAsync(dx, x_h, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    f64_to_inner_kernel<<<ew_grid(c, nnz), 256, 0, c->stream>>>(nnz, dv, bf16 ? nullptr : (float *)dw,
                                                                bf16 ? (uint16_t *)dw : nullptr);
    HGB_TRY(launch_check("f64_to_inner_kernel"));
    hgb_csr *A64 = nullptr, *Ai = nullptr;
    HGB_TRY(hgb_csr_create(c, n, n, nnz, dp, di, dv, HGB_F64, &A64));
    int st = hgb_csr_create(c, n, n, nnz, dp, di, dw, bf16 ? HGB_BF16 : HGB_F32, &Ai);
    if (!st) st = hgb_ir_pcg_solve(c, A64, Ai, Mi, db, dx, tol, inner_rtol, max_inner, max_outer, info);
    hgb_csr_destroy(A64);
    hgb_csr_destroy(Ai);
    if (info) info->kernel_launches += 1;
    if (st && st != HGB_ERR_NOT_CONVERGED) return st;
    HGB_CUDA(cudaMemcpyAsync(x_h, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    return st;
}
