/*
 * hgb.h — C ABI of the GB300-native sparse Krylov path (libhgb.so, sm_103a kernels).
 *
 * This is the boundary the reference's GPU backend crosses today through cuSPARSE / cuBLAS
 * (gpu/hala_cuda_sparse_general.hpp, gpu/hala_cuda_sparse_triangular.hpp, gpu/hala_gpu_ilu.hpp,
 * gpu/hala_gpu_blas1.hpp).  Every entry point below replaces one of those library calls or one
 * of the reference objects built on them; the comment on each cites the reference interface.
 *
 * Conventions
 *  - All array arguments are DEVICE pointers on the context's device, unless a name says host.
 *  - CSR matrices use int32 row pointers (pntr[n+1]) and int32 column indices (indx[nnz]) with
 *    columns sorted ascending inside each row, zero-based (sparse/hala_sparse_utils.hpp:31-40).
 *  - Work is ordered on the context's stream; calls that return a host scalar synchronise it.
 *  - Return value: HGB_OK (0) or an hgb_status code; hgb_last_error() gives a message.  The C++
 *    layer (include/hala_gb/) turns non-zero codes into std::runtime_error, as the reference's
 *    check_cuda() does (gpu/hala_cuda_common.hpp:78-152).
 *  - Handles (context, matrix, ILU, triangular) are not safe for concurrent use from several
 *    host threads or streams; use one per stream.
 */
#ifndef HGB_H
#define HGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum hgb_status {
    HGB_OK = 0,
    HGB_ERR_ARG = 1,           /* invalid argument (size, pointer, trans/uplo/diag character)   */
    HGB_ERR_CSR = 2,           /* malformed CSR: pntr not monotone, column out of range or
                                  unsorted, or (ILU / triangular) a missing diagonal entry       */
    HGB_ERR_ZERO_PIVOT = 3,    /* ILU(0) met an exactly zero pivot (factor still produced)      */
    HGB_ERR_TIMEOUT = 4,       /* a bounded device-side wait gave up (result is not valid)      */
    HGB_ERR_NOT_CONVERGED = 5, /* solver stopped at its iteration limit above the tolerance     */
    HGB_ERR_CUDA = 6,          /* a CUDA runtime call failed                                    */
    HGB_ERR_ALLOC = 7,         /* device or host allocation failed                              */
    HGB_ERR_UNSUPPORTED = 8    /* combination not implemented (e.g. transpose on a bf16 matrix) */
} hgb_status;

/* Element types.  HGB_C128 / HGB_C64: complex, interleaved (real, imaginary) pairs of doubles /
 * floats, the layout of std::complex and cuDoubleComplex / cuComplex. */
typedef enum hgb_dtype { HGB_F64 = 0, HGB_F32 = 1, HGB_BF16 = 2, HGB_C128 = 3, HGB_C64 = 4 } hgb_dtype;

/* Arithmetic of the non-transposed SpMV (and of every solver product built on it).
 * HGB_SPMV_FUSED: one fused multiply-add per entry in column order (the default; within a few
 *   ulps of the row sum of the reference's loop; the FP64 product is about twice as fast on
 *   sm_103, whose FP64 pipe is narrow).
 * HGB_SPMV_EXACT: separately rounded multiply and add in column order, the arithmetic of
 *   sparse_gemv_array (sparse/hala_sparse_utils.hpp:104-112): bit-identical to the reference's
 *   CPU product. */
typedef enum hgb_spmv_mode { HGB_SPMV_FUSED = 0, HGB_SPMV_EXACT = 1 } hgb_spmv_mode;

typedef struct hgb_ctx hgb_ctx;
typedef struct hgb_csr hgb_csr;
typedef struct hgb_ilu hgb_ilu;
typedef struct hgb_tri hgb_tri;
typedef struct hgb_batch hgb_batch;

/* Outcome of a solve (the reference returns only the iteration count). */
typedef struct hgb_solve_info {
    int iterations;      /* reference convention: CG counts 1 + loop SpMVs (cg.hpp:125,130);
                            GMRES counts operator+preconditioner applications (gmres.hpp:176,189);
                            iterative refinement counts inner iterations                        */
    int outer;           /* refinement sweeps (IR) or restarts (GMRES); 0 for plain CG          */
    double residual;     /* last residual norm the stopping test saw                            */
    double true_residual;/* ||b - A x||_2 recomputed in FP64 at exit (IR only; else -1)         */
    long long kernel_launches; /* kernels this solve executed (graph-replayed launches included) */
} hgb_solve_info;

/* ------------------------------------------------------------------ library / errors ---- */
const char *hgb_status_string(int status);
const char *hgb_last_error(void);    /* thread-local message of the last failing call */
int hgb_version(void);               /* 10000*major + 100*minor + patch */

/* -------------------------------------------------- engine (gpu_engine, engine.hpp:47) --- */
/* gpu_engine(device) constructor, gpu/hala_gpu_engine.hpp:60 */
int hgb_ctx_create(int device, hgb_ctx **ctx);
int hgb_ctx_destroy(hgb_ctx *ctx);
/* gpu_engine::set_stream, gpu/hala_gpu_engine.hpp:86-90 (stream is a cudaStream_t) */
int hgb_ctx_set_stream(hgb_ctx *ctx, void *stream);
int hgb_ctx_synchronize(hgb_ctx *ctx);
/* SpMV arithmetic of this context (hgb_spmv_mode); applies to products issued after the call. */
int hgb_ctx_set_spmv_mode(hgb_ctx *ctx, int mode);
int hgb_ctx_get_spmv_mode(hgb_ctx *ctx, int *mode);

/* ------------------------------------------------------- BLAS-1 (gpu/hala_gpu_blas1.hpp) --- */
/* result: host pointer (synchronises) when result_on_device == 0, else device pointer.
 * dot: :179-198 (cublasXdot); nrm2: :102-121 (cublasXnrm2); axpy: :205-222; scal: :229-245;
 * copy (vcopy): :49-62.  alpha is a host scalar (the reference uses CUBLAS_POINTER_MODE_HOST). */
int hgb_dot_f64(hgb_ctx *ctx, int n, const double *x, const double *y, double *result,
                int result_on_device);
int hgb_dot_f32(hgb_ctx *ctx, int n, const float *x, const float *y, float *result,
                int result_on_device);
int hgb_nrm2_f64(hgb_ctx *ctx, int n, const double *x, double *result, int result_on_device);
int hgb_nrm2_f32(hgb_ctx *ctx, int n, const float *x, float *result, int result_on_device);
int hgb_axpy_f64(hgb_ctx *ctx, int n, double alpha, const double *x, double *y);
int hgb_axpy_f32(hgb_ctx *ctx, int n, float alpha, const float *x, float *y);
int hgb_scal_f64(hgb_ctx *ctx, int n, double alpha, double *x);
int hgb_scal_f32(hgb_ctx *ctx, int n, float alpha, float *x);
int hgb_copy_f64(hgb_ctx *ctx, int n, const double *x, double *y);
int hgb_copy_f32(hgb_ctx *ctx, int n, const float *x, float *y);
/* set_zero(gpu_engine, ...), gpu/hala_gpu_engine.hpp:336-352 */
int hgb_set_zero(hgb_ctx *ctx, size_t bytes, void *x);

/* ------------------------------------------------ dense gemv (gpu/hala_gpu_blas2.hpp:40) --- */
/* y = alpha * op(W) x + beta * y, W column-major m x k (ld = m), tall and skinny: the GMRES Krylov
 * project and combine, hex/solvers/hala_solvers_gmres.hpp:67-77, and the column sums of the batch
 * reductions (wax/hala_blas_extensions.hpp:246).  'T' accumulates in double. */
int hgb_gemv_f64(hgb_ctx *ctx, char trans, int m, int k, double alpha, const double *W,
                 const double *x, double beta, double *y);
int hgb_gemv_f32(hgb_ctx *ctx, char trans, int m, int k, float alpha, const float *W,
                 const float *x, float beta, float *y);
/* C = diag(x) A (side 'L') or A diag(x) (side 'R'), A and C m x k column-major, packed: the column
 * scalings of batch_axpy / batch_scal / batch_dot (dgmm(gpu_engine,...), gpu/hala_gpu_overloads.hpp,
 * called from wax/hala_blas_extensions.hpp:211-265).  C may alias A. */
int hgb_dgmm_f64(hgb_ctx *ctx, char side, int m, int k, const double *A, const double *x, double *C);
int hgb_dgmm_f32(hgb_ctx *ctx, char side, int m, int k, const float *A, const float *x, float *C);

/* ------------------------------------------ SpMV (sparse_gemv(gpu_engine,...), :408-419) --- */
/* y = alpha * op(A) x + beta * y; A is n_rows x n_cols CSR.  trans 'N', 'T' or 'C' (real: C==T).
 * beta == 0 does not read y.  'N' rows are summed sequentially in column order, with the context's
 * hgb_spmv_mode (HGB_SPMV_EXACT: no fused multiply-add, the arithmetic of sparse_gemv_array,
 * sparse/hala_sparse_utils.hpp:104-112).  'T' without a matrix handle scatters with atomics
 * (order not fixed). */
int hgb_spmv_f64(hgb_ctx *ctx, char trans, int n_rows, int n_cols, int nnz, const int *pntr,
                 const int *indx, const double *vals, double alpha, const double *x, double beta,
                 double *y);
int hgb_spmv_f32(hgb_ctx *ctx, char trans, int n_rows, int n_cols, int nnz, const int *pntr,
                 const int *indx, const float *vals, float alpha, const float *x, float beta,
                 float *y);
/* bf16 values (uint16 bit patterns), fp32 vectors, fp32 accumulation ('N' only) */
int hgb_spmv_bf16f32(hgb_ctx *ctx, char trans, int n_rows, int n_cols, int nnz, const int *pntr,
                     const int *indx, const uint16_t *vals, float alpha, const float *x,
                     float beta, float *y);

/* ----------------------------------------------------------- complex (C128 / C64) ---------- */
/* The reference's templates take std::complex<double> / std::complex<float> throughout
 * (sparse/hala_sparse_utils.hpp:104-336; gpu/hala_gpu_blas1.hpp dispatches them to cuBLAS Z / C
 * routines).  Vectors and values are interleaved pairs; complex scalars are R[2] = {re, im}.
 * Products and sums are separately rounded (re = ac - bd, im = ad + bc); division by Smith's
 * method.  y = alpha op(A) x + beta y; trans 'N', 'T' or 'C' (conjugate transpose); 'T' / 'C'
 * without a matrix handle scatter with atomics. */
int hgb_spmv_c128(hgb_ctx *ctx, char trans, int n_rows, int n_cols, int nnz, const int *pntr,
                  const int *indx, const void *vals, const double *alpha, const void *x,
                  const double *beta, void *y);
int hgb_spmv_c64(hgb_ctx *ctx, char trans, int n_rows, int n_cols, int nnz, const int *pntr,
                 const int *indx, const void *vals, const float *alpha, const void *x,
                 const float *beta, void *y);
/* dot (conjugated: sum conj(x_i) y_i, cublasZdotc), dotu (sum x_i y_i), nrm2 (real result).
 * result: R[2] (R[1] for nrm2), on the device when result_on_device, else on the host
 * (synchronises).  Sums accumulate in double. */
int hgb_dotc_c128(hgb_ctx *ctx, int n, const void *x, const void *y, double *result, int result_on_device);
int hgb_dotc_c64(hgb_ctx *ctx, int n, const void *x, const void *y, float *result, int result_on_device);
int hgb_dotu_c128(hgb_ctx *ctx, int n, const void *x, const void *y, double *result, int result_on_device);
int hgb_dotu_c64(hgb_ctx *ctx, int n, const void *x, const void *y, float *result, int result_on_device);
int hgb_nrm2_c128(hgb_ctx *ctx, int n, const void *x, double *result, int result_on_device);
int hgb_nrm2_c64(hgb_ctx *ctx, int n, const void *x, float *result, int result_on_device);
/* y += alpha x, x *= alpha with complex alpha {re, im} (host); a copy is hgb_copy_f64 / _f32 over 2n reals */
int hgb_axpy_c128(hgb_ctx *ctx, int n, const double *alpha, const void *x, void *y);
int hgb_axpy_c64(hgb_ctx *ctx, int n, const float *alpha, const void *x, void *y);
int hgb_scal_c128(hgb_ctx *ctx, int n, const double *alpha, void *x);
int hgb_scal_c64(hgb_ctx *ctx, int n, const float *alpha, void *x);

/* ---------------------- sparse matrix object (gpu_sparse_matrix, general.hpp:192-375) ------ */
/* Non-owning view of pntr/indx/vals (general.hpp:202) plus cached analysis: the row tiling of
 * the SpMV kernel and, on first transposed use, a transpose that makes op='T' deterministic and
 * identical to sparse_gemv_array<'T'> (utils:113-118).  vals dtype: F64, F32, BF16, C128 or C64. */
int hgb_csr_create(hgb_ctx *ctx, int n_rows, int n_cols, int nnz, const int *pntr,
                   const int *indx, const void *vals, hgb_dtype dtype, hgb_csr **A);
/* gpu_sparse_matrix::gemv, general.hpp:265-277.  x/y are double for F64, float for F32 / BF16, complex
 * pairs for C128 / C64 (alpha, beta then act as real scalars).  trans 'C' conjugates complex values. */
int hgb_csr_gemv(hgb_csr *A, char trans, double alpha, const void *x, double beta, void *y);
/* the same with complex scalars {re, im} (doubles, also for C64 matrices); the matrix must be C128 or C64 */
int hgb_csr_gemv_z(hgb_csr *A, char trans, const double *alpha, const void *x, const double *beta, void *y);
/* y = A x and *dot_out (device) = <x, y> in one pass (the fused SpMV + BLAS-1 epilogue) */
int hgb_csr_gemv_dot(hgb_csr *A, const void *x, void *y, double *dot_out_device);
/* grad[p] = alpha * lam[i] * u[indx[p]] for every stored entry p of row i: dL/dA restricted to
 * A's pattern for L(u(A)) with adjoint lam (alpha = -1).  Vectors in A's precision (F64/F32). */
int hgb_csr_pattern_grad(hgb_csr *A, double alpha, const void *lam, const void *u, void *grad);
int hgb_csr_destroy(hgb_csr *A);

/* ------------------------------------------------------------ pattern analysis --------- */
/* get_diagonal_index, sparse/hala_sparse_core.hpp:45-60; HGB_ERR_CSR if a diagonal is missing */
int hgb_diag_index(hgb_ctx *ctx, int n, int nnz, const int *pntr, const int *indx, int *diag);

/* split_pattern (sparse/hala_sparse_core.hpp:72-94) in the two passes of split_pattern_array
 * (sparse/hala_sparse_utils.hpp:176-193).  Row i of the lower pattern is [pntr_i, diag_i], of the
 * upper [diag_i, pntr_{i+1}): the diagonal is in both.  First pass: upper_pntr[n+1], lower_pntr[n+1]
 * (device) and the two entry counts (host, synchronises), so the caller can size the index arrays;
 * HGB_ERR_CSR if a diag_i lies outside its row.  Second pass: the column indices. */
int hgb_split_pattern_pntr(hgb_ctx *ctx, int n, const int *pntr, const int *diag, int *upper_pntr,
                           int *lower_pntr, int *upper_nnz_host, int *lower_nnz_host);
int hgb_split_pattern_indx(hgb_ctx *ctx, int n, const int *pntr, const int *indx, const int *diag,
                           const int *upper_pntr, const int *lower_pntr, int *upper_indx, int *lower_indx);
/* split_values (core:97-120, split_values_array utils:201-221): each triangle's values; the diagonal
 * of the triangle uplo does NOT select is set to 0 (diag 'N') or 1 (diag 'U'). */
int hgb_split_values_f64(hgb_ctx *ctx, char uplo, char diag, int n, const int *pntr, const double *vals,
                         const int *upper_pntr, const int *lower_pntr, double *upper_vals, double *lower_vals);
int hgb_split_values_f32(hgb_ctx *ctx, char uplo, char diag, int n, const int *pntr, const float *vals,
                         const int *upper_pntr, const int *lower_pntr, float *upper_vals, float *lower_vals);

/* ------------------------------------------------ ILU(0) (gpu_ilu, gpu_ilu.hpp:45-185) ----- */
/* make_ilu(gpu_engine, pntr, indx, vals, policy), gpu_ilu.hpp:54-109,192.
 * Factorises a copy of vals (the pattern is aliased, as in the reference) with the row-wise IKJ
 * order of factorize_ilu_array (sparse/hala_sparse_utils.hpp:229-255) and no fused multiply-add,
 * so the F64 factor is bit-identical to the reference CPU factor.  vals_dtype F64 or F32 selects
 * the factorisation precision; store selects the precision the triangular solves read:
 * F64 (vectors double), F32 or BF16 (vectors float; the pivots stay FP64: each pivot's reciprocal
 * is computed in FP64 and rounded once to FP32, and the FP32 backward sweep multiplies by it).
 * policy 'L'/'N' is accepted for signature parity; level scheduling is
 * always used.  Returns HGB_ERR_ZERO_PIVOT (with a valid handle) when a pivot is exactly 0.
 * Complex factors: vals_dtype = store = HGB_C128 or HGB_C64 (the IKJ order with complex operations,
 * rows of one level factorised in parallel; the apply sweeps level by level; trans 'T' and 'C'). */
int hgb_ilu0_create(hgb_ctx *ctx, int n, int nnz, const int *pntr, const int *indx,
                    const void *vals, hgb_dtype vals_dtype, hgb_dtype store, char policy,
                    hgb_ilu **ilu);
/* make_ilu(mixed_engine, pntr, indx, vals, policy), wax/hala_lib_extensions.hpp:311-366 (mixed_ilu):
 * HOST pattern and values.  The handle owns device copies of them.  The copies go to the device in
 * chunks on the context's copy stream, from a helper thread, while the calling thread checks the
 * pattern and plans the triangular schedules from the host arrays; the factorisation follows as in
 * hgb_ilu0_create.  HGB_ERR_CSR for a malformed host pattern (checked before any copy). */
int hgb_ilu0_create_host(hgb_ctx *ctx, int n, int nnz, const int *pntr_host, const int *indx_host,
                         const void *vals_host, hgb_dtype vals_dtype, hgb_dtype store, char policy,
                         hgb_ilu **ilu);
/* gpu_ilu::apply(x, r), gpu_ilu.hpp:150-164: r = U^-1 L^-1 x (trans 'N'), the arithmetic of
 * apply_ilu_array (utils:263-276); trans 'T': r = (LU)^-T x (adjoint).  x and r may alias. */
int hgb_ilu0_apply(hgb_ilu *ilu, char trans, const void *x, void *r);
/* device copies of the factor (values in the factorisation precision) and diagonal index */
int hgb_ilu0_export(hgb_ilu *ilu, void *factor_vals, int *diag);
/* level sets of the forward ('L') / backward ('U') solve: level[n] (device), *nlevels (host) */
int hgb_ilu0_levels(hgb_ilu *ilu, char uplo, int *level, int *nlevels);
int hgb_ilu0_destroy(hgb_ilu *ilu);

/* ------------------------- triangular matrix (gpu_triangular_matrix, triangular.hpp:38) ---- */
/* make_triangular_matrix(gpu_engine, uplo, diag, pntr, indx, vals): the triangle of a CSR
 * matrix selected by uplo ('L'/'U'), unit or non-unit diagonal ('U'/'N').  The CSR may hold
 * the other triangle too (ignored), as the reference's fill mode does (general.hpp:97-123). */
int hgb_tri_create(hgb_ctx *ctx, char uplo, char diag, int n, int nnz, const int *pntr,
                   const int *indx, const void *vals, hgb_dtype dtype, hgb_tri **tri);
/* gpu_triangular_matrix::trsv, triangular.hpp:341-354: op(T) x = alpha b, with the arithmetic
 * of sparse_trsv_array (sparse/hala_sparse_utils.hpp:284-336).  dtype may be C128 / C64 (then
 * alpha is real and trans 'C' conjugates). */
int hgb_tri_solve(hgb_tri *tri, char trans, double alpha, const void *b, void *x);
int hgb_tri_destroy(hgb_tri *tri);

/* ------------------------------------------------------------------- solvers ---------- */
/* solve_cg / solve_cg_ilu over gpu_engine (hex/solvers/hala_solvers_cg.hpp:181-264,295-326),
 * fused: device-resident scalars, the SpMV+dot and axpy+nrm2 fused, iterations replayed from a
 * CUDA graph.  M may be NULL (identity preconditioner).  Stop: iterations == max_iter or
 * ||r||_2 < tol (absolute, as the reference; pass tol*||b|| for a relative target).
 * Precision follows A (F64: x,b double; F32/BF16: float).  C128 / C64 matrices: the same loop
 * with the conjugated inner product and host scalars, as the reference's GPU path runs it. */
int hgb_cg_solve(hgb_ctx *ctx, hgb_csr *A, hgb_ilu *M, const void *b, void *x, double tol,
                 int max_iter, hgb_solve_info *info);
/* Same on op(A) = A^T ('T') or A ('N'): the transposed product goes through the matrix's cached
 * transpose and the preconditioner applies (LU)^-T.  The adjoint solve A^T lambda = g. */
int hgb_cg_solve_op(hgb_ctx *ctx, hgb_csr *A, hgb_ilu *M, char trans, const void *b, void *x,
                    double tol, int max_iter, hgb_solve_info *info);

/* ---- several right-hand sides with one matrix (n x nrhs column-major blocks) ---- */

/* Y = alpha A X + beta Y: sparse_gemm_array 'N','N' (sparse/hala_sparse_utils.hpp:127-133) through
 * sparse_gemm (wax).  One kernel reads the matrix once and sums every column in the single-column
 * product's order, so each column is bit-identical to hgb_csr_gemv (in the context's SpMV mode).
 * ldx >= columns of A, ldy >= rows of A. */
int hgb_csr_gemm(hgb_csr *A, int nrhs, double alpha, const void *x, int ldx, double beta, void *y, int ldy);

/* R = M^-1 X (trans 'N') or M^-T X, column by column: gpu_ilu::apply with num_rhs
 * (gpu/hala_gpu_ilu.hpp:150-164) / apply_ilu_array per column. */
int hgb_ilu0_apply_nrhs(hgb_ilu *M, char trans, int nrhs, const void *x, void *r);

/* Multi right-hand side PCG, solve_batch_cg / solve_batch_cg_ilu
 * (hex/solvers/hala_solvers_cg_batch.hpp:68-248): the CG recurrence of solve_cg_core with one
 * scalar per column; all columns iterate until iterations >= max_iter or the largest column
 * residual norm (batch_max_norm2) is below tol (absolute).  M may be NULL (no preconditioner).
 * B, X: device, n x nrhs column-major, the matrix's precision (FP32 vectors for BF16 values). */
int hgb_cg_solve_nrhs(hgb_ctx *ctx, hgb_csr *A, hgb_ilu *M, int nrhs, const void *B, void *X, double tol,
                      int max_iter, hgb_solve_info *info);

/* Mixed precision iterative refinement: FP64 outer residual, update and stopping test on A64
 * (F64); inner ILU(0)-PCG on A_inner (F32 or BF16 values, FP32 vectors and accumulation) with
 * M_inner (store F32 or BF16, FP64 pivots), each inner solve to ||r|| < inner_rtol * ||r0||.
 * Stops when ||b - A x||_2 < tol.  No reference counterpart. */
int hgb_ir_pcg_solve(hgb_ctx *ctx, hgb_csr *A64, hgb_csr *A_inner, hgb_ilu *M_inner,
                     const double *b, double *x, double tol, double inner_rtol, int max_inner,
                     int max_outer, hgb_solve_info *info);
/* hgb_ir_pcg_solve on op(A) (trans 'N' or 'T'; 'T' needs an F32 inner matrix): the adjoint of
 * the mixed-precision forward solve. */
int hgb_ir_pcg_solve_op(hgb_ctx *ctx, hgb_csr *A64, hgb_csr *A_inner, hgb_ilu *M_inner, char trans,
                        const double *b, double *x, double tol, double inner_rtol, int max_inner,
                        int max_outer, hgb_solve_info *info);
/* Mixed precision PCG with reliable updates (van der Vorst and Ye, SIAM J. Sci. Comput. 22,
 * 2000): one ILU(0)-PCG on A_inner (F32 or BF16 values, FP32 vectors) with M_inner (store F32
 * or BF16) on the correction d; when ||r|| drops below delta (0 < delta < 1) times its largest
 * value since the last update, or below tol, or at max_iter, x += d in FP64 and r = b - A64 x
 * in FP64, continuing with the same search direction (restarted, beta = 0, when that update
 * reduced the FP64 residual less than twice).  Keeps the Krylov space (FP64 PCG's iteration
 * count) where hgb_ir_pcg_solve restarts it per sweep.  Stops when the FP64
 * ||b - A x||_2 < tol.  info->iterations: inner iterations, info->outer: reliable updates.
 * No reference counterpart. */
int hgb_ru_pcg_solve(hgb_ctx *ctx, hgb_csr *A64, hgb_csr *A_inner, hgb_ilu *M_inner, const double *b,
                     double *x, double tol, double delta, int max_iter, hgb_solve_info *info);
/* hgb_ru_pcg_solve on op(A) (trans 'N' or 'T'; 'T' needs an F32 inner matrix): the adjoint of the
 * mixed-precision forward solve, with the cached transposes and the transposed ILU apply. */
int hgb_ru_pcg_solve_op(hgb_ctx *ctx, hgb_csr *A64, hgb_csr *A_inner, hgb_ilu *M_inner, char trans,
                        const double *b, double *x, double tol, double delta, int max_iter,
                        hgb_solve_info *info);
/* solve_gmres / solve_gmres_ilu over gpu_engine (hex/solvers/hala_solvers_gmres.hpp:127-267):
 * left preconditioned restarted GMRES, one classical Gram-Schmidt pass, Givens rotations in
 * the reference's order.  The rotations and the back substitution run on the device and one
 * restart cycle is one CUDA graph (one host synchronisation per cycle, where the reference
 * reads the projection back in every inner iteration, :67-72).  max_iter bounds the restarts,
 * tol is absolute on the preconditioned residual estimate, restart 1..512.  F64, F32 or BF16
 * values (A's precision; FP32 vectors for BF16) with a preconditioner of matching precision.
 * C128 / C64: the same loop driven from the host; the projection does not conjugate (W^T r, as the
 * reference's krylov_project, gemv 'T' at hex/solvers/hala_solvers_gmres.hpp:47-50,67-72). */
int hgb_gmres_solve(hgb_ctx *ctx, hgb_csr *A, hgb_ilu *M, int restart, const void *b, void *x,
                    double tol, int max_iter, hgb_solve_info *info);
/* Mixed precision GMRES: FP64 iterative refinement (residual, update and stopping test
 * ||b - A x||_2 < tol on A64) around GMRES(restart) on A_inner (F32 or BF16 values, FP32
 * vectors) with M_inner (store F32 or BF16), each inner solve to a preconditioned residual
 * estimate below inner_rtol times its first one (max_inner inner iterations per sweep).
 * No reference counterpart; the inner solver is solve_gmres (hala_solvers_gmres.hpp:127-230). */
int hgb_ir_gmres_solve(hgb_ctx *ctx, hgb_csr *A64, hgb_csr *A_inner, hgb_ilu *M_inner, int restart,
                       const double *b, double *x, double tol, double inner_rtol, int max_inner,
                       int max_outer, hgb_solve_info *info);
/* mixed_engine form (wax/hala_lib_extensions.hpp:68; solve_cg_ilu(mixed_engine,...),
 * hala_solvers_cg.hpp:330-340): HOST pntr/indx/vals/b/x, loaded to the device per call, solved
 * with the device factor M, x written back to the host.  FP64. */
int hgb_mixed_cg_solve(hgb_ctx *ctx, int n, int nnz, const int *pntr_host, const int *indx_host,
                       const double *vals_host, hgb_ilu *M, const double *b_host, double *x_host,
                       double tol, int max_iter, hgb_solve_info *info);

/* Host-buffer form of hgb_ir_pcg_solve: HOST pntr/indx/vals (FP64) and b/x are loaded per call,
 * the inner matrix is converted on the device to FP32 (also beside a BF16-stored M_inner: a BF16
 * operator shifts the fixed point of the refinement, see the design notes), the refinement runs as
 * hgb_ir_pcg_solve and x is written back to the host. */
int hgb_mixed_ir_pcg_solve(hgb_ctx *ctx, int n, int nnz, const int *pntr_host, const int *indx_host,
                           const double *vals_host, hgb_ilu *M_inner, const double *b_host,
                           double *x_host, double tol, double inner_rtol, int max_inner,
                           int max_outer, hgb_solve_info *info);
/* Host-buffer form of hgb_ru_pcg_solve, loaded and converted as hgb_mixed_ir_pcg_solve. */
int hgb_mixed_ru_pcg_solve(hgb_ctx *ctx, int n, int nnz, const int *pntr_host, const int *indx_host,
                           const double *vals_host, hgb_ilu *M_inner, const double *b_host,
                           double *x_host, double tol, double delta, int max_iter, hgb_solve_info *info);

/* ------------------------------------------ batched independent systems (no reference
 * counterpart: the reference's batch is one matrix with many right-hand sides) -------------- */
/* Launch shape of the batched solver: threads per CTA (128, 256 or 512) and the largest system
 * solved by a single warp (larger systems get a whole CTA). */
typedef struct hgb_batch_config { int block_threads; int warp_max_n; } hgb_batch_config;
/* A batch of S independent systems stored as one block-diagonal CSR with FP32 values and global
 * column indices; sys_ptr[S+1] (device) holds the first row of each system.  Every column of a
 * system's rows must lie inside that system (checked, HGB_ERR_CSR).  Systems up to 4096 rows. */
int hgb_batch_create(hgb_ctx *ctx, int num_systems, const int *sys_ptr, int n_total, int nnz,
                     const int *pntr, const int *indx, const float *vals, hgb_batch **batch);
int hgb_batch_set_config(hgb_batch *batch, const hgb_batch_config *cfg);
int hgb_batch_get_config(hgb_batch *batch, hgb_batch_config *cfg);
/* Solves every system in ONE persistent kernel launch, replayed from a CUDA graph: FP32 CG
 * (inner relative tolerance inner_rtol, at most max_inner iterations) inside FP64 refinement
 * until ||b_s - A_s x_s|| <= rtol ||b_s|| for each system s (at most max_outer sweeps).  x holds
 * the initial guesses.  iters[S] / relres[S] (device, optional) receive per-system totals. */
int hgb_batch_cg_solve(hgb_batch *batch, const double *b, double *x, double rtol, double inner_rtol,
                       int max_inner, int max_outer, int *iters, double *relres);
/* Times the launch shapes on this batch (x is overwritten) and keeps the fastest; the choice
 * is cached under a size-histogram key in cache_path (text, may be NULL). */
int hgb_batch_autotune(hgb_batch *batch, const double *b, double *x, double rtol,
                       const char *cache_path, hgb_batch_config *best);
int hgb_batch_destroy(hgb_batch *batch);

/* ------------------------------------------------------- allocation-free reduction ---- */
/* No counterpart in the reference.  *result_device = <x, y> for callers that may not allocate
 * device memory where they need the reduction (an allocator or memory budget owned by another
 * component, or a host integration that may not create an hgb_ctx, which allocates).  Needs no
 * context and calls no allocating routine: the partial sums live in a static device array (one per
 * 2048 entries), so n <= 33,554,432; larger n returns HGB_ERR_ARG before any launch.  The first
 * call on a device (and in each new CUDA context on it) looks the array's address up with
 * cudaGetSymbolAddress: make it before any stream capture.  It makes CUDA runtime calls, so it
 * must not be called from a stream callback or host function node.  Calls share the array, so
 * calls whose kernels overlap on the GPU race.  Runs on the current device, on the given stream
 * (cudaStream_t, may be NULL); does not synchronise. */
int hgb_dot_f64_noalloc(int n, const double *x, const double *y, double *result_device,
                        void *stream);

/* ----------------------------------------------------------- fault-path self test ------ */
/* Launches one bounded device wait on a value nothing ever publishes; returns HGB_ERR_TIMEOUT
 * after spin_limit polls while leaving the context usable.  Test hook for the timeout path. */
int hgb_selftest_wait_timeout(hgb_ctx *ctx, int spin_limit);

#ifdef __cplusplus
}
#endif
#endif
