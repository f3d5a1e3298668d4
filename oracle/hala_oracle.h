/*
 * CPU oracle for the sparse Krylov path: a plain-C restatement of the reference's CPU algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * reference arm may load this library, and only as the checker or the timed CPU baseline; the
 * product (hala_gb300, libhgb.so) never links or calls it.
 *
 * Parity is pinned two ways: against the golden vectors of the reference's own tests
 * (tests/sparse_tests.hpp, tests/solvers_tests.hpp) and against the reference's CPU path
 * compiled from its unmodified headers (oracle/ref -> oracle/_ref/libhalaref.so).
 *
 * Suffix _d = double, _f = float.  Every function cites the reference code it restates.
 */
#ifndef HALA_ORACLE_H
#define HALA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* get_diagonal_index, sparse/hala_sparse_core.hpp:45-60.  Returns 0, or -(i+1) if row i has no
 * diagonal entry (the reference asserts presence; the restatement reports it). */
int or_diag_index(int n, const int *pntr, const int *indx, int *diag);

/* split_pattern_array, sparse/hala_sparse_utils.hpp:176-193 (both passes). */
void or_split_pattern(int n, const int *pntr, const int *indx, const int *diag,
                      int *up, int *ui, int *lp, int *li);

/* Level sets of the triangular solves (no reference counterpart: cuSPARSE analysis is opaque).
 * lower: lev(i) = 0 if row i has no strictly-lower entry, else 1 + max lev(j), j<i in row i.
 * upper: same over the strictly-upper entries, with rows visited in reverse order.
 * Returns the number of levels. */
int or_levels(int n, const int *pntr, const int *indx, const int *diag, char uplo, int *level);

/* ILU(0) factorisation, exactly as factorize_ilu_array (sparse/hala_sparse_utils.hpp:229-255):
 * O(n^2) pivot-row loop.  Only for small n. */
void or_ilu_factor_pivot_d(int n, const int *pntr, const int *indx, const int *diag, double *ilu);

/* Per-thread bf16 helpers: round-to-nearest-even conversion of float to bfloat16 bits. */
uint16_t or_f32_to_bf16(float v);
float or_bf16_to_f32(uint16_t v);

void or_spmv_bf16f32(char trans, int m, int ncols, float alpha, const int *pntr, const int *indx,
                     const uint16_t *vals, const float *x, float beta, float *y);

#define OR_DECLARE(T, S)                                                                       \
    /* sparse_gemv_array<T,'N'/'T'>, sparse/hala_sparse_utils.hpp:104-119 */                    \
    void or_spmv_##S(char trans, int m, int ncols, T alpha, const int *pntr, const int *indx,   \
                     const T *vals, const T *x, T beta, T *y);                                  \
    /* split_values_array, sparse/hala_sparse_utils.hpp:201-221 */                              \
    void or_split_values_##S(char uplo, char diag, int n, const int *pntr, const T *vals,      \
                             const int *up, const int *lp, T *uv, T *lv);                       \
    /* row-wise IKJ restatement of factorize_ilu_array: same per-entry update order */          \
    int or_ilu_factor_##S(int n, const int *pntr, const int *indx, const int *diag, T *ilu);   \
    /* apply_ilu_array, sparse/hala_sparse_utils.hpp:263-276 (in place on x) */                 \
    void or_ilu_apply_##S(int n, const int *pntr, const int *indx, const int *diag,            \
                          const T *ilu, T *x);                                                  \
    /* transposed apply: x <- (L U)^-T x = L^-T U^-T x (adjoint of apply_ilu_array) */          \
    void or_ilu_apply_t_##S(int n, const int *pntr, const int *indx, const int *diag,          \
                            const T *ilu, T *x);                                                \
    /* sparse_trsv_array, sparse/hala_sparse_utils.hpp:284-336 (triangular CSR, diag last/first) */ \
    void or_trsv_##S(char uplo, char diag, char trans, int n, T alpha, const int *pntr,        \
                     const int *indx, const T *vals, const T *b, T *x);                         \
    /* BLAS-1 as the netlib loops (blas/hala_blas_1.hpp) */                                      \
    T or_dot_##S(int n, const T *x, const T *y);                                                \
    T or_nrm2_##S(int n, const T *x);                                                           \
    /* solve_cg_core, hex/solvers/hala_solvers_cg.hpp:92-156, with identity (ilu == NULL) or    \
     * ILU(0) preconditioner.  Absolute tolerance on the recurrence residual.  Returns the      \
     * reference's iteration count; *res_out (if not NULL) gets the last ||r||. */              \
    int or_cg_##S(int n, const int *pntr, const int *indx, const T *vals, const int *diag,     \
                  const T *ilu, const T *b, T *x, T tol, int max_iter, T *res_out);            \
    /* solve_batch_cg[_ilu], hex/solvers/hala_solvers_cg_batch.hpp:68-248: nrhs column-major   \
     * right-hand sides, one CG scalar per column, stop on the largest column residual. */      \
    int or_batch_cg_##S(int n, const int *pntr, const int *indx, const T *vals, const int *diag, \
                        const T *ilu, int nrhs, const T *b, T *x, T tol, int max_iter,           \
                        T *res_out);                                                             \
    /* solve_gmres, hex/solvers/hala_solvers_gmres.hpp:127-230 (left preconditioned, one       \
     * classical Gram-Schmidt pass, host Givens).  Returns total operator applications. */      \
    int or_gmres_##S(int n, const int *pntr, const int *indx, const T *vals, const int *diag,  \
                     const T *ilu, int restart, const T *b, T *x, T tol, int max_iter);

OR_DECLARE(double, d)
OR_DECLARE(float, f)

/* Mixed-precision iterative refinement (no reference counterpart): outer r = b - A x in FP64,
 * inner ILU(0)-PCG in FP32 on (vals32, ilu32 with FP64 pivots piv) to relative tolerance
 * inner_rtol, x += d in FP64.  Stops when ||b - A x|| < tol.  Returns total inner iterations;
 * *outer_out gets the outer count. */
/* FP32 ILU(0) apply of an FP32 factor with FP64 pivots (the inner preconditioner of
 * or_ir_pcg): off-diagonal updates in float in the order of apply_ilu_array, then x_i times
 * (float)(1.0 / piv_i). */
void or_ilu_apply_mixed(int n, const int *pntr, const int *indx, const int *diag, const float *ilu32,
                        const double *piv, float *x);

int or_ir_pcg(int n, const int *pntr, const int *indx, const double *vals, const float *vals32,
              const int *diag, const float *ilu32, const double *piv, const double *b, double *x,
              double tol, double inner_rtol, int max_inner, int max_outer, int *outer_out);

/* Mixed-precision PCG with reliable updates (no reference counterpart): one FP32 ILU(0)-PCG on
 * the correction d (inner products in double); when ||r|| < delta * (its largest value since the
 * last update), or ||r|| < tol, or at max_iter: x += d in FP64, r = b - A x in FP64, and the
 * iteration continues with the same direction.  Stops when that FP64 residual is below tol.
 * Returns the iterations; *updates_out gets the reliable updates. */
int or_ru_pcg(int n, const int *pntr, const int *indx, const double *vals, const float *vals32,
              const int *diag, const float *ilu32, const double *piv, const double *b, double *x,
              double tol, double delta, int max_iter, int *updates_out);

/* Mixed-precision GMRES (no reference counterpart): outer r = b - A x in FP64, inner
 * GMRES(restart) (solve_gmres's loop) in FP32 vectors with double inner products and rotations,
 * on (vals32, ilu32 with FP64 pivots piv), each sweep to a relative preconditioned tolerance,
 * x += d in FP64.  Stops when ||b - A x|| < tol.  Returns the inner operator applications;
 * *outer_out gets the sweeps. */
int or_ir_gmres(int n, const int *pntr, const int *indx, const double *vals, const float *vals32,
                const int *diag, const float *ilu32, const double *piv, int restart, const double *b,
                double *x, double tol, double inner_rtol, int max_inner, int max_outer, int *outer_out);

#ifndef __cplusplus
/* ------------------------------------------------------------------- complex ------------ */
/* hala_oracle_cplx.c: suffix _z = double complex, _c = float complex (interleaved pairs, the
 * layout of std::complex).  Scalars alpha / beta of the products are {re, im} pairs.  The same
 * reference code as the real functions above, on std::complex values:
 *   or_spmv         sparse_gemv_array, sparse/hala_sparse_utils.hpp:104-119 ('C' conjugates)
 *   or_ilu_factor   factorize_ilu_array, utils:229-255 (returns first zero pivot row + 1, or 0)
 *   or_ilu_apply    apply_ilu_array, utils:263-276;  or_ilu_apply_t: (LU)^-T / (LU)^-H
 *   or_trsv         sparse_trsv_array, utils:284-336 (real alpha)
 *   or_dotc, or_nrm2  hala::dot (conjugated), dznrm2 / scnrm2
 *   or_cg           solve_cg_core + solve_cg, hex/solvers/hala_solvers_cg.hpp:92-156,207-226
 *   or_gmres        solve_gmres, hex/solvers/hala_solvers_gmres.hpp:127-230 (unconjugated
 *                   projection, gemv 'T' at :47-50, as the reference) */
#define OR_CPLX_DECL(CT, RT, S)                                                                        \
    void or_spmv_##S(char trans, int m, int ncols, const RT *alpha, const int *pntr, const int *indx,   \
                     const CT *vals, const CT *x, const RT *beta, CT *y);                               \
    int or_ilu_factor_##S(int n, const int *pntr, const int *indx, const int *diag, CT *ilu);          \
    void or_ilu_apply_##S(int n, const int *pntr, const int *indx, const int *diag, const CT *ilu,     \
                          CT *x);                                                                      \
    void or_ilu_apply_t_##S(char trans, int n, const int *pntr, const int *indx, const int *diag,      \
                            const CT *ilu, CT *x);                                                     \
    void or_trsv_##S(char uplo, char diag, char trans, int n, RT alpha, const int *pntr,              \
                     const int *indx, const CT *vals, const CT *b, CT *x);                              \
    void or_dotc_##S(int n, const CT *x, const CT *y, RT *out);                                        \
    RT or_nrm2_##S(int n, const CT *x);                                                                \
    int or_cg_##S(int n, const int *pntr, const int *indx, const CT *vals, const int *diag,            \
                  const CT *ilu, const CT *b, CT *x, RT tol, int max_iter, RT *res_out);               \
    int or_gmres_##S(int n, const int *pntr, const int *indx, const CT *vals, const int *diag,         \
                     const CT *ilu, int restart, const CT *b, CT *x, RT tol, int max_iter);
OR_CPLX_DECL(double _Complex, double, z)
OR_CPLX_DECL(float _Complex, float, c)
#undef OR_CPLX_DECL
#endif

#ifdef __cplusplus
}
#endif
#endif
