// Complex (C128 / C64) variants of the path (hgb_complex.cu): internal entry points.
#pragma once

#include "hgb_internal.cuh"
#include "hgb_kernels.cuh"

struct hgb_zilu;
struct hgb_ztri;

namespace hgb {

// y = alpha op(A) x + beta y with complex scalars (R[2] each); T: the matrix's cached transpose
// ('T' / 'C' without it scatter with atomics)
template <typename R>
int zspmv(hgb_ctx *c, char trans, int n_rows, int n_cols, const int *pntr, const int *indx, const void *vals,
          const R *alpha, const void *x, const R *beta, void *y, const Transpose *T);
// op 0: sum conj(x) y, op 1: sum x y (result R[2]); op 2: ||x||_2 (result R[1])
template <typename R> int zdot(hgb_ctx *c, int op, int n, const void *x, const void *y, R *result, int on_device);
template <typename R> int zaxpy(hgb_ctx *c, int n, const R *alpha, const void *x, void *y);
template <typename R> int zscal(hgb_ctx *c, int n, const R *alpha, void *x);

// ILU(0) of a complex matrix (rsize: bytes of one real part, 8 or 4)
int zilu_create(hgb_ctx *c, int n, int nnz, const int *pntr, const int *indx, const void *vals, int rsize,
                hgb_zilu **out, int *zero_pivot);
int zilu_apply(hgb_zilu *M, char trans, const void *x, void *r);
int zilu_export(hgb_zilu *M, void *factor, int *diag);
int zilu_rsize(const hgb_zilu *M);
void zilu_destroy(hgb_zilu *M);

int ztri_create(hgb_ctx *c, char uplo, char diag, int n, int nnz, const int *pntr, const int *indx, const void *vals,
                int rsize, hgb_ztri **out);
int ztri_solve(hgb_ztri *T, char trans, const void *alpha, const void *b, void *x);
void ztri_destroy(hgb_ztri *T);

int zcg_solve(hgb_ctx *c, hgb_csr *A, hgb_zilu *M, const void *b, void *x, double tol, int max_iter,
              hgb_solve_info *info);
int zgmres_solve(hgb_ctx *c, hgb_csr *A, hgb_zilu *M, int restart, const void *b, void *x, double tol, int max_iter,
                 hgb_solve_info *info);

}  // namespace hgb
