/*
 * extern "C" shim over the reference's own CPU templates (test infrastructure only).
 *
 * Compiled by oracle/ref/Makefile against the UNMODIFIED reference headers (HALA v1.1.0) into
 * oracle/_ref/libhalaref.so.  It is used to (1) pin the C restatement in oracle/hala_oracle.c
 * and (2) generate the golden fixtures under tests/golden/.  Each wrapper calls exactly one
 * reference entry point:
 *   sparse_gemv            sparse/hala_sparse_blas.hpp:79
 *   get_diagonal_index     sparse/hala_sparse_core.hpp:45
 *   split_pattern/values   sparse/hala_sparse_core.hpp:72,107
 *   factorize_ilu          sparse/hala_sparse_core.hpp:158 (O(n^2) reference loop)
 *   apply_ilu              sparse/hala_sparse_core.hpp:196
 *   sparse_trsv            sparse/hala_sparse_blas.hpp:183 (cpu_triangular_matrix)
 *   solve_cg               hex/solvers/hala_solvers_cg.hpp:181 (identity or ILU preconditioner)
 *   solve_gmres            hex/solvers/hala_solvers_gmres.hpp:127 (cpu_engine)
 *   solve_batch_cg         hex/solvers/hala_solvers_cg_batch.hpp (multi right-hand side)
 * Suffixes: _d double, _f float, _z std::complex<double>, _c std::complex<float> (complex scalars
 * of the products as {re, im} pairs, interleaved complex arrays).
 */
#include "hala.hpp"
#include "hala_solvers.hpp"

#include <complex>
#include <vector>

namespace {

using zd = std::complex<double>;
using zf = std::complex<float>;
template <typename T> using prec_t = hala::get_precision_type<std::vector<T>>;

template <typename T>
std::vector<T> vec(const T *p, long n) { return std::vector<T>(p, p + n); }

template <typename T>
void out(const std::vector<T> &v, T *p) { std::copy(v.begin(), v.end(), p); }

template <typename T>
void gemv_t(char trans, int M, int N, T alpha, const int *pntr, const int *indx, const T *vals,
            const T *x, T beta, T *y) {
    int nnz = pntr[M];
    auto P = vec(pntr, M + 1);
    auto I = vec(indx, nnz);
    auto V = vec(vals, nnz);
    auto X = vec(x, (trans == 'N') ? N : M);
    auto Y = vec(y, (trans == 'N') ? M : N);
    hala::sparse_gemv(trans, M, N, alpha, P, I, V, X, beta, Y);
    out(Y, y);
}

template <typename T>
void factorize_t(int n, const int *pntr, const int *indx, const T *vals, T *ilu) {
    auto P = vec(pntr, n + 1);
    auto I = vec(indx, pntr[n]);
    auto V = vec(vals, pntr[n]);
    std::vector<int> D;
    hala::get_diagonal_index(P, I, D);
    std::vector<T> F;
    hala::factorize_ilu(P, I, V, *const_cast<std::vector<int> const *>(&D), F);
    out(F, ilu);
}

template <typename T>
void apply_ilu_t(int n, const int *pntr, const int *indx, const int *diag, const T *ilu, T *x) {
    auto P = vec(pntr, n + 1);
    auto I = vec(indx, pntr[n]);
    auto D = vec(diag, n);
    auto F = vec(ilu, pntr[n]);
    auto X = vec(x, n);
    hala::apply_ilu(P, I, D, F, X);
    out(X, x);
}

template <typename T>
void trsv_t(char uplo, char diag, char trans, int n, T alpha, const int *pntr, const int *indx,
            const T *vals, const T *b, T *x) {
    int nnz = pntr[n];
    auto P = vec(pntr, n + 1);
    auto I = vec(indx, nnz);
    auto V = vec(vals, nnz);
    auto B = vec(b, n);
    std::vector<T> X;
    auto tri = hala::make_triangular_matrix(hala::cpu_engine(), uplo, diag, P, I, V);
    hala::sparse_trsv(trans, tri, alpha, B, X);
    out(X, x);
}

/* ilu == nullptr: identity preconditioner (plain CG); else the given ILU(0) factor values */
template <typename T>
int cg_t(int n, const int *pntr, const int *indx, const T *vals, const int *diag, const T *ilu,
         const T *b, T *x, prec_t<T> tol, int max_iter) {
    int nnz = pntr[n];
    auto P = vec(pntr, n + 1);
    auto I = vec(indx, nnz);
    auto V = vec(vals, nnz);
    auto B = vec(b, n);
    auto X = vec(x, n);
    std::vector<int> D;
    std::vector<T> F;
    if (ilu) { D = vec(diag, n); F = vec(ilu, nnz); }
    int it = hala::solve_cg(hala::stop_criteria<prec_t<T>>(tol, max_iter), P, I, V,
                            [&](std::vector<T> const &in, std::vector<T> &o) -> void {
                                hala::vcopy(in, o);
                                if (ilu) hala::apply_ilu(P, I, D, F, o);
                            },
                            B, X);
    out(X, x);
    return it;
}

template <typename T>
int gmres_t(int n, const int *pntr, const int *indx, const T *vals, const int *diag, const T *ilu,
            int restart, const T *b, T *x, prec_t<T> tol, int max_iter) {
    int nnz = pntr[n];
    auto P = vec(pntr, n + 1);
    auto I = vec(indx, nnz);
    auto V = vec(vals, nnz);
    auto B = vec(b, n);
    auto X = vec(x, n);
    std::vector<int> D;
    std::vector<T> F;
    if (ilu) { D = vec(diag, n); F = vec(ilu, nnz); }
    int it = hala::solve_gmres(hala::cpu_engine(), hala::stop_criteria<prec_t<T>>(tol, max_iter), restart,
                               P, I, V,
                               [&](std::vector<T> const &in, std::vector<T> &o) -> void {
                                   hala::vcopy(in, o);
                                   if (ilu) hala::apply_ilu(P, I, D, F, o);
                               },
                               B, X);
    out(X, x);
    return it;
}

}  // namespace

extern "C" {

void ref_sparse_gemv_d(char trans, int M, int N, double alpha, const int *pntr, const int *indx,
                       const double *vals, const double *x, double beta, double *y) {
    gemv_t<double>(trans, M, N, alpha, pntr, indx, vals, x, beta, y);
}
void ref_sparse_gemv_f(char trans, int M, int N, float alpha, const int *pntr, const int *indx,
                       const float *vals, const float *x, float beta, float *y) {
    gemv_t<float>(trans, M, N, alpha, pntr, indx, vals, x, beta, y);
}

void ref_get_diagonal_index(int n, const int *pntr, const int *indx, int *diag) {
    auto P = vec(pntr, n + 1);
    auto I = vec(indx, pntr[n]);
    std::vector<int> D;
    hala::get_diagonal_index(P, I, D);
    out(D, diag);
}

/* sizes: up/lp n+1, ui/li at most nnz; returns through *nu and *nl the split sizes */
void ref_split_pattern(int n, const int *pntr, const int *indx, const int *diag, int *up, int *ui,
                       int *lp, int *li, int *nu, int *nl) {
    auto P = vec(pntr, n + 1);
    auto I = vec(indx, pntr[n]);
    auto D = vec(diag, n);
    std::vector<int> UP, UI, LP, LI;
    hala::split_pattern(P, I, D, UP, UI, LP, LI);
    out(UP, up); out(UI, ui); out(LP, lp); out(LI, li);
    *nu = (int)UI.size();
    *nl = (int)LI.size();
}

void ref_split_values_d(char uplo, char diag, int n, const int *pntr, const double *vals,
                        const int *up, const int *lp, double *uv, double *lv) {
    auto P = vec(pntr, n + 1);
    auto V = vec(vals, pntr[n]);
    auto UP = vec(up, n + 1);
    auto LP = vec(lp, n + 1);
    std::vector<double> UV, LV;
    hala::split_values(uplo, diag, P, V, UP, LP, UV, LV);
    out(UV, uv); out(LV, lv);
}

void ref_factorize_ilu_d(int n, const int *pntr, const int *indx, const double *vals, double *ilu) {
    auto P = vec(pntr, n + 1);
    auto I = vec(indx, pntr[n]);
    auto V = vec(vals, pntr[n]);
    std::vector<int> D;
    hala::get_diagonal_index(P, I, D);
    std::vector<double> F;
    hala::factorize_ilu(P, I, V, *const_cast<std::vector<int> const *>(&D), F);
    out(F, ilu);
}
void ref_factorize_ilu_f(int n, const int *pntr, const int *indx, const float *vals, float *ilu) {
    auto P = vec(pntr, n + 1);
    auto I = vec(indx, pntr[n]);
    auto V = vec(vals, pntr[n]);
    std::vector<int> D;
    hala::get_diagonal_index(P, I, D);
    std::vector<float> F;
    hala::factorize_ilu(P, I, V, *const_cast<std::vector<int> const *>(&D), F);
    out(F, ilu);
}

void ref_apply_ilu_d(int n, const int *pntr, const int *indx, const int *diag, const double *ilu,
                     double *x) {
    auto P = vec(pntr, n + 1);
    auto I = vec(indx, pntr[n]);
    auto D = vec(diag, n);
    auto F = vec(ilu, pntr[n]);
    auto X = vec(x, n);
    hala::apply_ilu(P, I, D, F, X);
    out(X, x);
}
void ref_apply_ilu_f(int n, const int *pntr, const int *indx, const int *diag, const float *ilu,
                     float *x) {
    auto P = vec(pntr, n + 1);
    auto I = vec(indx, pntr[n]);
    auto D = vec(diag, n);
    auto F = vec(ilu, pntr[n]);
    auto X = vec(x, n);
    hala::apply_ilu(P, I, D, F, X);
    out(X, x);
}

void ref_trsv_d(char uplo, char diag, char trans, int n, double alpha, const int *pntr,
                const int *indx, const double *vals, const double *b, double *x) {
    trsv_t<double>(uplo, diag, trans, n, alpha, pntr, indx, vals, b, x);
}

int ref_solve_cg_d(int n, const int *pntr, const int *indx, const double *vals, const int *diag,
                   const double *ilu, const double *b, double *x, double tol, int max_iter) {
    return cg_t<double>(n, pntr, indx, vals, diag, ilu, b, x, tol, max_iter);
}
int ref_solve_cg_f(int n, const int *pntr, const int *indx, const float *vals, const int *diag,
                   const float *ilu, const float *b, float *x, float tol, int max_iter) {
    return cg_t<float>(n, pntr, indx, vals, diag, ilu, b, x, tol, max_iter);
}

int ref_solve_gmres_d(int n, const int *pntr, const int *indx, const double *vals, const int *diag,
                      const double *ilu, int restart, const double *b, double *x, double tol,
                      int max_iter) {
    return gmres_t<double>(n, pntr, indx, vals, diag, ilu, restart, b, x, tol, max_iter);
}
int ref_solve_gmres_f(int n, const int *pntr, const int *indx, const float *vals, const int *diag,
                      const float *ilu, int restart, const float *b, float *x, float tol,
                      int max_iter) {
    return gmres_t<float>(n, pntr, indx, vals, diag, ilu, restart, b, x, tol, max_iter);
}

/* multi right-hand side CG with the reference's own ILU (factorised by the reference) */
int ref_solve_batch_cg_ilu_d(int n, const int *pntr, const int *indx, const double *vals, int nrhs,
                             const double *b, double *x, double tol, int max_iter) {
    int nnz = pntr[n];
    auto P = vec(pntr, n + 1);
    auto I = vec(indx, nnz);
    auto V = vec(vals, nnz);
    auto B = vec(b, (long)n * nrhs);
    auto X = vec(x, (long)n * nrhs);
    auto ilu = hala::make_ilu(hala::cpu_engine(), P, I, V, 'N');
    int it = hala::solve_batch_cg_ilu(hala::cpu_engine(), hala::stop_criteria<double>(tol, max_iter),
                                      P, I, V, ilu, B, X);
    out(X, x);
    return it;
}

/* complex: the same templates on std::complex (alpha / beta {re, im}; trsv's alpha real) */
#define REF_COMPLEX(S, Z, R)                                                                            \
    void ref_sparse_gemv_##S(char trans, int M, int N, const R *alpha, const int *pntr, const int *indx, \
                             const Z *vals, const Z *x, const R *beta, Z *y) {                           \
        gemv_t<Z>(trans, M, N, Z(alpha[0], alpha[1]), pntr, indx, vals, x, Z(beta[0], beta[1]), y);     \
    }                                                                                                    \
    void ref_factorize_ilu_##S(int n, const int *pntr, const int *indx, const Z *vals, Z *ilu) {         \
        factorize_t<Z>(n, pntr, indx, vals, ilu);                                                        \
    }                                                                                                    \
    void ref_apply_ilu_##S(int n, const int *pntr, const int *indx, const int *diag, const Z *ilu,       \
                           Z *x) {                                                                       \
        apply_ilu_t<Z>(n, pntr, indx, diag, ilu, x);                                                     \
    }                                                                                                    \
    void ref_trsv_##S(char uplo, char diag, char trans, int n, R alpha, const int *pntr,                \
                      const int *indx, const Z *vals, const Z *b, Z *x) {                                \
        trsv_t<Z>(uplo, diag, trans, n, Z(alpha), pntr, indx, vals, b, x);                               \
    }                                                                                                    \
    int ref_solve_cg_##S(int n, const int *pntr, const int *indx, const Z *vals, const int *diag,        \
                         const Z *ilu, const Z *b, Z *x, R tol, int max_iter) {                          \
        return cg_t<Z>(n, pntr, indx, vals, diag, ilu, b, x, tol, max_iter);                             \
    }                                                                                                    \
    int ref_solve_gmres_##S(int n, const int *pntr, const int *indx, const Z *vals, const int *diag,     \
                            const Z *ilu, int restart, const Z *b, Z *x, R tol, int max_iter) {          \
        return gmres_t<Z>(n, pntr, indx, vals, diag, ilu, restart, b, x, tol, max_iter);                 \
    }
REF_COMPLEX(z, zd, double)
REF_COMPLEX(c, zf, float)
#undef REF_COMPLEX

}  // extern "C"
