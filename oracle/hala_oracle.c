/*
 * CPU oracle for the sparse Krylov path (TEST INFRASTRUCTURE ONLY; see hala_oracle.h).
 * Compiled with -ffp-contract=off so that no multiply-add is fused: the reference's CPU path is
 * ISO C++ and its results are the sequence of separately rounded IEEE operations written here.
 */
#include "hala_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* get_diagonal_index, sparse/hala_sparse_core.hpp:45-60 (scan each row up to column i) */
int or_diag_index(int n, const int *pntr, const int *indx, int *diag) {
    for (int i = 0; i < n; i++) {
        int d = pntr[i];
        while (d < pntr[i + 1] && indx[d] < i) d++;
        if (d == pntr[i + 1] || indx[d] != i) return -(i + 1);
        diag[i] = d;
    }
    return 0;
}

/* split_pattern_array<true> then <false>, sparse/hala_sparse_utils.hpp:176-193 */
void or_split_pattern(int n, const int *pntr, const int *indx, const int *diag, int *up, int *ui,
                      int *lp, int *li) {
    up[0] = 0;
    lp[0] = 0;
    for (int i = 0; i < n; i++) {
        lp[i + 1] = lp[i] + diag[i] - pntr[i] + 1;
        up[i + 1] = up[i] + pntr[i + 1] - diag[i];
    }
    for (int i = 0; i < n; i++) {
        memcpy(li + lp[i], indx + pntr[i], sizeof(int) * (size_t)(lp[i + 1] - lp[i]));
        memcpy(ui + up[i], indx + diag[i], sizeof(int) * (size_t)(up[i + 1] - up[i]));
    }
}

int or_levels(int n, const int *pntr, const int *indx, const int *diag, char uplo, int *level) {
    int nlev = 0;
    if (uplo == 'L' || uplo == 'l') {
        for (int i = 0; i < n; i++) {
            int lv = 0;
            for (int p = pntr[i]; p < diag[i]; p++) {
                int c = level[indx[p]] + 1;
                if (c > lv) lv = c;
            }
            level[i] = lv;
            if (lv + 1 > nlev) nlev = lv + 1;
        }
    } else {
        for (int i = n - 1; i >= 0; i--) {
            int lv = 0;
            for (int p = diag[i] + 1; p < pntr[i + 1]; p++) {
                int c = level[indx[p]] + 1;
                if (c > lv) lv = c;
            }
            level[i] = lv;
            if (lv + 1 > nlev) nlev = lv + 1;
        }
    }
    return nlev;
}

/* factorize_ilu_array, sparse/hala_sparse_utils.hpp:229-255: for every pivot row i, every later
 * row j holding column i is scaled and updated.  O(n^2); only for small matrices. */
void or_ilu_factor_pivot_d(int n, const int *pntr, const int *indx, const int *diag, double *ilu) {
    for (int i = 0; i < n; i++) {
        double u = ilu[diag[i]];
        for (int j = i + 1; j < n; j++) {
            int jc = pntr[j];
            while (jc < pntr[j + 1] && indx[jc] < i) jc++;
            if (jc < pntr[j + 1] && indx[jc] == i) {
                ilu[jc] /= u;
                double l = ilu[jc];
                int ik = diag[i] + 1, jk = jc + 1;
                while (ik < pntr[i + 1] && jk < pntr[j + 1]) {
                    if (indx[ik] == indx[jk]) { ilu[jk] -= l * ilu[ik]; ik++; jk++; }
                    else if (indx[ik] < indx[jk]) ik++;
                    else jk++;
                }
            }
        }
    }
}

uint16_t or_f32_to_bf16(float v) {
    uint32_t u;
    memcpy(&u, &v, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u); /* quiet NaN */
    u += 0x7fffu + ((u >> 16) & 1u);                                            /* nearest-even */
    return (uint16_t)(u >> 16);
}

float or_bf16_to_f32(uint16_t v) {
    uint32_t u = (uint32_t)v << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

/* bf16 values, fp32 vectors and accumulation; same loop order as sparse_gemv_array */
void or_spmv_bf16f32(char trans, int m, int ncols, float alpha, const int *pntr, const int *indx,
                     const uint16_t *vals, const float *x, float beta, float *y) {
    if (trans == 'N' || trans == 'n') {
        for (int i = 0; i < m; i++) {
            float sum = 0;
            for (int j = pntr[i]; j < pntr[i + 1]; j++) sum += or_bf16_to_f32(vals[j]) * x[indx[j]];
            y[i] = (beta == 0) ? alpha * sum : alpha * sum + beta * y[i];
        }
    } else {
        for (int c = 0; c < ncols; c++) y[c] = (beta == 0) ? 0.0f : beta * y[c];
        for (int i = 0; i < m; i++)
            for (int j = pntr[i]; j < pntr[i + 1]; j++)
                y[indx[j]] += alpha * x[i] * or_bf16_to_f32(vals[j]);
    }
}

#define OT double
#define OS d
#define OSQRT sqrt
#define OFABS fabs
#include "hala_oracle_impl.h"
#undef OT
#undef OS
#undef OSQRT
#undef OFABS

#define OT float
#define OS f
#define OSQRT sqrtf
#define OFABS fabsf
#include "hala_oracle_impl.h"
#undef OT
#undef OS
#undef OSQRT
#undef OFABS

static double dnorm(int n, const double *x) {
    double s = 0;
    for (int i = 0; i < n; i++) s += x[i] * x[i];
    return sqrt(s);
}

/* FP32 ILU(0) apply with FP64 pivots: off-diagonal updates in float; x_i times the pivot's
 * reciprocal, formed in double and rounded to float once. */
static void ilu_apply_mixed(int n, const int *pntr, const int *indx, const int *diag,
                            const float *ilu32, const double *piv, float *x) {
    for (int i = 1; i < n; i++)
        for (int j = pntr[i]; j < diag[i]; j++) x[i] -= ilu32[j] * x[indx[j]];
    for (int i = n - 1; i >= 0; i--) {
        for (int j = diag[i] + 1; j < pntr[i + 1]; j++) x[i] -= ilu32[j] * x[indx[j]];
        x[i] = x[i] * (float)(1.0 / piv[i]);
    }
}

void or_ilu_apply_mixed(int n, const int *pntr, const int *indx, const int *diag, const float *ilu32,
                        const double *piv, float *x) {
    ilu_apply_mixed(n, pntr, indx, diag, ilu32, piv, x);
}

/* Iterative refinement (outer FP64, inner FP32 ILU(0)-PCG following solve_cg_core's order;
 * inner dot products accumulate in double). */
int or_ir_pcg(int n, const int *pntr, const int *indx, const double *vals, const float *vals32,
              const int *diag, const float *ilu32, const double *piv, const double *b, double *x,
              double tol, double inner_rtol, int max_inner, int max_outer, int *outer_out) {
    size_t nd = sizeof(double) * (size_t)n, nf = sizeof(float) * (size_t)n;
    double *r = (double *)malloc(nd);
    float *rf = (float *)malloc(nf), *d = (float *)malloc(nf), *p = (float *)malloc(nf);
    float *Ap = (float *)malloc(nf), *z = (float *)malloc(nf);
    int total = 0, outer = 0;
    for (;;) {
        or_spmv_d('N', n, n, 1.0, pntr, indx, vals, x, 0.0, r);
        for (int i = 0; i < n; i++) r[i] = b[i] - r[i];
        double res = dnorm(n, r);
        if (res < tol || res == 0 || outer >= max_outer) break;   /* 0: x is exact */
        for (int i = 0; i < n; i++) { rf[i] = (float)r[i]; d[i] = 0.0f; }
        /* inner PCG on A32 d = rf, x0 = 0 */
        double rn0 = 0;
        for (int i = 0; i < n; i++) rn0 += (double)rf[i] * rf[i];
        rn0 = sqrt(rn0);
        float *rr = rf;
        memcpy(z, rr, nf);
        ilu_apply_mixed(n, pntr, indx, diag, ilu32, piv, z);
        memcpy(p, z, nf);
        double zr = 0;
        for (int i = 0; i < n; i++) zr += (double)rr[i] * z[i];
        int it = 0;
        for (;;) {
            or_spmv_f('N', n, n, 1.0f, pntr, indx, vals32, p, 0.0f, Ap);
            it++;
            double pap = 0;
            for (int i = 0; i < n; i++) pap += (double)p[i] * Ap[i];
            float a = (float)(zr / pap);
            for (int i = 0; i < n; i++) d[i] += a * p[i];
            for (int i = 0; i < n; i++) rr[i] -= a * Ap[i];
            double rn = 0;
            for (int i = 0; i < n; i++) rn += (double)rr[i] * rr[i];
            rn = sqrt(rn);
            if (it >= max_inner || rn < inner_rtol * rn0) break;
            memcpy(z, rr, nf);
            ilu_apply_mixed(n, pntr, indx, diag, ilu32, piv, z);
            double nzr = 0;
            for (int i = 0; i < n; i++) nzr += (double)rr[i] * z[i];
            float bt = (float)(nzr / zr);
            for (int i = 0; i < n; i++) p[i] = bt * p[i] + z[i];
            zr = nzr;
        }
        total += it;
        for (int i = 0; i < n; i++) x[i] += (double)d[i];
        outer++;
    }
    if (outer_out) *outer_out = outer;
    free(r); free(rf); free(d); free(p); free(Ap); free(z);
    return total;
}

/* Givens helpers of the refinement's inner GMRES: drotg / drot in double, as or_gmres_d. */
static void ir_rotg(double *a, double *b, double *c, double *s) {
    double roe = (fabs(*a) > fabs(*b)) ? *a : *b;
    double scale = fabs(*a) + fabs(*b), r, zz;
    if (scale == 0) { *c = 1; *s = 0; r = 0; zz = 0; }
    else {
        r = scale * sqrt((*a / scale) * (*a / scale) + (*b / scale) * (*b / scale));
        if (roe < 0) r = -r;
        *c = *a / r; *s = *b / r;
        zz = 1;
        if (fabs(*a) > fabs(*b)) zz = *s;
        if (fabs(*b) >= fabs(*a) && *c != 0) zz = 1 / *c;
    }
    *a = r; *b = zz;
}

static void ir_rot(double *x, double *y, double c, double s) {
    double t = c * *x + s * *y;
    *y = c * *y - s * *x;
    *x = t;
}

/* Inner solve of or_ir_gmres: solve_gmres (hex/solvers/hala_solvers_gmres.hpp:127-230) on the
 * FP32 system from d = 0, with FP32 vectors and basis, inner products and norms accumulated in
 * double, the rotations, the residual estimate and tpsv in double, and the stopping threshold
 * rel * (first preconditioned residual).  Returns the operator applications. */
static int ir_gmres_inner(int n, const int *pntr, const int *indx, const float *vals32, const int *diag,
                          const float *ilu32, const double *piv, int restart, const float *b, float *d,
                          double rel, int max_cycles) {
    size_t nf = sizeof(float) * (size_t)n;
    float *t = (float *)malloc(nf), *r = (float *)malloc(nf), *W = (float *)malloc(nf * (size_t)restart);
    double *H = (double *)malloc(sizeof(double) * (size_t)restart * (restart + 1));
    double *S = (double *)malloc(sizeof(double) * (restart + 1)), *Cc = (double *)malloc(sizeof(double) * (restart + 1));
    double *Z = (double *)malloc(sizeof(double) * (restart + 1)), *cf = (double *)malloc(sizeof(double) * (restart + 1));
    double tol = 0, inner_res = 0, outer_res = 1;
    int total = 0, cycles = 0, first = 1;
    while (max_cycles > 0) {
        /* t = b - A d ; r = P^-1 t ; beta = ||r|| */
        memcpy(t, b, nf);
        or_spmv_f('N', n, n, -1.0f, pntr, indx, vals32, d, 1.0f, t);
        memcpy(r, t, nf);
        ilu_apply_mixed(n, pntr, indx, diag, ilu32, piv, r);
        double s2 = 0;
        for (int i = 0; i < n; i++) s2 += (double)r[i] * r[i];
        double beta = sqrt(s2);
        if (first) { first = 0; if (rel * beta > tol) tol = rel * beta; }
        total++;
        inner_res = beta;
        Z[0] = beta;
        int nh = 0, k = 0;
        if (beta > tol) {
            float sc = (float)(1.0 / beta);
            for (int i = 0; i < n; i++) { r[i] *= sc; W[i] = r[i]; }
        }
        while (inner_res > tol && k < restart) {
            or_spmv_f('N', n, n, 1.0f, pntr, indx, vals32, r, 0.0f, t);
            memcpy(r, t, nf);
            ilu_apply_mixed(n, pntr, indx, diag, ilu32, piv, r);
            for (int j = 0; j <= k; j++) {
                double s = 0;
                for (int i = 0; i < n; i++) s += (double)W[(size_t)j * n + i] * (double)r[i];
                cf[j] = s;
            }
            double rn = 0;
            for (int i = 0; i < n; i++) {
                float ri = r[i];
                for (int j = 0; j <= k; j++) ri = ri + (float)(-cf[j]) * W[(size_t)j * n + i];
                r[i] = ri;
                rn += (double)ri * ri;
            }
            double nrm = sqrt(rn);
            for (int i = 0; i < k; i++) ir_rot(&cf[i], &cf[i + 1], Cc[i], S[i]);
            double bt = nrm, ic, is;
            ir_rotg(&cf[k], &bt, &ic, &is);
            for (int j = 0; j <= k; j++) H[nh++] = cf[j];
            S[k] = is; Cc[k] = ic;
            inner_res = fabs(is * Z[k]);
            total++;
            k++;
            if (inner_res > tol && k < restart) {
                Z[k] = 0;
                ir_rot(&Z[k - 1], &Z[k], ic, is);
                float sc = (float)(1.0 / nrm);
                for (int i = 0; i < n; i++) { r[i] *= sc; W[(size_t)k * n + i] = r[i]; }
            }
        }
        if (nh > 0) {
            long kk = (long)k * (k + 1) / 2 - 1;
            for (int j = k - 1; j >= 0; j--) {
                if (Z[j] != 0) {
                    Z[j] /= H[kk];
                    double tt = Z[j];
                    long q = kk - 1;
                    for (int i = j - 1; i >= 0; i--, q--) Z[i] -= tt * H[q];
                }
                kk -= j + 1;
            }
            for (int i = 0; i < n; i++) {
                float di = d[i];
                for (int j = 0; j < k; j++) di = di + (float)Z[j] * W[(size_t)j * n + i];
                d[i] = di;
            }
        }
        cycles++;
        outer_res = inner_res;
        if (!(outer_res > tol && cycles < max_cycles)) break;
    }
    free(t); free(r); free(W); free(H); free(S); free(Cc); free(Z); free(cf);
    return total;
}

/* Mixed-precision GMRES (no reference counterpart): outer r = b - A x in FP64, inner GMRES(restart)
 * in FP32 (ir_gmres_inner) with the FP32 ILU(0) and FP64 pivots, each sweep to
 * rel = min(0.5, max(inner_rtol, 0.5 tol / ||r||)) of its first preconditioned residual,
 * x += d in FP64.  Stops when ||b - A x|| < tol.  Returns the inner applications; *outer_out
 * gets the sweeps. */
int or_ir_gmres(int n, const int *pntr, const int *indx, const double *vals, const float *vals32,
                const int *diag, const float *ilu32, const double *piv, int restart, const double *b,
                double *x, double tol, double inner_rtol, int max_inner, int max_outer, int *outer_out) {
    size_t nd = sizeof(double) * (size_t)n, nf = sizeof(float) * (size_t)n;
    double *r = (double *)malloc(nd);
    float *rf = (float *)malloc(nf), *d = (float *)malloc(nf);
    int total = 0, outer = 0;
    const int cycles = (max_inner + restart - 1) / restart;
    for (;;) {
        or_spmv_d('N', n, n, 1.0, pntr, indx, vals, x, 0.0, r);
        for (int i = 0; i < n; i++) r[i] = b[i] - r[i];
        double res = dnorm(n, r);
        if (res < tol || res == 0 || outer >= max_outer || res != res) break;
        for (int i = 0; i < n; i++) { rf[i] = (float)r[i]; d[i] = 0.0f; }
        double rel = 0.5 * tol / res;
        if (rel < inner_rtol) rel = inner_rtol;
        if (rel > 0.5) rel = 0.5;
        total += ir_gmres_inner(n, pntr, indx, vals32, diag, ilu32, piv, restart, rf, d, rel, cycles);
        for (int i = 0; i < n; i++) x[i] += (double)d[i];
        outer++;
    }
    if (outer_out) *outer_out = outer;
    free(r); free(rf); free(d);
    return total;
}

/* Mixed-precision PCG with reliable updates (no reference counterpart): one FP32 ILU(0)-PCG
 * (solve_cg_core's order, FP32 vectors, inner products in double) on the correction; whenever
 * the iterated residual falls below delta times its largest value since the last update, the
 * correction is added to x in FP64, the residual is recomputed as b - A x in FP64 and the
 * iteration continues from it with the same search direction (restarted, beta = 0, when the update
 * reduced the FP64 residual less than twice).  Stops when the FP64 residual
 * after an update is below tol (an update is forced when the iterated residual is below tol and
 * at the iteration limit).
 * Returns the iterations; *updates_out gets the number of reliable updates. */
int or_ru_pcg(int n, const int *pntr, const int *indx, const double *vals, const float *vals32,
              const int *diag, const float *ilu32, const double *piv, const double *b, double *x,
              double tol, double delta, int max_iter, int *updates_out) {
    if (updates_out) *updates_out = 0;
    if (n <= 0) return 0;
    size_t nd = sizeof(double) * (size_t)n, nf = sizeof(float) * (size_t)n;
    double *r64 = (double *)malloc(nd);
    float *r = (float *)malloc(nf), *d = (float *)malloc(nf), *p = (float *)malloc(nf);
    float *Ap = (float *)malloc(nf), *z = (float *)malloc(nf);
    int it = 0, updates = 0;
    or_spmv_d('N', n, n, 1.0, pntr, indx, vals, x, 0.0, r64);
    for (int i = 0; i < n; i++) r64[i] = b[i] - r64[i];
    double rn = dnorm(n, r64), rmax = rn, last = rn;
    int restart = 0;
    if (rn < tol || rn == 0) { free(r64); free(r); free(d); free(p); free(Ap); free(z); if (updates_out) *updates_out = 0; return 0; }
    for (int i = 0; i < n; i++) { r[i] = (float)r64[i]; d[i] = 0.0f; }
    memcpy(z, r, nf);
    ilu_apply_mixed(n, pntr, indx, diag, ilu32, piv, z);
    memcpy(p, z, nf);
    double zr = 0;
    for (int i = 0; i < n; i++) zr += (double)r[i] * z[i];
    while (it < max_iter) {
        or_spmv_f('N', n, n, 1.0f, pntr, indx, vals32, p, 0.0f, Ap);
        it++;
        double pap = 0;
        for (int i = 0; i < n; i++) pap += (double)p[i] * Ap[i];
        float a = (float)(zr / pap);
        for (int i = 0; i < n; i++) d[i] += a * p[i];
        double s = 0;
        for (int i = 0; i < n; i++) { r[i] -= a * Ap[i]; s += (double)r[i] * r[i]; }
        rn = sqrt(s);
        if (rn > rmax) rmax = rn;
        if (rn < delta * rmax || rn < tol || !(rn == rn) || it >= max_iter) {
            /* reliable update: x += d (FP64), r = b - A x (FP64) */
            for (int i = 0; i < n; i++) { x[i] += (double)d[i]; d[i] = 0.0f; }
            or_spmv_d('N', n, n, 1.0, pntr, indx, vals, x, 0.0, r64);
            s = 0;
            for (int i = 0; i < n; i++) { r64[i] = b[i] - r64[i]; s += r64[i] * r64[i]; r[i] = (float)r64[i]; }
            rn = sqrt(s);
            rmax = rn;
            updates++;
            if (rn < tol || !(rn == rn) || it >= max_iter) break;
            /* the update reduced the true residual less than twice: the kept directions are stale,
             * restart the recurrence from the new residual */
            restart = rn > 0.5 * last;
            last = rn;
        }
        memcpy(z, r, nf);
        ilu_apply_mixed(n, pntr, indx, diag, ilu32, piv, z);
        double nzr = 0;
        for (int i = 0; i < n; i++) nzr += (double)r[i] * z[i];
        float bt = restart ? 0.0f : (float)(nzr / zr);
        restart = 0;
        for (int i = 0; i < n; i++) p[i] = bt * p[i] + z[i];
        zr = nzr;
    }
    if (updates_out) *updates_out = updates;
    free(r64); free(r); free(d); free(p); free(Ap); free(z);
    return it;
}
