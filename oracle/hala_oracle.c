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
        if (res < tol || outer >= max_outer) break;
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
