/*
 * Type-generic body of the CPU oracle; included twice by hala_oracle.c with
 * OT (value type), OS (suffix), OSQRT and OFABS defined.  Test infrastructure only.
 */
#define OR_CAT2(a, b) a##_##b
#define OR_CAT(a, b) OR_CAT2(a, b)
#define OR_FN(name) OR_CAT(name, OS)

/* sparse_gemv_array, sparse/hala_sparse_utils.hpp:104-119.
 * 'N': y[i] = alpha * (sequential row sum) + beta * y[i]; beta == 0 does not read y (BLAS rule).
 * 'T'/'C': y = beta*y (scal), then y[indx[j]] += alpha * x[i] * vals[j] in row order. */
void OR_FN(or_spmv)(char trans, int m, int ncols, OT alpha, const int *pntr, const int *indx,
                    const OT *vals, const OT *x, OT beta, OT *y) {
    if (trans == 'N' || trans == 'n') {
        for (int i = 0; i < m; i++) {
            OT sum = 0;
            for (int j = pntr[i]; j < pntr[i + 1]; j++) sum += vals[j] * x[indx[j]];
            y[i] = (beta == 0) ? alpha * sum : alpha * sum + beta * y[i];
        }
    } else {
        for (int c = 0; c < ncols; c++) y[c] = (beta == 0) ? (OT)0 : beta * y[c];
        for (int i = 0; i < m; i++)
            for (int j = pntr[i]; j < pntr[i + 1]; j++) y[indx[j]] += alpha * x[i] * vals[j];
    }
}

/* split_values_array, sparse/hala_sparse_utils.hpp:201-221 */
void OR_FN(or_split_values)(char uplo, char diag, int n, const int *pntr, const OT *vals,
                            const int *up, const int *lp, OT *uv, OT *lv) {
    OT alpha = (diag == 'N' || diag == 'n') ? (OT)0 : (OT)1;
    for (int i = 0; i < n; i++) {
        int nl = lp[i + 1] - lp[i];
        for (int k = 0; k < nl; k++) lv[lp[i] + k] = vals[pntr[i] + k];
        for (int k = 0; k < up[i + 1] - up[i]; k++) uv[up[i] + k] = vals[pntr[i] + nl - 1 + k];
        if (uplo == 'L' || uplo == 'l') uv[up[i]] = alpha;
        else lv[lp[i + 1] - 1] = alpha;
    }
}

/* Row-wise IKJ ILU(0).  For row i, pivots k = indx[p] (p in [pntr_i, diag_i), ascending):
 *   a_ik /= a_kk ; a_ij -= a_ik * a_kj for every j > k present in both row i and row k.
 * Each entry receives the same updates in the same order as the pivot-row loop of
 * factorize_ilu_array (sparse/hala_sparse_utils.hpp:229-255), so the result is bit-identical.
 * Returns 0, or -(i+1) when the pivot of row i is exactly zero (the reference divides anyway). */
int OR_FN(or_ilu_factor)(int n, const int *pntr, const int *indx, const int *diag, OT *ilu) {
    int status = 0;
    for (int i = 0; i < n; i++) {
        for (int p = pntr[i]; p < diag[i]; p++) {
            int k = indx[p];
            OT u = ilu[diag[k]];
            if (u == 0 && status == 0) status = -(k + 1);
            ilu[p] /= u;
            OT l = ilu[p];
            int kk = diag[k] + 1, q = p + 1;
            while (kk < pntr[k + 1] && q < pntr[i + 1]) {
                if (indx[kk] == indx[q]) { ilu[q] -= l * ilu[kk]; kk++; q++; }
                else if (indx[kk] < indx[q]) kk++;
                else q++;
            }
        }
        if (ilu[diag[i]] == 0 && status == 0) status = -(i + 1);
    }
    return status;
}

/* apply_ilu_array, sparse/hala_sparse_utils.hpp:263-276 */
void OR_FN(or_ilu_apply)(int n, const int *pntr, const int *indx, const int *diag, const OT *ilu,
                         OT *x) {
    for (int i = 1; i < n; i++)
        for (int j = pntr[i]; j < diag[i]; j++) x[i] -= ilu[j] * x[indx[j]];
    for (int i = n - 1; i >= 0; i--) {
        for (int j = diag[i] + 1; j < pntr[i + 1]; j++) x[i] -= ilu[j] * x[indx[j]];
        x[i] /= ilu[diag[i]];
    }
}

/* (L U)^-T x = L^-T (U^-T x), written as the column-oriented scatter of the reference's
 * transposed triangular solve (sparse_trsv_array 'T', sparse/hala_sparse_utils.hpp:318-335):
 *   U^T w = x : rows ascending,  w_i = (x_i - t_i) / u_ii,  t_j += w_i * u_ij  (j > i)
 *   L^T z = w : rows descending, z_i =  w_i - s_i,          s_j += z_i * l_ij  (j < i)
 * Accumulators start at zero, contributions arrive in row order. */
void OR_FN(or_ilu_apply_t)(int n, const int *pntr, const int *indx, const int *diag, const OT *ilu,
                           OT *x) {
    OT *t = (OT *)calloc((size_t)n, sizeof(OT));
    for (int i = 0; i < n; i++) {
        x[i] = (x[i] - t[i]) / ilu[diag[i]];
        for (int j = diag[i] + 1; j < pntr[i + 1]; j++) t[indx[j]] += x[i] * ilu[j];
    }
    for (int i = 0; i < n; i++) t[i] = 0;
    for (int i = n - 1; i >= 0; i--) {
        x[i] = x[i] - t[i];
        for (int j = pntr[i]; j < diag[i]; j++) t[indx[j]] += x[i] * ilu[j];
    }
    free(t);
}

/* sparse_trsv_array, sparse/hala_sparse_utils.hpp:284-336 (real types: 'C' == 'T').
 * The triangular CSR holds the diagonal last ('L') or first ('U') in every row. */
void OR_FN(or_trsv)(char uplo, char diag, char trans, int n, OT alpha, const int *pntr,
                    const int *indx, const OT *vals, const OT *b, OT *x) {
    int unit = (diag == 'U' || diag == 'u');
    int lower = (uplo == 'L' || uplo == 'l');
    if (trans == 'N' || trans == 'n') {
        if (lower) {
            x[0] = unit ? alpha * b[0] : alpha * b[0] / vals[0];
            for (int i = 1; i < n; i++) {
                OT s = 0;
                for (int j = pntr[i]; j < pntr[i + 1] - 1; j++) s += vals[j] * x[indx[j]];
                x[i] = unit ? (alpha * b[i] - s) : (alpha * b[i] - s) / vals[pntr[i + 1] - 1];
            }
        } else {
            x[n - 1] = unit ? alpha * b[n - 1] : alpha * b[n - 1] / vals[pntr[n] - 1];
            for (int i = n - 2; i >= 0; i--) {
                OT s = 0;
                for (int j = pntr[i] + 1; j < pntr[i + 1]; j++) s += vals[j] * x[indx[j]];
                x[i] = unit ? (alpha * b[i] - s) : (alpha * b[i] - s) / vals[pntr[i]];
            }
        }
    } else {
        for (int i = 0; i < n; i++) x[i] = 0;
        if (lower) {
            for (int i = n - 1; i >= 0; i--) {
                x[i] = unit ? (alpha * b[i] - x[i]) : (alpha * b[i] - x[i]) / vals[pntr[i + 1] - 1];
                for (int j = pntr[i]; j < pntr[i + 1] - 1; j++) x[indx[j]] += x[i] * vals[j];
            }
        } else {
            for (int i = 0; i < n; i++) {
                x[i] = unit ? (alpha * b[i] - x[i]) : (alpha * b[i] - x[i]) / vals[pntr[i]];
                for (int j = pntr[i] + 1; j < pntr[i + 1]; j++) x[indx[j]] += x[i] * vals[j];
            }
        }
    }
}

OT OR_FN(or_dot)(int n, const OT *x, const OT *y) {
    OT s = 0;
    for (int i = 0; i < n; i++) s += x[i] * y[i];
    return s;
}

/* netlib scaled sum of squares */
OT OR_FN(or_nrm2)(int n, const OT *x) {
    if (n < 1) return 0;
    if (n == 1) return OFABS(x[0]);
    OT scale = 0, ssq = 1;
    for (int i = 0; i < n; i++) {
        if (x[i] != 0) {
            OT a = OFABS(x[i]);
            if (scale < a) { ssq = 1 + ssq * (scale / a) * (scale / a); scale = a; }
            else ssq += (a / scale) * (a / scale);
        }
    }
    return scale * OSQRT(ssq);
}

static void OR_FN(or_precond)(int n, const int *pntr, const int *indx, const int *diag,
                              const OT *ilu, const OT *in, OT *out) {
    memcpy(out, in, sizeof(OT) * (size_t)n);
    if (ilu) OR_FN(or_ilu_apply)(n, pntr, indx, diag, ilu, out);
}

/* solve_cg_core, hex/solvers/hala_solvers_cg.hpp:92-156 with the lambdas of solve_cg (:207-226) */
int OR_FN(or_cg)(int n, const int *pntr, const int *indx, const OT *vals, const int *diag,
                 const OT *ilu, const OT *b, OT *x, OT tol, int max_iter, OT *res_out) {
    size_t sz = sizeof(OT) * (size_t)n;
    OT *r = (OT *)malloc(sz), *p = (OT *)malloc(sz), *Ap = (OT *)malloc(sz), *z = (OT *)malloc(sz);
    memcpy(r, b, sz);
    OR_FN(or_spmv)('N', n, n, 1, pntr, indx, vals, x, 0, p);
    for (int i = 0; i < n; i++) r[i] += (OT)(-1.0) * p[i];          /* axpy(-1, p, r) */
    OR_FN(or_precond)(n, pntr, indx, diag, ilu, r, z);
    memcpy(p, z, sz);
    OT zr = OR_FN(or_dot)(n, r, z);
    int iterations = 1;
    OT res = 0;
    for (;;) {
        OR_FN(or_spmv)('N', n, n, 1, pntr, indx, vals, p, 0, Ap);
        iterations++;
        OT nzr = OR_FN(or_dot)(n, p, Ap);
        OT a = zr / nzr;
        for (int i = 0; i < n; i++) x[i] += a * p[i];              /* axpy(a, p, x) */
        OT ma = -a;
        for (int i = 0; i < n; i++) r[i] += ma * Ap[i];            /* axpy(-a, Ap, r) */
        res = OR_FN(or_nrm2)(n, r);
        if (iterations == max_iter || res < tol) break;
        OR_FN(or_precond)(n, pntr, indx, diag, ilu, r, z);
        nzr = OR_FN(or_dot)(n, r, z);
        a = nzr / zr;
        for (int i = 0; i < n; i++) p[i] *= a;                     /* scal(a, p) */
        for (int i = 0; i < n; i++) p[i] += z[i];                  /* axpy(1, z, p) */
        zr = nzr;
    }
    if (res_out) *res_out = res;
    free(r); free(p); free(Ap); free(z);
    return iterations;
}

/* solve_batch_cg / solve_batch_cg_ilu, hex/solvers/hala_solvers_cg_batch.hpp:68-248: the
 * recurrence of solve_cg_core on n x nrhs column-major blocks with one scalar per column
 * (batch_dot, vdivide, batch_axpy, batch_scal, wax/hala_blas_extensions.hpp:30-140); stops when
 * iterations == max_iter or batch_max_norm2(r) = sqrt(max_c <r_c, r_c>) < tol (:369-380). */
int OR_FN(or_batch_cg)(int n, const int *pntr, const int *indx, const OT *vals, const int *diag,
                       const OT *ilu, int nrhs, const OT *b, OT *x, OT tol, int max_iter, OT *res_out) {
    const size_t tot = (size_t)n * nrhs, sz = sizeof(OT) * tot;
    OT *r = (OT *)malloc(sz), *p = (OT *)malloc(sz), *Ap = (OT *)malloc(sz), *z = (OT *)malloc(sz);
    OT *zr = (OT *)malloc(sizeof(OT) * nrhs), *nzr = (OT *)malloc(sizeof(OT) * nrhs), *a = (OT *)malloc(sizeof(OT) * nrhs);
    memcpy(r, b, sz);
    for (int c = 0; c < nrhs; c++) OR_FN(or_spmv)('N', n, n, 1, pntr, indx, vals, x + (size_t)c * n, 0, p + (size_t)c * n);
    for (size_t i = 0; i < tot; i++) r[i] += (OT)(-1.0) * p[i];                  /* axpy(-1, p, r) */
    for (int c = 0; c < nrhs; c++) OR_FN(or_precond)(n, pntr, indx, diag, ilu, r + (size_t)c * n, z + (size_t)c * n);
    memcpy(p, z, sz);
    for (int c = 0; c < nrhs; c++) zr[c] = OR_FN(or_dot)(n, r + (size_t)c * n, z + (size_t)c * n);
    int iterations = 1;
    OT res = 0;
    for (;;) {
        for (int c = 0; c < nrhs; c++)
            OR_FN(or_spmv)('N', n, n, 1, pntr, indx, vals, p + (size_t)c * n, 0, Ap + (size_t)c * n);
        iterations++;
        for (int c = 0; c < nrhs; c++) nzr[c] = OR_FN(or_dot)(n, p + (size_t)c * n, Ap + (size_t)c * n);
        for (int c = 0; c < nrhs; c++) a[c] = zr[c] / nzr[c];                     /* vdivide */
        for (int c = 0; c < nrhs; c++)
            for (int i = 0; i < n; i++) x[(size_t)c * n + i] += ((OT)1.0 * a[c]) * p[(size_t)c * n + i];
        for (int c = 0; c < nrhs; c++)
            for (int i = 0; i < n; i++) r[(size_t)c * n + i] += ((OT)(-1.0) * a[c]) * Ap[(size_t)c * n + i];
        OT mx = 0;
        for (int c = 0; c < nrhs; c++) {
            OT d = OR_FN(or_dot)(n, r + (size_t)c * n, r + (size_t)c * n);
            if (OFABS(d) > mx) mx = OFABS(d);
        }
        res = OSQRT(mx);
        if (iterations == max_iter || res < tol) break;
        for (int c = 0; c < nrhs; c++) OR_FN(or_precond)(n, pntr, indx, diag, ilu, r + (size_t)c * n, z + (size_t)c * n);
        for (int c = 0; c < nrhs; c++) nzr[c] = OR_FN(or_dot)(n, r + (size_t)c * n, z + (size_t)c * n);
        for (int c = 0; c < nrhs; c++) a[c] = nzr[c] / zr[c];
        for (int c = 0; c < nrhs; c++)
            for (int i = 0; i < n; i++) p[(size_t)c * n + i] *= a[c];               /* batch_scal */
        for (size_t i = 0; i < tot; i++) p[i] += z[i];                             /* axpy(1, z, p) */
        memcpy(zr, nzr, sizeof(OT) * nrhs);
    }
    if (res_out) *res_out = res;
    free(r); free(p); free(Ap); free(z); free(zr); free(nzr); free(a);
    return iterations;
}

static void OR_FN(or_rotg)(OT *a, OT *b, OT *c, OT *s) {
    OT roe = (OFABS(*a) > OFABS(*b)) ? *a : *b;
    OT scale = OFABS(*a) + OFABS(*b), r, zz;
    if (scale == 0) { *c = 1; *s = 0; r = 0; zz = 0; }
    else {
        r = scale * OSQRT((*a / scale) * (*a / scale) + (*b / scale) * (*b / scale));
        if (roe < 0) r = -r;
        *c = *a / r; *s = *b / r;
        zz = 1;
        if (OFABS(*a) > OFABS(*b)) zz = *s;
        if (OFABS(*b) >= OFABS(*a) && *c != 0) zz = 1 / *c;
    }
    *a = r; *b = zz;
}

static void OR_FN(or_rot)(OT *x, OT *y, OT c, OT s) {
    OT t = c * *x + s * *y;
    *y = c * *y - s * *x;
    *x = t;
}

/* solve_gmres, hex/solvers/hala_solvers_gmres.hpp:127-230.  Reproduces the reference exactly,
 * including that the last Givens rotation is not applied to Z when the inner loop stops
 * (the rotation of Z happens only when the basis is expanded, :210-216). */
int OR_FN(or_gmres)(int n, const int *pntr, const int *indx, const OT *vals, const int *diag,
                    const OT *ilu, int restart, const OT *b, OT *x, OT tol, int max_iter) {
    size_t sz = sizeof(OT) * (size_t)n;
    OT *t = (OT *)malloc(sz), *r = (OT *)malloc(sz);
    OT *W = (OT *)malloc(sz * (size_t)restart);
    OT *H = (OT *)malloc(sizeof(OT) * (size_t)restart * (restart + 1));
    OT *S = (OT *)malloc(sizeof(OT) * (restart + 1)), *C = (OT *)malloc(sizeof(OT) * (restart + 1));
    OT *Z = (OT *)malloc(sizeof(OT) * (restart + 1)), *cf = (OT *)malloc(sizeof(OT) * (restart + 1));
    OT inner_res, outer_res = tol + 1;
    int total = 0, outer = 0;
    while (outer_res > tol && outer < max_iter) {
        int nh = 0, nz = 0;
        memcpy(t, b, sz);
        OR_FN(or_spmv)('N', n, n, -1, pntr, indx, vals, x, 1, t);
        OR_FN(or_precond)(n, pntr, indx, diag, ilu, t, r);
        total++;
        inner_res = OR_FN(or_nrm2)(n, r);
        OT sc = (OT)(1.0 / (double)inner_res);   /* scal(engine, 1.0 / inner_res, r) */
        for (int i = 0; i < n; i++) r[i] *= sc;
        Z[nz++] = inner_res;
        memcpy(W, r, sz);
        int k = 0;
        while (inner_res > tol && k < restart) {
            OR_FN(or_spmv)('N', n, n, 1, pntr, indx, vals, r, 0, t);
            OR_FN(or_precond)(n, pntr, indx, diag, ilu, t, r);
            total++;
            /* krylov_project: cf = W^T r ; r -= W cf  (gemv T then gemv N, :47-50) */
            for (int j = 0; j <= k; j++) {
                OT s = 0;
                for (int i = 0; i < n; i++) s += W[(size_t)j * n + i] * r[i];
                cf[j] = s;
            }
            for (int j = 0; j <= k; j++) {
                OT tj = (OT)(-1.0) * cf[j];
                for (int i = 0; i < n; i++) r[i] += tj * W[(size_t)j * n + i];
            }
            OT nrm = OR_FN(or_nrm2)(n, r);
            sc = (OT)(1.0 / (double)nrm);
            for (int i = 0; i < n; i++) r[i] *= sc;
            for (int i = 0; i < k; i++) OR_FN(or_rot)(&cf[i], &cf[i + 1], C[i], S[i]);
            OT beta = nrm, ic, is;
            OR_FN(or_rotg)(&cf[k], &beta, &ic, &is);
            for (int j = 0; j <= k; j++) H[nh++] = cf[j];
            S[k] = is; C[k] = ic;
            inner_res = OFABS(S[k] * Z[nz - 1]);
            k++;
            if (inner_res > tol && k < restart) {
                memcpy(W + (size_t)k * n, r, sz);
                Z[nz++] = 0;
                OR_FN(or_rot)(&Z[k - 1], &Z[k], C[k - 1], S[k - 1]);
            }
        }
        if (nh > 0) {
            /* tpsv('U','N','N', nz, H, Z): packed upper, column-oriented back substitution */
            long kk = (long)nz * (nz + 1) / 2 - 1;
            for (int j = nz - 1; j >= 0; j--) {
                if (Z[j] != 0) {
                    Z[j] /= H[kk];
                    OT tt = Z[j];
                    long q = kk - 1;
                    for (int i = j - 1; i >= 0; i--, q--) Z[i] -= tt * H[q];
                }
                kk -= j + 1;
            }
            /* krylov_combine: x += W Z (gemv N, column by column) */
            for (int j = 0; j < nz; j++) {
                OT tj = Z[j];
                for (int i = 0; i < n; i++) x[i] += tj * W[(size_t)j * n + i];
            }
        }
        outer++;
        outer_res = inner_res;
    }
    free(t); free(r); free(W); free(H); free(S); free(C); free(Z); free(cf);
    return total;
}

#undef OR_FN
#undef OR_CAT
#undef OR_CAT2
