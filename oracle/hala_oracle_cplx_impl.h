/*
 * Type-generic body of the complex CPU oracle; included twice by hala_oracle_cplx.c with
 * CT (complex type), RT (its real type), CS (suffix: z or c), RSQRT, RFABS, CCONJ and CABS defined.
 * Test infrastructure only.  Complex products and quotients are C99's (separately rounded
 * re = ac - bd, im = ad + bc with -ffp-contract=off; division through the runtime's complex
 * division), the same operations std::complex performs in the reference's templates.
 */
#define OC_CAT2(a, b) a##_##b
#define OC_CAT(a, b) OC_CAT2(a, b)
#define OC_FN(name) OC_CAT(name, CS)

/* sparse_gemv_array, sparse/hala_sparse_utils.hpp:104-119 with complex alpha / beta.
 * 'N': y[i] = alpha * (sequential row sum) + beta * y[i]; beta == 0 does not read y.
 * 'T' / 'C': y = beta * y, then y[indx[j]] += alpha * x[i] * op(vals[j]) in row order. */
void OC_FN(or_spmv)(char trans, int m, int ncols, const RT *alpha2, const int *pntr, const int *indx,
                    const CT *vals, const CT *x, const RT *beta2, CT *y) {
    const CT alpha = alpha2[0] + alpha2[1] * I, beta = beta2[0] + beta2[1] * I;
    if (trans == 'N' || trans == 'n') {
        for (int i = 0; i < m; i++) {
            CT s = 0;
            for (int j = pntr[i]; j < pntr[i + 1]; j++) s += vals[j] * x[indx[j]];
            y[i] = (beta == 0) ? alpha * s : alpha * s + beta * y[i];
        }
        return;
    }
    const int cj = (trans == 'C' || trans == 'c');
    for (int c = 0; c < ncols; c++) y[c] = (beta == 0) ? 0 : beta * y[c];
    for (int i = 0; i < m; i++)
        for (int j = pntr[i]; j < pntr[i + 1]; j++) y[indx[j]] += alpha * x[i] * (cj ? CCONJ(vals[j]) : vals[j]);
}

/* factorize_ilu_array, sparse/hala_sparse_utils.hpp:229-255: for every pivot row i, every later
 * row j with an entry in column i is divided and updated.  Returns the first zero pivot row + 1
 * (0: none); the factorisation runs to the end regardless, as the reference's does. */
int OC_FN(or_ilu_factor)(int n, const int *pntr, const int *indx, const int *diag, CT *ilu) {
    int zero = 0;
    for (int i = 0; i < n; i++) {
        const CT u = ilu[diag[i]];
        if (u == 0 && !zero) zero = i + 1;
        for (int j = i + 1; j < n; j++) {
            int jc = pntr[j];
            while (jc < pntr[j + 1] && indx[jc] < i) jc++;
            if (jc < pntr[j + 1] && indx[jc] == i) {
                ilu[jc] /= u;
                const CT l = ilu[jc];
                int ik = diag[i] + 1, jk = jc + 1;
                while (ik < pntr[i + 1] && jk < pntr[j + 1]) {
                    if (indx[ik] == indx[jk]) {
                        ilu[jk] -= l * ilu[ik];
                        ik++;
                        jk++;
                    } else if (indx[ik] < indx[jk]) {
                        ik++;
                    } else {
                        jk++;
                    }
                }
            }
        }
    }
    return zero;
}

/* apply_ilu_array, sparse/hala_sparse_utils.hpp:263-276 (in place) */
void OC_FN(or_ilu_apply)(int n, const int *pntr, const int *indx, const int *diag, const CT *ilu, CT *x) {
    for (int i = 1; i < n; i++)
        for (int j = pntr[i]; j < diag[i]; j++) x[i] -= ilu[j] * x[indx[j]];
    for (int i = n - 1; i >= 0; i--) {
        for (int j = diag[i] + 1; j < pntr[i + 1]; j++) x[i] -= ilu[j] * x[indx[j]];
        x[i] /= ilu[diag[i]];
    }
}

/* (LU)^-T x ('T') or (LU)^-H x ('C') in place: U^T (U^H) first, column-oriented as the transposed
 * branches of sparse_trsv_array (utils:310-334), then the unit L^T (L^H). */
void OC_FN(or_ilu_apply_t)(char trans, int n, const int *pntr, const int *indx, const int *diag, const CT *ilu,
                           CT *x) {
    const int cj = (trans == 'C' || trans == 'c');
    CT *t = (CT *)calloc((size_t)n, sizeof(CT));
    for (int i = 0; i < n; i++) {
        const CT d = cj ? CCONJ(ilu[diag[i]]) : ilu[diag[i]];
        x[i] = (x[i] - t[i]) / d;
        for (int j = diag[i] + 1; j < pntr[i + 1]; j++) t[indx[j]] += x[i] * (cj ? CCONJ(ilu[j]) : ilu[j]);
    }
    for (int i = 0; i < n; i++) t[i] = 0;
    for (int i = n - 1; i >= 0; i--) {
        x[i] = x[i] - t[i];
        for (int j = pntr[i]; j < diag[i]; j++) t[indx[j]] += x[i] * (cj ? CCONJ(ilu[j]) : ilu[j]);
    }
    free(t);
}

/* sparse_trsv_array, sparse/hala_sparse_utils.hpp:284-336 with a real alpha.  The triangular CSR
 * holds the diagonal last ('L') or first ('U') in every row. */
void OC_FN(or_trsv)(char uplo, char diag, char trans, int n, RT alpha, const int *pntr, const int *indx,
                    const CT *vals, const CT *b, CT *x) {
    const int unit = (diag == 'U' || diag == 'u'), lower = (uplo == 'L' || uplo == 'l');
    if (trans == 'N' || trans == 'n') {
        if (lower) {
            x[0] = unit ? alpha * b[0] : alpha * b[0] / vals[0];
            for (int i = 1; i < n; i++) {
                CT s = 0;
                for (int j = pntr[i]; j < pntr[i + 1] - 1; j++) s += vals[j] * x[indx[j]];
                x[i] = unit ? (alpha * b[i] - s) : (alpha * b[i] - s) / vals[pntr[i + 1] - 1];
            }
        } else {
            x[n - 1] = unit ? alpha * b[n - 1] : alpha * b[n - 1] / vals[pntr[n] - 1];
            for (int i = n - 2; i >= 0; i--) {
                CT s = 0;
                for (int j = pntr[i] + 1; j < pntr[i + 1]; j++) s += vals[j] * x[indx[j]];
                x[i] = unit ? (alpha * b[i] - s) : (alpha * b[i] - s) / vals[pntr[i]];
            }
        }
        return;
    }
    const int cj = (trans == 'C' || trans == 'c');
#define OC_V(p) (cj ? CCONJ(vals[p]) : vals[p])
    for (int i = 0; i < n; i++) x[i] = 0;
    if (lower) {
        for (int i = n - 1; i >= 0; i--) {
            x[i] = unit ? (alpha * b[i] - x[i]) : (alpha * b[i] - x[i]) / OC_V(pntr[i + 1] - 1);
            for (int j = pntr[i]; j < pntr[i + 1] - 1; j++) x[indx[j]] += x[i] * OC_V(j);
        }
    } else {
        for (int i = 0; i < n; i++) {
            x[i] = unit ? (alpha * b[i] - x[i]) : (alpha * b[i] - x[i]) / OC_V(pntr[i]);
            for (int j = pntr[i] + 1; j < pntr[i + 1]; j++) x[indx[j]] += x[i] * OC_V(j);
        }
    }
#undef OC_V
}

/* hala::dot (conjugated, the manual loop of dot_array, blas/hala_blas_1.hpp:229-246) and dotu */
void OC_FN(or_dotc)(int n, const CT *x, const CT *y, RT *out) {
    CT s = 0;
    for (int i = 0; i < n; i++) s += CCONJ(x[i]) * y[i];
    out[0] = creal(s);
    out[1] = cimag(s);
}
static CT OC_FN(dotu_)(int n, const CT *x, const CT *y) {
    CT s = 0;
    for (int i = 0; i < n; i++) s += x[i] * y[i];
    return s;
}

/* netlib dznrm2 / scnrm2 before 3.10: scaled sum of squares over the real and imaginary parts */
RT OC_FN(or_nrm2)(int n, const CT *x) {
    if (n < 1) return 0;
    RT scale = 0, ssq = 1;
    for (int i = 0; i < n; i++) {
        const RT part[2] = {creal(x[i]), cimag(x[i])};
        for (int k = 0; k < 2; k++) {
            if (part[k] != 0) {
                const RT a = RFABS(part[k]);
                if (scale < a) {
                    ssq = 1 + ssq * (scale / a) * (scale / a);
                    scale = a;
                } else {
                    ssq += (a / scale) * (a / scale);
                }
            }
        }
    }
    return scale * RSQRT(ssq);
}

static void OC_FN(precond_)(int n, const int *pntr, const int *indx, const int *diag, const CT *ilu, const CT *in,
                            CT *out) {
    memcpy(out, in, sizeof(CT) * (size_t)n);
    if (ilu) OC_FN(or_ilu_apply)(n, pntr, indx, diag, ilu, out);
}

static void OC_FN(spmv1_)(int n, const int *pntr, const int *indx, const CT *vals, const CT *x, CT *y) {
    const RT one[2] = {1, 0}, zero[2] = {0, 0};
    OC_FN(or_spmv)('N', n, n, one, pntr, indx, vals, x, zero, y);
}

/* solve_cg_core, hex/solvers/hala_solvers_cg.hpp:92-156 with the lambdas of solve_cg (:207-226):
 * dot conjugates, norm2 is dznrm2, axpy / scal as netlib zaxpy / zscal. */
int OC_FN(or_cg)(int n, const int *pntr, const int *indx, const CT *vals, const int *diag, const CT *ilu,
                 const CT *b, CT *x, RT tol, int max_iter, RT *res_out) {
    const size_t sz = sizeof(CT) * (size_t)n;
    CT *r = (CT *)malloc(sz), *p = (CT *)malloc(sz), *Ap = (CT *)malloc(sz), *z = (CT *)malloc(sz);
    memcpy(r, b, sz);
    OC_FN(spmv1_)(n, pntr, indx, vals, x, p);
    for (int i = 0; i < n; i++) r[i] += (CT)(-1.0) * p[i];   /* axpy(-1, p, r) */
    OC_FN(precond_)(n, pntr, indx, diag, ilu, r, z);
    memcpy(p, z, sz);
    RT t[2];
    OC_FN(or_dotc)(n, r, z, t);
    CT zr = t[0] + t[1] * I;
    int iterations = 1;
    RT res = 0;
    for (;;) {
        OC_FN(spmv1_)(n, pntr, indx, vals, p, Ap);
        iterations++;
        OC_FN(or_dotc)(n, p, Ap, t);
        CT nzr = t[0] + t[1] * I;
        CT a = zr / nzr;
        for (int i = 0; i < n; i++) x[i] += a * p[i];
        const CT ma = -a;
        for (int i = 0; i < n; i++) r[i] += ma * Ap[i];
        res = OC_FN(or_nrm2)(n, r);
        if (iterations == max_iter || res < tol) break;
        OC_FN(precond_)(n, pntr, indx, diag, ilu, r, z);
        OC_FN(or_dotc)(n, r, z, t);
        nzr = t[0] + t[1] * I;
        a = nzr / zr;
        for (int i = 0; i < n; i++) p[i] = a * p[i];          /* scal(a, p) */
        for (int i = 0; i < n; i++) p[i] += (CT)1.0 * z[i];   /* axpy(1, z, p) */
        zr = nzr;
    }
    if (res_out) *res_out = res;
    free(r);
    free(p);
    free(Ap);
    free(z);
    return iterations;
}

/* netlib zrotg (before 3.10): c real, s complex */
static void OC_FN(rotg_)(CT *ca, CT cb, RT *c, CT *s) {
    if (CABS(*ca) == 0) {
        *c = 0;
        *s = 1;
        *ca = cb;
        return;
    }
    const RT scale = CABS(*ca) + CABS(cb);
    const RT p = CABS(*ca / scale), q = CABS(cb / scale);
    const RT norm = scale * RSQRT(p * p + q * q);
    const CT alpha = *ca / CABS(*ca);
    *c = CABS(*ca) / norm;
    *s = alpha * CCONJ(cb) / norm;
    *ca = alpha * norm;
}
/* LAPACK zrot: x' = c x + s y, y' = c y - conj(s) x */
static void OC_FN(rot_)(CT *x, CT *y, RT c, CT s) {
    const CT t = c * *x + s * *y;
    *y = c * *y - CCONJ(s) * *x;
    *x = t;
}

/* solve_gmres, hex/solvers/hala_solvers_gmres.hpp:127-230 on complex data: krylov_project with the
 * UNCONJUGATED transpose (gemv 'T', :47-50), zrotg / zrot, ztpsv('U','N','N') and krylov_combine;
 * the last rotation is not applied to Z when the inner loop stops (:210-216), as in the reference. */
int OC_FN(or_gmres)(int n, const int *pntr, const int *indx, const CT *vals, const int *diag, const CT *ilu,
                    int restart, const CT *b, CT *x, RT tol, int max_iter) {
    const size_t sz = sizeof(CT) * (size_t)n;
    CT *t = (CT *)malloc(sz), *r = (CT *)malloc(sz), *W = (CT *)malloc(sz * (size_t)restart);
    CT *H = (CT *)malloc(sizeof(CT) * (size_t)restart * (restart + 1));
    CT *S = (CT *)malloc(sizeof(CT) * (restart + 1)), *Z = (CT *)malloc(sizeof(CT) * (restart + 1));
    CT *cf = (CT *)malloc(sizeof(CT) * (restart + 1));
    RT *C = (RT *)malloc(sizeof(RT) * (restart + 1));
    RT inner_res = 0, outer_res = tol + 1;
    int total = 0, outer = 0;
    const RT m1[2] = {-1, 0}, one[2] = {1, 0};
    while (outer_res > tol && outer < max_iter) {
        int nh = 0, nz = 0;
        memcpy(t, b, sz);
        OC_FN(or_spmv)('N', n, n, m1, pntr, indx, vals, x, one, t);
        OC_FN(precond_)(n, pntr, indx, diag, ilu, t, r);
        total++;
        inner_res = OC_FN(or_nrm2)(n, r);
        RT sc = (RT)(1.0 / (double)inner_res);   /* scal(engine, 1.0 / inner_res, r): zdscal */
        for (int i = 0; i < n; i++) r[i] = sc * r[i];
        Z[nz++] = inner_res;
        memcpy(W, r, sz);
        int k = 0;
        while (inner_res > tol && k < restart) {
            OC_FN(spmv1_)(n, pntr, indx, vals, r, t);
            OC_FN(precond_)(n, pntr, indx, diag, ilu, t, r);
            total++;
            for (int j = 0; j <= k; j++) cf[j] = OC_FN(dotu_)(n, W + (size_t)j * n, r);   /* gemv 'T' */
            for (int j = 0; j <= k; j++) {                                               /* gemv 'N', alpha -1 */
                const CT tj = (CT)(-1.0) * cf[j];
                for (int i = 0; i < n; i++) r[i] += tj * W[(size_t)j * n + i];
            }
            const RT nrm = OC_FN(or_nrm2)(n, r);
            sc = (RT)(1.0 / (double)nrm);
            for (int i = 0; i < n; i++) r[i] = sc * r[i];
            for (int i = 0; i < k; i++) OC_FN(rot_)(&cf[i], &cf[i + 1], C[i], S[i]);
            RT ic;
            CT is;
            OC_FN(rotg_)(&cf[k], (CT)nrm, &ic, &is);
            for (int j = 0; j <= k; j++) H[nh++] = cf[j];
            S[k] = is;
            C[k] = ic;
            inner_res = CABS(S[k] * Z[nz - 1]);
            k++;
            if (inner_res > tol && k < restart) {
                memcpy(W + (size_t)k * n, r, sz);
                Z[nz++] = 0;
                OC_FN(rot_)(&Z[k - 1], &Z[k], C[k - 1], S[k - 1]);
            }
        }
        if (nh > 0) {
            long kk = (long)nz * (nz + 1) / 2 - 1;
            for (int j = nz - 1; j >= 0; j--) {
                if (Z[j] != 0) {
                    Z[j] /= H[kk];
                    const CT tt = Z[j];
                    long q = kk - 1;
                    for (int i = j - 1; i >= 0; i--, q--) Z[i] -= tt * H[q];
                }
                kk -= j + 1;
            }
            for (int j = 0; j < nz; j++) {
                const CT tj = Z[j];
                for (int i = 0; i < n; i++) x[i] += tj * W[(size_t)j * n + i];
            }
        }
        outer++;
        outer_res = inner_res;
    }
    free(t);
    free(r);
    free(W);
    free(H);
    free(S);
    free(Z);
    free(cf);
    free(C);
    return total;
}

#undef OC_FN
#undef OC_CAT
#undef OC_CAT2
