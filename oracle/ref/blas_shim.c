/*
 * Minimal Fortran-ABI BLAS for building the reference's CPU path (test infrastructure only).
 *
 * The reference (HALA) calls an external Fortran BLAS (blas/hala_blas_external.hpp:29-338).
 * No BLAS library is installed in this image, so this file restates the published netlib
 * reference-BLAS algorithms for exactly the routines the reference's sparse + solver path
 * instantiates (ddot_, daxpy_, dnrm2_, dscal_, dcopy_, dgemv_, drot_, drotg_, dtpsv_, idamax_, the
 * single-precision twins, and for the complex solvers zcopy_, zaxpy_, zscal_, zdscal_, dznrm2_,
 * zrotg_, zrot_, zgemv_, ztpsv_ with their single-precision twins).  Summation order follows the netlib loops (sequential), which is
 * what the oracle restatement in oracle/hala_oracle.c assumes as well.
 *
 * Built only by oracle/ref/Makefile into oracle/_ref/; never linked into the product.
 */
#include <complex.h>
#include <math.h>

#define BLAS_DOT(NAME, T)                                                              \
    T NAME(const int *n, const T *x, const int *incx, const T *y, const int *incy) {   \
        T s = 0;                                                                       \
        int ix = (*incx >= 0) ? 0 : (1 - *n) * *incx;                                  \
        int iy = (*incy >= 0) ? 0 : (1 - *n) * *incy;                                  \
        for (int i = 0; i < *n; i++, ix += *incx, iy += *incy) s += x[ix] * y[iy];     \
        return s;                                                                      \
    }
BLAS_DOT(ddot_, double)
BLAS_DOT(sdot_, float)

#define BLAS_AXPY(NAME, T)                                                                  \
    void NAME(const int *n, const T *a, const T *x, const int *incx, T *y, const int *incy) { \
        if (*n <= 0 || *a == 0) return;                                                     \
        int ix = (*incx >= 0) ? 0 : (1 - *n) * *incx;                                       \
        int iy = (*incy >= 0) ? 0 : (1 - *n) * *incy;                                       \
        for (int i = 0; i < *n; i++, ix += *incx, iy += *incy) y[iy] += *a * x[ix];         \
    }
BLAS_AXPY(daxpy_, double)
BLAS_AXPY(saxpy_, float)

#define BLAS_SCAL(NAME, T)                                              \
    void NAME(const int *n, const T *a, T *x, const int *incx) {        \
        if (*n <= 0 || *incx <= 0) return;                              \
        for (int i = 0; i < *n; i++) x[i * *incx] *= *a;                \
    }
BLAS_SCAL(dscal_, double)
BLAS_SCAL(sscal_, float)

#define BLAS_COPY(NAME, T)                                                          \
    void NAME(const int *n, const T *x, const int *incx, T *y, const int *incy) {   \
        int ix = (*incx >= 0) ? 0 : (1 - *n) * *incx;                               \
        int iy = (*incy >= 0) ? 0 : (1 - *n) * *incy;                               \
        for (int i = 0; i < *n; i++, ix += *incx, iy += *incy) y[iy] = x[ix];       \
    }
BLAS_COPY(dcopy_, double)
BLAS_COPY(scopy_, float)

/* netlib scaled sum of squares (the pre-3.10 dnrm2 loop) */
#define BLAS_NRM2(NAME, T, SQRT, FABS)                                  \
    T NAME(const int *n, const T *x, const int *incx) {                 \
        if (*n < 1 || *incx < 1) return 0;                              \
        if (*n == 1) return FABS(x[0]);                                 \
        T scale = 0, ssq = 1;                                           \
        for (int i = 0; i < *n; i++) {                                  \
            T v = x[i * *incx];                                         \
            if (v != 0) {                                               \
                T a = FABS(v);                                          \
                if (scale < a) { ssq = 1 + ssq * (scale / a) * (scale / a); scale = a; } \
                else { ssq += (a / scale) * (a / scale); }              \
            }                                                           \
        }                                                               \
        return scale * SQRT(ssq);                                       \
    }
BLAS_NRM2(dnrm2_, double, sqrt, fabs)
BLAS_NRM2(snrm2_, float, sqrtf, fabsf)

#define BLAS_ROT(NAME, T)                                                                         \
    void NAME(const int *n, T *x, const int *incx, T *y, const int *incy, const T *c, const T *s) { \
        int ix = (*incx >= 0) ? 0 : (1 - *n) * *incx;                                             \
        int iy = (*incy >= 0) ? 0 : (1 - *n) * *incy;                                             \
        for (int i = 0; i < *n; i++, ix += *incx, iy += *incy) {                                  \
            T t = *c * x[ix] + *s * y[iy];                                                        \
            y[iy] = *c * y[iy] - *s * x[ix];                                                      \
            x[ix] = t;                                                                            \
        }                                                                                         \
    }
BLAS_ROT(drot_, double)
BLAS_ROT(srot_, float)

/* classic netlib rotg: r = sign(roe) * scale * sqrt((a/scale)^2 + (b/scale)^2) */
#define BLAS_ROTG(NAME, T, SQRT, FABS)                                      \
    void NAME(T *a, T *b, T *c, T *s) {                                     \
        T roe = (FABS(*a) > FABS(*b)) ? *a : *b;                            \
        T scale = FABS(*a) + FABS(*b);                                      \
        T r, z;                                                             \
        if (scale == 0) { *c = 1; *s = 0; r = 0; z = 0; }                   \
        else {                                                              \
            r = scale * SQRT((*a / scale) * (*a / scale) + (*b / scale) * (*b / scale)); \
            if (roe < 0) r = -r;                                            \
            *c = *a / r; *s = *b / r;                                       \
            z = 1;                                                          \
            if (FABS(*a) > FABS(*b)) z = *s;                                \
            if (FABS(*b) >= FABS(*a) && *c != 0) z = 1 / *c;                \
        }                                                                   \
        *a = r; *b = z;                                                     \
    }
BLAS_ROTG(drotg_, double, sqrt, fabs)
BLAS_ROTG(srotg_, float, sqrtf, fabsf)

/* y = alpha*op(A)*x + beta*y, column-major A (lda >= m), unit strides as used by the solvers */
#define BLAS_GEMV(NAME, T)                                                                  \
    void NAME(const char *trans, const int *m, const int *n, const T *alpha, const T *A,     \
              const int *lda, const T *x, const int *incx, const T *beta, T *y,              \
              const int *incy) {                                                            \
        int notrans = (*trans == 'N' || *trans == 'n');                                     \
        int leny = notrans ? *m : *n, lenx = notrans ? *n : *m;                             \
        if (*m == 0 || *n == 0) return;                                                     \
        if (*beta != 1) for (int i = 0; i < leny; i++) y[i * *incy] = (*beta == 0) ? 0 : *beta * y[i * *incy]; \
        if (*alpha == 0) return;                                                            \
        if (notrans) {                                                                      \
            for (int j = 0; j < lenx; j++) {                                                \
                T t = *alpha * x[j * *incx];                                                \
                for (int i = 0; i < leny; i++) y[i * *incy] += t * A[i + (long)j * *lda];   \
            }                                                                               \
        } else {                                                                            \
            for (int j = 0; j < leny; j++) {                                                \
                T t = 0;                                                                    \
                for (int i = 0; i < lenx; i++) t += A[i + (long)j * *lda] * x[i * *incx];   \
                y[j * *incy] += *alpha * t;                                                 \
            }                                                                               \
        }                                                                                   \
    }
BLAS_GEMV(dgemv_, double)
BLAS_GEMV(sgemv_, float)

/* packed triangular solve, only the (U, N, N) and (L, N, N) forms used by GMRES */
#define BLAS_TPSV(NAME, T)                                                                  \
    void NAME(const char *uplo, const char *trans, const char *diag, const int *n,           \
              const T *ap, T *x, const int *incx) {                                         \
        int nounit = (*diag == 'N' || *diag == 'n');                                        \
        (void)trans;                                                                        \
        if (*uplo == 'U' || *uplo == 'u') {                                                 \
            long kk = (long)(*n) * (*n + 1) / 2 - 1;                                        \
            for (int j = *n - 1; j >= 0; j--) {                                             \
                if (x[j * *incx] != 0) {                                                    \
                    if (nounit) x[j * *incx] /= ap[kk];                                     \
                    T t = x[j * *incx];                                                     \
                    long k = kk - 1;                                                        \
                    for (int i = j - 1; i >= 0; i--, k--) x[i * *incx] -= t * ap[k];        \
                }                                                                           \
                kk -= j + 1;                                                                \
            }                                                                               \
        } else {                                                                            \
            long kk = 0;                                                                    \
            for (int j = 0; j < *n; j++) {                                                  \
                if (x[j * *incx] != 0) {                                                    \
                    if (nounit) x[j * *incx] /= ap[kk];                                     \
                    T t = x[j * *incx];                                                     \
                    long k = kk + 1;                                                        \
                    for (int i = j + 1; i < *n; i++, k++) x[i * *incx] -= t * ap[k];        \
                }                                                                           \
                kk += *n - j;                                                               \
            }                                                                               \
        }                                                                                   \
    }
BLAS_TPSV(dtpsv_, double)
BLAS_TPSV(stpsv_, float)

/* index (1-based) of the first entry of largest magnitude (batch_max_norm2 in the batch CG) */
int idamax_(const int *n, const double *x, const int *incx) {
    if (*n < 1 || *incx <= 0) return 0;
    int best = 1;
    double m = fabs(x[0]);
    for (int i = 1; i < *n; i++)
        if (fabs(x[i * *incx]) > m) { m = fabs(x[i * *incx]); best = i + 1; }
    return best;
}

/* ------------------------------------------------------------------ complex ------------- */
/* Complex arithmetic is C99's, with -ffp-contract=off (separately rounded ac - bd, ad + bc). */
#define CBLAS_COPY(NAME, T) BLAS_COPY(NAME, T)
CBLAS_COPY(zcopy_, double complex)
CBLAS_COPY(ccopy_, float complex)

#define CBLAS_AXPY(NAME, T, RABS)                                                           \
    void NAME(const int *n, const T *a, const T *x, const int *incx, T *y, const int *incy) { \
        if (*n <= 0 || RABS(creal(*a)) + RABS(cimag(*a)) == 0) return;                      \
        int ix = (*incx >= 0) ? 0 : (1 - *n) * *incx;                                       \
        int iy = (*incy >= 0) ? 0 : (1 - *n) * *incy;                                       \
        for (int i = 0; i < *n; i++, ix += *incx, iy += *incy) y[iy] += *a * x[ix];         \
    }
CBLAS_AXPY(zaxpy_, double complex, fabs)
CBLAS_AXPY(caxpy_, float complex, fabsf)

#define CBLAS_SCAL(NAME, T, A)                                          \
    void NAME(const int *n, const A *a, T *x, const int *incx) {        \
        if (*n <= 0 || *incx <= 0) return;                              \
        for (int i = 0; i < *n; i++) x[i * *incx] = *a * x[i * *incx];  \
    }
CBLAS_SCAL(zscal_, double complex, double complex)
CBLAS_SCAL(cscal_, float complex, float complex)
CBLAS_SCAL(zdscal_, double complex, double)
CBLAS_SCAL(csscal_, float complex, float)

/* netlib dznrm2 / scnrm2 (before 3.10): scaled sum of squares over real and imaginary parts */
#define CBLAS_NRM2(NAME, T, R, SQRT, FABS)                              \
    R NAME(const int *n, const T *x, const int *incx) {                 \
        if (*n < 1 || *incx < 1) return 0;                              \
        R scale = 0, ssq = 1;                                           \
        for (int i = 0; i < *n; i++) {                                  \
            R part[2] = {creal(x[i * *incx]), cimag(x[i * *incx])};     \
            for (int k = 0; k < 2; k++) {                               \
                if (part[k] != 0) {                                     \
                    R a = FABS(part[k]);                                \
                    if (scale < a) { ssq = 1 + ssq * (scale / a) * (scale / a); scale = a; } \
                    else { ssq += (a / scale) * (a / scale); }          \
                }                                                       \
            }                                                           \
        }                                                               \
        return scale * SQRT(ssq);                                       \
    }
CBLAS_NRM2(dznrm2_, double complex, double, sqrt, fabs)
CBLAS_NRM2(scnrm2_, float complex, float, sqrtf, fabsf)

/* netlib zrotg (before 3.10): c real, s complex */
#define CBLAS_ROTG(NAME, T, R, SQRT, CABS, CONJ)                        \
    void NAME(T *ca, const T *cb, R *c, T *s) {                         \
        if (CABS(*ca) == 0) { *c = 0; *s = 1; *ca = *cb; return; }     \
        R scale = CABS(*ca) + CABS(*cb);                                \
        R p = CABS(*ca / scale), q = CABS(*cb / scale);                 \
        R norm = scale * SQRT(p * p + q * q);                           \
        T alpha = *ca / CABS(*ca);                                      \
        *c = CABS(*ca) / norm;                                          \
        *s = alpha * CONJ(*cb) / norm;                                  \
        *ca = alpha * norm;                                             \
    }
CBLAS_ROTG(zrotg_, double complex, double, sqrt, cabs, conj)
CBLAS_ROTG(crotg_, float complex, float, sqrtf, cabsf, conjf)

/* LAPACK zrot / crot: c real, s complex; x' = c x + s y, y' = c y - conj(s) x */
#define CBLAS_ROT(NAME, T, R, CONJ)                                                               \
    void NAME(const int *n, T *x, const int *incx, T *y, const int *incy, const R *c, const T *s) { \
        int ix = (*incx >= 0) ? 0 : (1 - *n) * *incx;                                             \
        int iy = (*incy >= 0) ? 0 : (1 - *n) * *incy;                                             \
        for (int i = 0; i < *n; i++, ix += *incx, iy += *incy) {                                  \
            T t = *c * x[ix] + *s * y[iy];                                                        \
            y[iy] = *c * y[iy] - CONJ(*s) * x[ix];                                                \
            x[ix] = t;                                                                            \
        }                                                                                         \
    }
CBLAS_ROT(zrot_, double complex, double, conj)
CBLAS_ROT(crot_, float complex, float, conjf)

/* y = alpha op(A) x + beta y, column-major; 'T' does not conjugate, 'C' does (netlib zgemv) */
#define CBLAS_GEMV(NAME, T, CONJ)                                                           \
    void NAME(const char *trans, const int *m, const int *n, const T *alpha, const T *A,     \
              const int *lda, const T *x, const int *incx, const T *beta, T *y,              \
              const int *incy) {                                                            \
        int notrans = (*trans == 'N' || *trans == 'n');                                     \
        int cj = (*trans == 'C' || *trans == 'c');                                          \
        int leny = notrans ? *m : *n, lenx = notrans ? *n : *m;                             \
        if (*m == 0 || *n == 0) return;                                                     \
        if (*beta != 1) for (int i = 0; i < leny; i++) y[i * *incy] = (*beta == 0) ? 0 : *beta * y[i * *incy]; \
        if (*alpha == 0) return;                                                            \
        if (notrans) {                                                                      \
            for (int j = 0; j < lenx; j++) {                                                \
                T t = *alpha * x[j * *incx];                                                \
                for (int i = 0; i < leny; i++) y[i * *incy] += t * A[i + (long)j * *lda];   \
            }                                                                               \
        } else {                                                                            \
            for (int j = 0; j < leny; j++) {                                                \
                T t = 0;                                                                    \
                for (int i = 0; i < lenx; i++)                                              \
                    t += (cj ? CONJ(A[i + (long)j * *lda]) : A[i + (long)j * *lda]) * x[i * *incx]; \
                y[j * *incy] += *alpha * t;                                                 \
            }                                                                               \
        }                                                                                   \
    }
CBLAS_GEMV(zgemv_, double complex, conj)
CBLAS_GEMV(cgemv_, float complex, conjf)

BLAS_TPSV(ztpsv_, double complex)
BLAS_TPSV(ctpsv_, float complex)
