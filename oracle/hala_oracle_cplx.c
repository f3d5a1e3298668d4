/*
 * Complex (C128 / C64) CPU oracle for the sparse Krylov path (TEST INFRASTRUCTURE ONLY; see
 * hala_oracle.h).  The reference's templates run on std::complex<double> / std::complex<float>
 * (sparse/hala_sparse_utils.hpp and the solver headers under hex/solvers); this is their restatement on C99 complex
 * types, compiled with -ffp-contract=off like the real oracle.
 */
#include "hala_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define CT double complex
#define RT double
#define CS z
#define RSQRT sqrt
#define RFABS fabs
#define CCONJ conj
#define CABS cabs
#include "hala_oracle_cplx_impl.h"
#undef CT
#undef RT
#undef CS
#undef RSQRT
#undef RFABS
#undef CCONJ
#undef CABS

#define CT float complex
#define RT float
#define CS c
#define RSQRT sqrtf
#define RFABS fabsf
#define CCONJ conjf
#define CABS cabsf
#include "hala_oracle_cplx_impl.h"
