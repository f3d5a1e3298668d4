// Kernel-level building blocks shared between libhgb translation units.
#pragma once

#include "hgb_internal.cuh"

struct hgb_zilu;

namespace hgb {

// ------------------------------------------------------------ shared-memory addressing ----
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Per-thread asynchronous copies global -> shared (cp.async), completion tracked per thread in
// commit groups.  16-byte copies go through L2 only (.cg); dst and src 16B aligned.
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// wait until at most N of this thread's most recent commit groups are still in flight
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void named_bar_sync(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

template <typename V> struct Val;
template <> struct Val<double> {
    using X = double;
    __device__ static double get(double v) { return v; }
};
template <> struct Val<float> {
    using X = float;
    __device__ static float get(float v) { return v; }
};
template <> struct Val<uint16_t> {   // bfloat16 bit pattern
    using X = float;
    __device__ static float get(uint16_t v) { return __uint_as_float((uint32_t)v << 16); }
};

// Per-thread running sum of products for the grid reductions.  FP64 data: a double sum.  FP32
// data: a float sum (FMA) flushed into a double every 16 terms.  The FP64 pipe of sm_103 is narrow
// (a warp-wide FP64 instruction holds it for 64 cycles), so converting every FP32 term to double
// and accumulating it with an FP64 FMA bounds an FP32 reduction by the FP64 pipe rather than by
// memory; the float partials of 16 terms keep the per-thread error at the FP32 level of the data.
template <typename X> struct DotAcc {
    double d = 0.0;
    __device__ __forceinline__ void add(X a, X b) { d += (double)a * (double)b; }
    __device__ __forceinline__ double get() const { return d; }
};
template <> struct DotAcc<float> {
    double d = 0.0;
    float f = 0.0f;
    int k = 0;
    __device__ __forceinline__ void add(float a, float b) {
        f = __fmaf_rn(a, b, f);
        if (++k == 16) {
            d += (double)f;
            f = 0.0f;
            k = 0;
        }
    }
    __device__ __forceinline__ double get() const { return d + (double)f; }
};

__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }


// Cached transpose of a CSR pattern: pntr[n+1], row[nnz] (original row of each entry, ascending
// inside a transposed row) and map[nnz] (position of the entry in the original arrays).
struct Transpose {
    int n = 0;
    int *pntr = nullptr, *row = nullptr, *map = nullptr;
    void release();
};

int exclusive_scan(hgb_ctx *c, const int *in, int *out, int n, int *total_dev, int *scratch);
int csr_check(hgb_ctx *c, int n_rows, int n_cols, int nnz, const int *pntr, const int *indx);
int build_transpose(hgb_ctx *c, int n_rows, int n_cols, int nnz, const int *pntr, const int *indx,
                    Transpose &T);

template <typename V>
int spmv_n_launch(hgb_ctx *c, int n_rows, const int *pntr, const int *indx, const V *vals,
                  typename Val<V>::X alpha, const typename Val<V>::X *x, typename Val<V>::X beta,
                  typename Val<V>::X *y, double *dot_out, const int *skip = nullptr, int *nparts = nullptr);
// Y = alpha A X + beta Y over nrhs column-major columns, the matrix read once (each column
// bit-identical to spmv_n_launch's product)
template <typename V>
int spmm_n_launch(hgb_ctx *c, int n_rows, const int *pntr, const int *indx, const V *vals, int nrhs,
                  typename Val<V>::X alpha, const typename Val<V>::X *x, long ldx, typename Val<V>::X beta,
                  typename Val<V>::X *y, long ldy);
template <typename V>
int spmv_t_launch(hgb_ctx *c, int n_rows, int n_cols, const int *pntr, const int *indx, const V *vals,
                  typename Val<V>::X alpha, const typename Val<V>::X *x, typename Val<V>::X beta,
                  typename Val<V>::X *y, const Transpose *T);

// ILU internals used by the fused solvers (skip: device flag that turns the launches into no-ops)
int ilu_apply_internal(hgb_ilu *M, char trans, const void *x, void *r, const int *skip = nullptr);
hgb_dtype ilu_store(const hgb_ilu *M);
int ilu_n(const hgb_ilu *M);
size_t ilu_xbytes(const hgb_ilu *M);       // bytes of one element of the vectors the apply reads and writes
hgb_zilu *ilu_zfactor(const hgb_ilu *M);   // the complex factor of a C128 / C64 handle, else null
inline bool real_inner(hgb_dtype t) { return t == HGB_F32 || t == HGB_BF16; }
// a preconditioner stored in precision s serves a matrix of dtype t: F64, C128 and C64 alike,
// F32 / BF16 matrices with either F32 or BF16 stores (vectors float)
inline bool ilu_matches(hgb_dtype s, hgb_dtype t) {
    if (t == HGB_F64 || t == HGB_C128 || t == HGB_C64) return s == t;
    return real_inner(s);
}

// transposed operator for the adjoint solves: build (once) the cached transpose, then
// y = alpha A^T x + beta y with an optional fused <dot_x, y>
int csr_ensure_transpose(hgb_csr *A);
template <typename V>
int spmv_t_fused_launch(hgb_csr *A, typename Val<V>::X alpha, const typename Val<V>::X *x, typename Val<V>::X beta,
                        typename Val<V>::X *y, const typename Val<V>::X *dot_x, double *dot_out, const int *skip);

// accessors of the opaque matrix handle
const int *csr_pntr(const hgb_csr *A);
const int *csr_indx(const hgb_csr *A);
const void *csr_vals(const hgb_csr *A);
int csr_rows(const hgb_csr *A);
int csr_cols(const hgb_csr *A);
int csr_nnz(const hgb_csr *A);
hgb_dtype csr_dtype(const hgb_csr *A);
hgb_ctx *csr_ctx(const hgb_csr *A);

}  // namespace hgb
