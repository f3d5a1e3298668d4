// CSR SpMV for sm_103a.  One warp takes 32 consecutive rows at a time: it copies the tile's whole
// vals / indx range into its own shared-memory buffer with coalesced 16-byte cp.async (no
// handshake between warps), then every lane sums its row from shared memory, gathering x from
// global memory (L2) kGW entries at a time.  The warp double-buffers: the copy of tile k+1 and the
// row pointers of tile k+2 are in flight while tile k is summed.  Tiles of more than kWarpCap
// entries read their rows directly.
//
// Two arithmetic modes, chosen per context (hgb_ctx_set_spmv_mode):
//  - exact: each row summed in column order with separately rounded multiply and add, the
//    arithmetic of the reference's sparse_gemv_array<T,'N'> (sparse/hala_sparse_utils.hpp:104-112),
//    so FP64 results are bit-identical to the reference CPU path.  That is two FP64 operations per
//    entry; sm_103's FP64 pipe is narrow (a warp-wide FP64 instruction holds an SMSP's FP64 unit
//    for 64 cycles), so the exact FP64 product is bound by the FP64 pipe, not by HBM.
//  - fused (the default): the same column order with one fused multiply-add per entry; a product
//    with alpha = 1 and beta = 0 skips the scaling.  Results differ from the reference's by the
//    rounding of the individual products (a few ulps of the row sum).
#include "hgb_internal.cuh"
#include "hgb_kernels.cuh"
#include "hgb_complex.cuh"

#include <algorithm>
#include <cstdlib>
#include <string>
#include <vector>

namespace hgb {

static bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

constexpr int kWarpCap = 256;
constexpr int kWarpBlock = 256;   // 8 warps per CTA
constexpr int kGW = 4;            // x gathers in flight per lane

// acc += v * x in the mode's rounding
template <bool EXACT>
__device__ __forceinline__ double spmv_acc(double acc, double v, double x) {
    return EXACT ? add_rn(acc, mul_rn(v, x)) : __fma_rn(v, x, acc);
}
template <bool EXACT>
__device__ __forceinline__ float spmv_acc(float acc, float v, float x) {
    return EXACT ? add_rn(acc, mul_rn(v, x)) : __fmaf_rn(v, x, acc);
}
// alpha * acc + beta * y (y read only when beta != 0)
template <bool EXACT, typename X>
__device__ __forceinline__ X spmv_out(X alpha, X acc, X beta, const X *yp) {
    if (EXACT) return (beta == X(0)) ? mul_rn(alpha, acc) : add_rn(mul_rn(alpha, acc), mul_rn(beta, *yp));
    if (beta == X(0)) return (alpha == X(1)) ? acc : mul_rn(alpha, acc);
    return spmv_acc<false>(mul_rn(beta, *yp), alpha, acc);
}

// The fused <x, y> (DOT): 0 none; 1 the grid reduction into *dot_out (the last CTA adds the
// parts); 2 each CTA's part to partials[blockIdx.x], summed by the consuming kernel (in one order
// in every CTA), which keeps the serial last-CTA step out of the product.
template <int DOT>
__device__ __forceinline__ void spmv_dot_epilogue(double d, double *partials, unsigned *counter, double *dot_out) {
    double dsum[1] = {d};
    if (DOT == 1) {
        grid_sum<1>(dsum, partials, counter, [&](double (&v)[1]) { *dot_out = v[0]; });
    } else if (DOT == 2) {
        block_sum<1>(dsum);
        if (threadIdx.x == 0) partials[blockIdx.x] = dsum[0];
    }
}

// y = alpha * A x + beta * y ; optionally <x, y> (square A; DOT as spmv_dot_epilogue)
template <typename V, int DOT, bool EXACT>
__global__ void __launch_bounds__(kWarpBlock)
spmv_warp_kernel(int n_rows, const int *__restrict__ pntr, const int *__restrict__ indx, const V *__restrict__ vals,
                 typename Val<V>::X alpha, const typename Val<V>::X *__restrict__ x, typename Val<V>::X beta,
                 typename Val<V>::X *__restrict__ y, double *partials, unsigned *counter, double *dot_out,
                 const int *skip) {
    using X = typename Val<V>::X;
    constexpr int EV = 16 / (int)sizeof(V);   // values per 16-byte unit
    constexpr int SV = kWarpCap + 2 * EV, SI = kWarpCap + 8;
    if (skip && *skip) return;
    __shared__ __align__(16) V s_vals[kWarpBlock / 32][2][SV];
    __shared__ __align__(16) int s_idx[kWarpBlock / 32][2][SI];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int nnz = __ldg(pntr + n_rows);
    const long ntiles = ((long)n_rows + 31) / 32;
    const long nwarps = (long)gridDim.x * (kWarpBlock / 32);
    const long per = (ntiles + nwarps - 1) / nwarps;
    const long tb = ((long)blockIdx.x * (kWarpBlock / 32) + wib) * per;
    const long te = min(ntiles, tb + per);
    DotAcc<X> dacc;   // fused <x, y> (per-thread partial)

    // lane's row pointers of tile k (loads only; nothing waits on them yet)
    auto load_ptrs = [&](long k, int &ps, int &pe) {
        const int row = (int)(k * 32) + lane;
        ps = __ldg(pntr + min(row, n_rows));
        pe = __ldg(pntr + min(row + 1, n_rows));
    };
    // the tile's entry range, and its copy into buffer buf when it fits
    auto start_tile = [&](long k, int ps, int pe, int buf, int &base, int &end) {
        const int nr = min(32, n_rows - (int)(k * 32));
        base = __shfl_sync(0xffffffffu, ps, 0);
        end = __shfl_sync(0xffffffffu, pe, nr - 1);
        if (end - base <= kWarpCap) {
            V *sv = s_vals[wib][buf];
            int *si = s_idx[wib][buf];
            const int av = base & ~(EV - 1), ai = base & ~3;
            for (int g = av + lane * EV; g < end; g += 32 * EV) {
                if (g + EV <= nnz) cp_async16(sv + (g - av), vals + g);
                else
                    for (int q = 0; q < EV && g + q < end; q++) sv[g - av + q] = vals[g + q];
            }
            for (int g = ai + lane * 4; g < end; g += 32 * 4) {
                if (g + 4 <= nnz) cp_async16(si + (g - ai), indx + g);
                else
                    for (int q = 0; q < 4 && g + q < end; q++) si[g - ai + q] = indx[g + q];
            }
        }
        cp_async_commit();
    };

    if (tb < te) {
        int ps0, pe0, ps1 = 0, pe1 = 0, base0, end0;
        load_ptrs(tb, ps0, pe0);
        start_tile(tb, ps0, pe0, 0, base0, end0);
        if (tb + 1 < te) load_ptrs(tb + 1, ps1, pe1);
        for (long k = tb; k < te; k++) {
            const int buf = (int)((k - tb) & 1);
            int base1 = 0, end1 = 0, ps2 = 0, pe2 = 0;
            if (k + 1 < te) start_tile(k + 1, ps1, pe1, buf ^ 1, base1, end1);
            else cp_async_commit();
            if (k + 2 < te) load_ptrs(k + 2, ps2, pe2);
            cp_async_wait<1>();   // tile k has landed
            __syncwarp();
            const int row = (int)(k * 32) + lane;
            X acc = X(0);
            if (row < n_rows) {
                if (end0 - base0 <= kWarpCap) {
                    const V *sv = s_vals[wib][buf];
                    const int *si = s_idx[wib][buf];
                    const int ov = base0 & ~(EV - 1), oi = base0 & ~3;
                    for (int j0 = ps0; j0 < pe0; j0 += kGW) {
                        X xv[kGW], vv[kGW];
#pragma unroll
                        for (int q = 0; q < kGW; q++)
                            if (j0 + q < pe0) {
                                vv[q] = Val<V>::get(sv[j0 + q - ov]);
                                xv[q] = __ldg(x + si[j0 + q - oi]);
                            }
#pragma unroll
                        for (int q = 0; q < kGW; q++)
                            if (j0 + q < pe0) acc = spmv_acc<EXACT>(acc, vv[q], xv[q]);
                    }
                } else {
                    for (int j0 = ps0; j0 < pe0; j0 += kGW) {
                        X xv[kGW], vv[kGW];
#pragma unroll
                        for (int q = 0; q < kGW; q++)
                            if (j0 + q < pe0) {
                                vv[q] = Val<V>::get(__ldg(vals + j0 + q));
                                xv[q] = __ldg(x + __ldg(indx + j0 + q));
                            }
#pragma unroll
                        for (int q = 0; q < kGW; q++)
                            if (j0 + q < pe0) acc = spmv_acc<EXACT>(acc, vv[q], xv[q]);
                    }
                }
                const X out = spmv_out<EXACT>(alpha, acc, beta, y + row);
                y[row] = out;
                if (DOT) dacc.add(__ldg(x + row), out);
            }
            __syncwarp();   // buffer buf is refilled by tile k+2
            ps0 = ps1;
            pe0 = pe1;
            base0 = base1;
            end0 = end1;
            ps1 = ps2;
            pe1 = pe2;
        }
    }
    cp_async_wait<0>();
    if (DOT) spmv_dot_epilogue<DOT>(dacc.get(), partials, counter, dot_out);
}

// Y = alpha * A X + beta * Y for nrhs column-major columns (x column c at x + c * ldx): the tiles
// of spmv_warp_kernel, each staged in shared memory once and summed for kMmCols columns at a time
// (the matrix is read once, not once per column).  Every column is summed in column order in
// the mode's rounding, so each column equals the single-column product bit for bit.
constexpr int kMmCols = 4;   // columns summed per pass over a tile (gathers in flight per lane)
template <typename V, bool EXACT>
__global__ void __launch_bounds__(kWarpBlock)
spmm_warp_kernel(int n_rows, const int *__restrict__ pntr, const int *__restrict__ indx, const V *__restrict__ vals,
                 int nrhs, typename Val<V>::X alpha, const typename Val<V>::X *__restrict__ x, long ldx,
                 typename Val<V>::X beta, typename Val<V>::X *__restrict__ y, long ldy) {
    using X = typename Val<V>::X;
    constexpr int EV = 16 / (int)sizeof(V);
    constexpr int SV = kWarpCap + 2 * EV, SI = kWarpCap + 8;
    __shared__ __align__(16) V s_vals[kWarpBlock / 32][2][SV];
    __shared__ __align__(16) int s_idx[kWarpBlock / 32][2][SI];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int nnz = __ldg(pntr + n_rows);
    const long ntiles = ((long)n_rows + 31) / 32;
    const long nwarps = (long)gridDim.x * (kWarpBlock / 32);
    const long per = (ntiles + nwarps - 1) / nwarps;
    const long tb = ((long)blockIdx.x * (kWarpBlock / 32) + wib) * per;
    const long te = min(ntiles, tb + per);
    auto load_ptrs = [&](long k, int &ps, int &pe) {
        const int row = (int)(k * 32) + lane;
        ps = __ldg(pntr + min(row, n_rows));
        pe = __ldg(pntr + min(row + 1, n_rows));
    };
    auto start_tile = [&](long k, int ps, int pe, int buf, int &base, int &end) {
        const int nr = min(32, n_rows - (int)(k * 32));
        base = __shfl_sync(0xffffffffu, ps, 0);
        end = __shfl_sync(0xffffffffu, pe, nr - 1);
        if (end - base <= kWarpCap) {
            V *sv = s_vals[wib][buf];
            int *si = s_idx[wib][buf];
            const int av = base & ~(EV - 1), ai = base & ~3;
            for (int g = av + lane * EV; g < end; g += 32 * EV) {
                if (g + EV <= nnz) cp_async16(sv + (g - av), vals + g);
                else
                    for (int q = 0; q < EV && g + q < end; q++) sv[g - av + q] = vals[g + q];
            }
            for (int g = ai + lane * 4; g < end; g += 32 * 4) {
                if (g + 4 <= nnz) cp_async16(si + (g - ai), indx + g);
                else
                    for (int q = 0; q < 4 && g + q < end; q++) si[g - ai + q] = indx[g + q];
            }
        }
        cp_async_commit();
    };
    if (tb >= te) return;
    int ps0, pe0, ps1 = 0, pe1 = 0, base0, end0;
    load_ptrs(tb, ps0, pe0);
    start_tile(tb, ps0, pe0, 0, base0, end0);
    if (tb + 1 < te) load_ptrs(tb + 1, ps1, pe1);
    for (long k = tb; k < te; k++) {
        const int buf = (int)((k - tb) & 1);
        int base1 = 0, end1 = 0, ps2 = 0, pe2 = 0;
        if (k + 1 < te) start_tile(k + 1, ps1, pe1, buf ^ 1, base1, end1);
        else cp_async_commit();
        if (k + 2 < te) load_ptrs(k + 2, ps2, pe2);
        cp_async_wait<1>();   // tile k has landed
        __syncwarp();
        const int row = (int)(k * 32) + lane;
        if (row < n_rows) {
            const bool staged = end0 - base0 <= kWarpCap;
            const V *sv = s_vals[wib][buf];
            const int *si = s_idx[wib][buf];
            const int ov = base0 & ~(EV - 1), oi = base0 & ~3;
            for (int c0 = 0; c0 < nrhs; c0 += kMmCols) {
                const int nc = min(kMmCols, nrhs - c0);
                const X *xc = x + (long)c0 * ldx;
                X acc[kMmCols];
#pragma unroll
                for (int q = 0; q < kMmCols; q++) acc[q] = X(0);
                for (int j = ps0; j < pe0; j++) {
                    const X v = staged ? Val<V>::get(sv[j - ov]) : Val<V>::get(__ldg(vals + j));
                    const int col = staged ? si[j - oi] : __ldg(indx + j);
                    X xv[kMmCols];
#pragma unroll
                    for (int q = 0; q < kMmCols; q++)
                        if (q < nc) xv[q] = __ldg(xc + (long)q * ldx + col);
#pragma unroll
                    for (int q = 0; q < kMmCols; q++)
                        if (q < nc) acc[q] = spmv_acc<EXACT>(acc[q], v, xv[q]);
                }
#pragma unroll
                for (int q = 0; q < kMmCols; q++)
                    if (q < nc) {
                        X *yp = y + (long)(c0 + q) * ldy + row;
                        *yp = spmv_out<EXACT>(alpha, acc[q], beta, yp);
                    }
            }
        }
        __syncwarp();   // buffer buf is refilled by tile k+2
        ps0 = ps1;
        pe0 = pe1;
        base0 = base1;
        end0 = end1;
        ps1 = ps2;
        pe1 = pe2;
    }
    cp_async_wait<0>();
}

// Arrays that are not 16-byte aligned cannot be staged with cp.async: one row per thread,
// grid-stride, the row's vals/indx and x gathers (8 at a time) straight from global memory
// through L1.  Same arithmetic as spmv_warp_kernel.
template <typename V, int DOT, bool EXACT>
__global__ void __launch_bounds__(256)
spmv_direct_kernel(int n_rows, const int *__restrict__ pntr, const int *__restrict__ indx,
                   const V *__restrict__ vals, typename Val<V>::X alpha, const typename Val<V>::X *__restrict__ x,
                   typename Val<V>::X beta, typename Val<V>::X *__restrict__ y, double *partials, unsigned *counter,
                   double *dot_out, const int *skip) {
    using X = typename Val<V>::X;
    if (skip && *skip) return;
    DotAcc<X> dacc;   // fused <x, y> (per-thread partial)
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += gridDim.x * blockDim.x) {
        const int ps = __ldg(pntr + r), pe = __ldg(pntr + r + 1);
        X acc = X(0);
        for (int j0 = ps; j0 < pe; j0 += 8) {
            X xv[8], vv[8];
#pragma unroll
            for (int k = 0; k < 8; k++)
                if (j0 + k < pe) {
                    vv[k] = Val<V>::get(__ldg(vals + j0 + k));
                    xv[k] = __ldg(x + __ldg(indx + j0 + k));
                }
#pragma unroll
            for (int k = 0; k < 8; k++)
                if (j0 + k < pe) acc = spmv_acc<EXACT>(acc, vv[k], xv[k]);
        }
        const X out = spmv_out<EXACT>(alpha, acc, beta, y + r);
        y[r] = out;
        if (DOT) dacc.add(__ldg(x + r), out);
    }
    if (DOT) spmv_dot_epilogue<DOT>(dacc.get(), partials, counter, dot_out);
}


// transposed product by atomic scatter (stateless path): y[c] += (alpha * x[i]) * v_ic
template <typename V>
__global__ void spmv_t_atomic_kernel(int n_rows, const int *__restrict__ pntr, const int *__restrict__ indx,
                                     const V *__restrict__ vals, typename Val<V>::X alpha,
                                     const typename Val<V>::X *__restrict__ x, typename Val<V>::X *y) {
    using X = typename Val<V>::X;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_rows; i += gridDim.x * blockDim.x) {
        X ax = mul_rn(alpha, x[i]);
        for (int p = __ldg(pntr + i); p < __ldg(pntr + i + 1); p++)
            atomicAdd(y + __ldg(indx + p), mul_rn(ax, Val<V>::get(__ldg(vals + p))));
    }
}

template <typename X>
__global__ void scale_or_zero_kernel(long n, X beta, X *y) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        y[i] = (beta == X(0)) ? X(0) : mul_rn(beta, y[i]);
}

// transposed product through the cached transpose: one thread per column, entries in ascending
// original row, which is the accumulation order of sparse_gemv_array<'T'> (utils:113-118).
// FUSE_DOT additionally reduces <x', y> with x' = the vector y is paired with (dot_x, indexed by
// column), for the CG on the transposed operator.
template <typename V, bool FUSE_DOT>
__global__ void spmv_t_cached_kernel(int n_cols, const int *__restrict__ pntrT, const int *__restrict__ rowT,
                                     const int *__restrict__ mapT, const V *__restrict__ vals,
                                     typename Val<V>::X alpha, const typename Val<V>::X *__restrict__ x,
                                     typename Val<V>::X beta, typename Val<V>::X *__restrict__ y,
                                     const typename Val<V>::X *__restrict__ dot_x, double *partials,
                                     unsigned *counter, double *dot_out, const int *skip) {
    using X = typename Val<V>::X;
    if (skip && *skip) return;
    DotAcc<X> dacc;   // fused <x, y> (per-thread partial)
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n_cols; c += gridDim.x * blockDim.x) {
        X acc = (beta == X(0)) ? X(0) : mul_rn(beta, y[c]);
        for (int p = __ldg(pntrT + c); p < __ldg(pntrT + c + 1); p++) {
            int i = __ldg(rowT + p);
            acc = add_rn(acc, mul_rn(mul_rn(alpha, __ldg(x + i)), Val<V>::get(__ldg(vals + __ldg(mapT + p)))));
        }
        y[c] = acc;
        if (FUSE_DOT) dacc.add(dot_x[c], acc);
    }
    if (FUSE_DOT) {
        double dsum[1] = {dacc.get()};
        grid_sum<1>(dsum, partials, counter, [&](double (&v)[1]) { *dot_out = v[0]; });
    }
}

// ------------------------------------------------------------- CSR validation ----------
__global__ void csr_check_kernel(int n_rows, int n_cols, int nnz, const int *__restrict__ pntr,
                                 const int *__restrict__ indx, int *err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_rows; i += gridDim.x * blockDim.x) {
        int a = pntr[i], b = pntr[i + 1];
        if (a < 0 || b < a || b > nnz) { atomicOr(err, DEV_ERR_CSR); continue; }
        int prev = -1;
        for (int p = a; p < b; p++) {
            int c = indx[p];
            if (c <= prev || c >= n_cols) { atomicOr(err, DEV_ERR_CSR); break; }
            prev = c;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && (pntr[0] != 0 || pntr[n_rows] != nnz)) atomicOr(err, DEV_ERR_CSR);
}

// ------------------------------------------------------------- scan / transpose -------
__global__ void scan_blocks_kernel(const int *__restrict__ in, int *__restrict__ out, int n, int *block_tot) {
    // exclusive scan of 1024-element chunks (one per CTA of 1024 threads)
    __shared__ int sh[1024];
    int i = blockIdx.x * 1024 + threadIdx.x;
    int v = (i < n) ? in[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        int t = (threadIdx.x >= o) ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = sh[threadIdx.x] - v;
    if (threadIdx.x == 1023) block_tot[blockIdx.x] = sh[1023];
}

__global__ void scan_tot_kernel(int *tot, int nb, int *grand) {
    // sequential exclusive scan of the block totals by one thread (nb is small)
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int run = 0;
        for (int b = 0; b < nb; b++) {
            int t = tot[b];
            tot[b] = run;
            run += t;
        }
        *grand = run;
    }
}

__global__ void scan_add_kernel(int *out, int n, const int *tot) {
    int i = blockIdx.x * 1024 + threadIdx.x;
    if (i < n) out[i] += tot[blockIdx.x];
}

__global__ void count_cols_kernel(int nnz, const int *__restrict__ indx, int *cnt) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x)
        atomicAdd(cnt + indx[p], 1);
}

__global__ void fill_transpose_kernel(int n_rows, const int *__restrict__ pntr, const int *__restrict__ indx,
                                      const int *__restrict__ pntrT, int *cursor, int *rowT, int *mapT) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_rows; i += gridDim.x * blockDim.x)
        for (int p = pntr[i]; p < pntr[i + 1]; p++) {
            int c = indx[p];
            int slot = pntrT[c] + atomicAdd(cursor + c, 1);
            rowT[slot] = i;
            mapT[slot] = p;
        }
}

__global__ void sort_segments_kernel(int n, const int *__restrict__ ptr, int *key, int *val) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        int a = ptr[r], b = ptr[r + 1];
        for (int i = a + 1; i < b; i++) {   // insertion sort: segments are short
            int k = key[i], v = val[i], j = i - 1;
            while (j >= a && key[j] > k) {
                key[j + 1] = key[j];
                val[j + 1] = val[j];
                j--;
            }
            key[j + 1] = k;
            val[j + 1] = v;
        }
    }
}

int exclusive_scan(hgb_ctx *c, const int *in, int *out, int n, int *total_dev, int *scratch) {
    // scratch: at least ceil(n/1024) ints
    int nb = (n + 1023) / 1024;
    if (nb == 0) return HGB_OK;
    scan_blocks_kernel<<<nb, 1024, 0, c->stream>>>(in, out, n, scratch);
    scan_tot_kernel<<<1, 32, 0, c->stream>>>(scratch, nb, total_dev);
    scan_add_kernel<<<nb, 1024, 0, c->stream>>>(out, n, scratch);
    return launch_check("exclusive_scan");
}

int csr_check(hgb_ctx *c, int n_rows, int n_cols, int nnz, const int *pntr, const int *indx) {
    if (n_rows <= 0) return HGB_OK;
    csr_check_kernel<<<std::min((n_rows + 255) / 256, c->num_sms * 8), 256, 0, c->stream>>>(n_rows, n_cols, nnz,
                                                                                           pntr, indx, c->err);
    HGB_TRY(launch_check("csr_check_kernel"));
    return collect_dev_error(c);
}

int build_transpose(hgb_ctx *c, int n_rows, int n_cols, int nnz, const int *pntr, const int *indx,
                    Transpose &T) {
    T.n = n_cols;
    size_t nb = (size_t)(n_cols + 1 + 1023) / 1024 + 1;
    HGB_CUDA(cudaMalloc(&T.pntr, sizeof(int) * (size_t)(n_cols + 1)));
    HGB_CUDA(cudaMalloc(&T.row, sizeof(int) * (size_t)std::max(nnz, 1)));
    HGB_CUDA(cudaMalloc(&T.map, sizeof(int) * (size_t)std::max(nnz, 1)));
    int *cnt = nullptr, *scratch = nullptr;
    HGB_CUDA(cudaMalloc(&cnt, sizeof(int) * (size_t)(n_cols + 1)));
    HGB_CUDA(cudaMalloc(&scratch, sizeof(int) * (nb + 1)));
    int st = HGB_OK;
    do {
        if (cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)(n_cols + 1), c->stream) != cudaSuccess) { st = HGB_ERR_CUDA; break; }
        int g = std::max(1, std::min((nnz + 255) / 256, c->num_sms * 8));
        count_cols_kernel<<<g, 256, 0, c->stream>>>(nnz, indx, cnt);
        st = exclusive_scan(c, cnt, T.pntr, n_cols + 1, scratch + nb, scratch);
        if (st) break;
        if (cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)(n_cols + 1), c->stream) != cudaSuccess) { st = HGB_ERR_CUDA; break; }
        int gr = std::max(1, std::min((n_rows + 255) / 256, c->num_sms * 8));
        fill_transpose_kernel<<<gr, 256, 0, c->stream>>>(n_rows, pntr, indx, T.pntr, cnt, T.row, T.map);
        int gc = std::max(1, std::min((n_cols + 255) / 256, c->num_sms * 8));
        sort_segments_kernel<<<gc, 256, 0, c->stream>>>(n_cols, T.pntr, T.row, T.map);
        st = launch_check("build_transpose");
        if (!st && cudaStreamSynchronize(c->stream) != cudaSuccess) st = cuda_fail(cudaGetLastError(), "build_transpose");
    } while (0);
    cudaFree(cnt);
    cudaFree(scratch);
    return st;
}

void Transpose::release() {
    cudaFree(pntr);
    cudaFree(row);
    cudaFree(map);
    pntr = row = map = nullptr;
}

template <typename V, int DOT, bool EXACT>
static int spmv_n_launch_mode(hgb_ctx *c, int n_rows, const int *pntr, const int *indx, const V *vals,
                              typename Val<V>::X alpha, const typename Val<V>::X *x, typename Val<V>::X beta,
                              typename Val<V>::X *y, double *dot_out, const int *skip, int *nparts) {
    // DOT 2: the per-CTA parts of <x, y> stay in the context's parts slots (their count to *nparts)
    double *partials = DOT == 2 ? c->partials + kSpmvPartsOffset : (DOT == 1 ? c->partials : nullptr);
    unsigned *counter = DOT == 1 ? c->counter : nullptr;
    if (aligned16(vals) && aligned16(indx)) {
        // persistent grid: the resident CTAs of every SM (occupancy queried once per kernel)
        static int occ = 0;
        if (!occ) {
            HGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, spmv_warp_kernel<V, DOT, EXACT>, kWarpBlock, 0));
            occ = std::max(occ, 1);
        }
        const long tiles = ((long)n_rows + 31) / 32;
        const int g = (int)std::max<long>(1, std::min<long>((tiles + 7) / 8, std::min(c->num_sms * occ, kMaxReduceBlocks)));
        if (nparts) *nparts = g;
        spmv_warp_kernel<V, DOT, EXACT><<<g, kWarpBlock, 0, c->stream>>>(n_rows, pntr, indx, vals, alpha, x, beta, y,
                                                                            partials, counter, dot_out, skip);
        return launch_check("spmv_warp_kernel");
    }
    const int g = std::min((n_rows + 255) / 256, std::min(c->num_sms * 8, kMaxReduceBlocks));
    if (nparts) *nparts = g;
    spmv_direct_kernel<V, DOT, EXACT><<<g, 256, 0, c->stream>>>(n_rows, pntr, indx, vals, alpha, x, beta, y, partials,
                                                                   counter, dot_out, skip);
    return launch_check("spmv_direct_kernel");
}

template <typename V>
int spmv_n_launch(hgb_ctx *c, int n_rows, const int *pntr, const int *indx, const V *vals,
                  typename Val<V>::X alpha, const typename Val<V>::X *x, typename Val<V>::X beta,
                  typename Val<V>::X *y, double *dot_out, const int *skip, int *nparts) {
    if (nparts) *nparts = 0;
    if (n_rows <= 0) return HGB_OK;
    const bool exact = c->spmv_mode == HGB_SPMV_EXACT;
    if (nparts)
        return exact ? spmv_n_launch_mode<V, 2, true>(c, n_rows, pntr, indx, vals, alpha, x, beta, y, nullptr, skip, nparts)
                     : spmv_n_launch_mode<V, 2, false>(c, n_rows, pntr, indx, vals, alpha, x, beta, y, nullptr, skip, nparts);
    if (dot_out)
        return exact ? spmv_n_launch_mode<V, 1, true>(c, n_rows, pntr, indx, vals, alpha, x, beta, y, dot_out, skip, nullptr)
                     : spmv_n_launch_mode<V, 1, false>(c, n_rows, pntr, indx, vals, alpha, x, beta, y, dot_out, skip, nullptr);
    return exact ? spmv_n_launch_mode<V, 0, true>(c, n_rows, pntr, indx, vals, alpha, x, beta, y, nullptr, skip, nullptr)
                 : spmv_n_launch_mode<V, 0, false>(c, n_rows, pntr, indx, vals, alpha, x, beta, y, nullptr, skip, nullptr);
}

template <typename V>
int spmm_n_launch(hgb_ctx *c, int n_rows, const int *pntr, const int *indx, const V *vals, int nrhs,
                  typename Val<V>::X alpha, const typename Val<V>::X *x, long ldx, typename Val<V>::X beta,
                  typename Val<V>::X *y, long ldy) {
    if (n_rows <= 0 || nrhs <= 0) return HGB_OK;
    if (!aligned16(vals) || !aligned16(indx)) {   // no staging: the single-column products
        for (int k = 0; k < nrhs; k++)
            HGB_TRY(spmv_n_launch<V>(c, n_rows, pntr, indx, vals, alpha, x + (long)k * ldx, beta, y + (long)k * ldy,
                                     nullptr));
        return HGB_OK;
    }
    const bool exact = c->spmv_mode == HGB_SPMV_EXACT;
    static int occ_dev[2][64] = {};
    if (c->device < 0 || c->device >= 64) return fail(HGB_ERR_UNSUPPORTED, "spmm: device ordinal %d", c->device);
    int &occ = occ_dev[exact ? 1 : 0][c->device];
    if (!occ) {
        HGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &occ, exact ? (const void *)spmm_warp_kernel<V, true> : (const void *)spmm_warp_kernel<V, false>,
            kWarpBlock, 0));
        occ = std::max(occ, 1);
    }
    const long tiles = ((long)n_rows + 31) / 32;
    const int g = (int)std::max<long>(1, std::min<long>((tiles + 7) / 8, (long)c->num_sms * occ));
    if (exact)
        spmm_warp_kernel<V, true><<<g, kWarpBlock, 0, c->stream>>>(n_rows, pntr, indx, vals, nrhs, alpha, x, ldx,
                                                                    beta, y, ldy);
    else
        spmm_warp_kernel<V, false><<<g, kWarpBlock, 0, c->stream>>>(n_rows, pntr, indx, vals, nrhs, alpha, x, ldx,
                                                                     beta, y, ldy);
    return launch_check("spmm_warp_kernel");
}

template int spmv_n_launch<double>(hgb_ctx *, int, const int *, const int *, const double *, double,
                                   const double *, double, double *, double *, const int *, int *);
template int spmv_n_launch<float>(hgb_ctx *, int, const int *, const int *, const float *, float,
                                  const float *, float, float *, double *, const int *, int *);
template int spmv_n_launch<uint16_t>(hgb_ctx *, int, const int *, const int *, const uint16_t *, float,
                                     const float *, float, float *, double *, const int *, int *);
template int spmm_n_launch<double>(hgb_ctx *, int, const int *, const int *, const double *, int, double,
                                   const double *, long, double, double *, long);
template int spmm_n_launch<float>(hgb_ctx *, int, const int *, const int *, const float *, int, float,
                                  const float *, long, float, float *, long);
template int spmm_n_launch<uint16_t>(hgb_ctx *, int, const int *, const int *, const uint16_t *, int, float,
                                     const float *, long, float, float *, long);

template <typename V>
int spmv_t_launch(hgb_ctx *c, int n_rows, int n_cols, const int *pntr, const int *indx, const V *vals,
                  typename Val<V>::X alpha, const typename Val<V>::X *x, typename Val<V>::X beta,
                  typename Val<V>::X *y, const Transpose *T) {
    using X = typename Val<V>::X;
    if (n_cols <= 0) return HGB_OK;
    int gc = std::max(1, std::min((n_cols + 255) / 256, c->num_sms * 8));
    if (T) {
        spmv_t_cached_kernel<V, false><<<gc, 256, 0, c->stream>>>(n_cols, T->pntr, T->row, T->map, vals, alpha, x,
                                                                 beta, y, nullptr, nullptr, nullptr, nullptr, nullptr);
        return launch_check("spmv_t_cached_kernel");
    }
    scale_or_zero_kernel<X><<<gc, 256, 0, c->stream>>>(n_cols, beta, y);
    if (n_rows > 0) {
        int gr = std::max(1, std::min((n_rows + 255) / 256, c->num_sms * 8));
        spmv_t_atomic_kernel<V><<<gr, 256, 0, c->stream>>>(n_rows, pntr, indx, vals, alpha, x, y);
    }
    return launch_check("spmv_t_atomic_kernel");
}

template int spmv_t_launch<double>(hgb_ctx *, int, int, const int *, const int *, const double *, double,
                                   const double *, double, double *, const Transpose *);
template int spmv_t_launch<float>(hgb_ctx *, int, int, const int *, const int *, const float *, float,
                                  const float *, float, float *, const Transpose *);

}  // namespace hgb

using namespace hgb;

struct hgb_csr {
    hgb_ctx *ctx;
    int n_rows, n_cols, nnz;
    const int *pntr, *indx;
    const void *vals;
    hgb_dtype dtype;
    Transpose T;
    bool has_T = false;
};

namespace hgb {
template <typename T>
__global__ void pattern_grad_kernel(int n_rows, const int *__restrict__ pntr, const int *__restrict__ indx, T alpha,
                                    const T *__restrict__ lam, const T *__restrict__ u, T *__restrict__ grad) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_rows; i += gridDim.x * blockDim.x) {
        const T li = alpha * lam[i];
        for (int p = pntr[i]; p < pntr[i + 1]; p++) grad[p] = li * u[indx[p]];
    }
}

int csr_ensure_transpose(hgb_csr *A) {
    if (A->has_T) return HGB_OK;
    DeviceGuard g(A->ctx->device);
    HGB_TRY(build_transpose(A->ctx, A->n_rows, A->n_cols, A->nnz, A->pntr, A->indx, A->T));
    A->has_T = true;
    return HGB_OK;
}

template <typename V>
int spmv_t_fused_launch(hgb_csr *A, typename Val<V>::X alpha, const typename Val<V>::X *x, typename Val<V>::X beta,
                        typename Val<V>::X *y, const typename Val<V>::X *dot_x, double *dot_out, const int *skip) {
    hgb_ctx *c = A->ctx;
    if (!A->has_T) return fail(HGB_ERR_ARG, "transposed product before the transpose was built");
    const int n = A->n_cols;
    if (n <= 0) return HGB_OK;
    int gc = std::max(1, std::min((n + 255) / 256, std::min(c->num_sms * 8, kMaxReduceBlocks)));
    if (dot_out)
        spmv_t_cached_kernel<V, true><<<gc, 256, 0, c->stream>>>(n, A->T.pntr, A->T.row, A->T.map, (const V *)A->vals,
                                                                alpha, x, beta, y, dot_x, c->partials, c->counter, dot_out, skip);
    else
        spmv_t_cached_kernel<V, false><<<gc, 256, 0, c->stream>>>(n, A->T.pntr, A->T.row, A->T.map, (const V *)A->vals,
                                                                 alpha, x, beta, y, nullptr, nullptr, nullptr, nullptr, skip);
    return launch_check("spmv_t_cached_kernel");
}
template int spmv_t_fused_launch<double>(hgb_csr *, double, const double *, double, double *, const double *, double *, const int *);
template int spmv_t_fused_launch<float>(hgb_csr *, float, const float *, float, float *, const float *, double *, const int *);

const int *csr_pntr(const hgb_csr *A) { return A->pntr; }
const int *csr_indx(const hgb_csr *A) { return A->indx; }
const void *csr_vals(const hgb_csr *A) { return A->vals; }
int csr_rows(const hgb_csr *A) { return A->n_rows; }
int csr_cols(const hgb_csr *A) { return A->n_cols; }
int csr_nnz(const hgb_csr *A) { return A->nnz; }
hgb_dtype csr_dtype(const hgb_csr *A) { return A->dtype; }
hgb_ctx *csr_ctx(const hgb_csr *A) { return A->ctx; }
}  // namespace hgb

static int check_spmv_args(hgb_ctx *c, char trans, int n_rows, int n_cols, int nnz, const int *pntr,
                           const int *indx, const void *vals, const void *x, const void *y) {
    if (!c) return fail(HGB_ERR_ARG, "spmv: null context");
    if (n_rows < 0 || n_cols < 0 || nnz < 0) return fail(HGB_ERR_ARG, "spmv: negative size");
    if (trans != 'N' && trans != 'n' && trans != 'T' && trans != 't' && trans != 'C' && trans != 'c')
        return fail(HGB_ERR_ARG, "spmv: trans '%c'", trans);
    if (n_rows > 0 && !pntr) return fail(HGB_ERR_ARG, "spmv: null pntr");
    if (nnz > 0 && (!indx || !vals)) return fail(HGB_ERR_ARG, "spmv: null indx/vals");
    bool nt = (trans == 'N' || trans == 'n');
    if ((nt ? n_rows : n_cols) > 0 && !y) return fail(HGB_ERR_ARG, "spmv: null y");
    if ((nt ? n_cols : n_rows) > 0 && !x && nnz > 0) return fail(HGB_ERR_ARG, "spmv: null x");
    return HGB_OK;
}

extern "C" {

int hgb_spmv_f64(hgb_ctx *c, char trans, int n_rows, int n_cols, int nnz, const int *pntr, const int *indx,
                 const double *vals, double alpha, const double *x, double beta, double *y) {
    HGB_TRY(check_spmv_args(c, trans, n_rows, n_cols, nnz, pntr, indx, vals, x, y));
    DeviceGuard g(c->device);
    if (trans == 'N' || trans == 'n') return spmv_n_launch<double>(c, n_rows, pntr, indx, vals, alpha, x, beta, y, nullptr, nullptr);
    return spmv_t_launch<double>(c, n_rows, n_cols, pntr, indx, vals, alpha, x, beta, y, nullptr);
}

int hgb_spmv_f32(hgb_ctx *c, char trans, int n_rows, int n_cols, int nnz, const int *pntr, const int *indx,
                 const float *vals, float alpha, const float *x, float beta, float *y) {
    HGB_TRY(check_spmv_args(c, trans, n_rows, n_cols, nnz, pntr, indx, vals, x, y));
    DeviceGuard g(c->device);
    if (trans == 'N' || trans == 'n') return spmv_n_launch<float>(c, n_rows, pntr, indx, vals, alpha, x, beta, y, nullptr, nullptr);
    return spmv_t_launch<float>(c, n_rows, n_cols, pntr, indx, vals, alpha, x, beta, y, nullptr);
}

int hgb_spmv_bf16f32(hgb_ctx *c, char trans, int n_rows, int n_cols, int nnz, const int *pntr,
                     const int *indx, const uint16_t *vals, float alpha, const float *x, float beta, float *y) {
    HGB_TRY(check_spmv_args(c, trans, n_rows, n_cols, nnz, pntr, indx, vals, x, y));
    if (trans != 'N' && trans != 'n') return fail(HGB_ERR_UNSUPPORTED, "spmv_bf16f32: only trans 'N'");
    DeviceGuard g(c->device);
    return spmv_n_launch<uint16_t>(c, n_rows, pntr, indx, vals, alpha, x, beta, y, nullptr, nullptr);
}

int hgb_csr_create(hgb_ctx *c, int n_rows, int n_cols, int nnz, const int *pntr, const int *indx,
                   const void *vals, hgb_dtype dtype, hgb_csr **out) {
    if (!out) return fail(HGB_ERR_ARG, "csr_create: null output");
    *out = nullptr;
    HGB_TRY(check_spmv_args(c, 'N', n_rows, n_cols, nnz, pntr, indx, vals, pntr, pntr));
    if (dtype != HGB_F64 && dtype != HGB_F32 && dtype != HGB_BF16 && dtype != HGB_C128 && dtype != HGB_C64)
        return fail(HGB_ERR_ARG, "csr_create: dtype");
    DeviceGuard g(c->device);
    HGB_TRY(csr_check(c, n_rows, n_cols, nnz, pntr, indx));
    hgb_csr *A = new hgb_csr();
    A->ctx = c;
    A->n_rows = n_rows;
    A->n_cols = n_cols;
    A->nnz = nnz;
    A->pntr = pntr;
    A->indx = indx;
    A->vals = vals;
    A->dtype = dtype;
    *out = A;
    return HGB_OK;
}

int hgb_csr_gemv(hgb_csr *A, char trans, double alpha, const void *x, double beta, void *y) {
    if (!A) return fail(HGB_ERR_ARG, "csr_gemv: null matrix");
    hgb_ctx *c = A->ctx;
    HGB_TRY(check_spmv_args(c, trans, A->n_rows, A->n_cols, A->nnz, A->pntr, A->indx, A->vals, x, y));
    DeviceGuard g(c->device);
    bool nt = (trans == 'N' || trans == 'n');
    if (A->dtype == HGB_C128 || A->dtype == HGB_C64) {
        const double a[2] = {alpha, 0.0}, b[2] = {beta, 0.0};
        return hgb_csr_gemv_z(A, trans, a, x, b, y);
    }
    if (nt) {
        switch (A->dtype) {
            case HGB_F64: return spmv_n_launch<double>(c, A->n_rows, A->pntr, A->indx, (const double *)A->vals, alpha, (const double *)x, beta, (double *)y, nullptr, nullptr);
            case HGB_F32: return spmv_n_launch<float>(c, A->n_rows, A->pntr, A->indx, (const float *)A->vals, (float)alpha, (const float *)x, (float)beta, (float *)y, nullptr, nullptr);
            default: return spmv_n_launch<uint16_t>(c, A->n_rows, A->pntr, A->indx, (const uint16_t *)A->vals, (float)alpha, (const float *)x, (float)beta, (float *)y, nullptr, nullptr);
        }
    }
    if (A->dtype == HGB_BF16) return fail(HGB_ERR_UNSUPPORTED, "csr_gemv: transpose of a bf16 matrix");
    if (!A->has_T) {
        HGB_TRY(build_transpose(c, A->n_rows, A->n_cols, A->nnz, A->pntr, A->indx, A->T));
        A->has_T = true;
    }
    if (A->dtype == HGB_F64)
        return spmv_t_launch<double>(c, A->n_rows, A->n_cols, A->pntr, A->indx, (const double *)A->vals, alpha, (const double *)x, beta, (double *)y, &A->T);
    return spmv_t_launch<float>(c, A->n_rows, A->n_cols, A->pntr, A->indx, (const float *)A->vals, (float)alpha, (const float *)x, (float)beta, (float *)y, &A->T);
}

int hgb_csr_gemv_z(hgb_csr *A, char trans, const double *alpha, const void *x, const double *beta, void *y) {
    if (!A || !alpha || !beta) return fail(HGB_ERR_ARG, "csr_gemv_z: bad arguments");
    if (A->dtype != HGB_C128 && A->dtype != HGB_C64) return fail(HGB_ERR_ARG, "csr_gemv_z: a complex matrix");
    hgb_ctx *c = A->ctx;
    HGB_TRY(check_spmv_args(c, trans, A->n_rows, A->n_cols, A->nnz, A->pntr, A->indx, A->vals, x, y));
    DeviceGuard g(c->device);
    const bool nt = (trans == 'N' || trans == 'n');
    if (!nt && !A->has_T) {
        HGB_TRY(build_transpose(c, A->n_rows, A->n_cols, A->nnz, A->pntr, A->indx, A->T));
        A->has_T = true;
    }
    const Transpose *T = nt ? nullptr : &A->T;
    if (A->dtype == HGB_C128)
        return zspmv<double>(c, trans, A->n_rows, A->n_cols, A->pntr, A->indx, A->vals, alpha, x, beta, y, T);
    const float a[2] = {(float)alpha[0], (float)alpha[1]}, b[2] = {(float)beta[0], (float)beta[1]};
    return zspmv<float>(c, trans, A->n_rows, A->n_cols, A->pntr, A->indx, A->vals, a, x, b, y, T);
}

int hgb_spmv_c128(hgb_ctx *c, char trans, int n_rows, int n_cols, int nnz, const int *pntr, const int *indx,
                  const void *vals, const double *alpha, const void *x, const double *beta, void *y) {
    HGB_TRY(check_spmv_args(c, trans, n_rows, n_cols, nnz, pntr, indx, vals, x, y));
    if (!alpha || !beta) return fail(HGB_ERR_ARG, "spmv_c128: null scalar");
    DeviceGuard g(c->device);
    return zspmv<double>(c, trans, n_rows, n_cols, pntr, indx, vals, alpha, x, beta, y, nullptr);
}

int hgb_spmv_c64(hgb_ctx *c, char trans, int n_rows, int n_cols, int nnz, const int *pntr, const int *indx,
                 const void *vals, const float *alpha, const void *x, const float *beta, void *y) {
    HGB_TRY(check_spmv_args(c, trans, n_rows, n_cols, nnz, pntr, indx, vals, x, y));
    if (!alpha || !beta) return fail(HGB_ERR_ARG, "spmv_c64: null scalar");
    DeviceGuard g(c->device);
    return zspmv<float>(c, trans, n_rows, n_cols, pntr, indx, vals, alpha, x, beta, y, nullptr);
}

int hgb_csr_gemv_dot(hgb_csr *A, const void *x, void *y, double *dot_out) {
    if (!A || !dot_out) return fail(HGB_ERR_ARG, "csr_gemv_dot: bad arguments");
    if (A->dtype == HGB_C128 || A->dtype == HGB_C64) return fail(HGB_ERR_UNSUPPORTED, "csr_gemv_dot: real matrices");
    if (A->n_rows != A->n_cols) return fail(HGB_ERR_ARG, "csr_gemv_dot: square matrix required");
    hgb_ctx *c = A->ctx;
    DeviceGuard g(c->device);
    switch (A->dtype) {
        case HGB_F64: return spmv_n_launch<double>(c, A->n_rows, A->pntr, A->indx, (const double *)A->vals, 1.0, (const double *)x, 0.0, (double *)y, dot_out, nullptr);
        case HGB_F32: return spmv_n_launch<float>(c, A->n_rows, A->pntr, A->indx, (const float *)A->vals, 1.0f, (const float *)x, 0.0f, (float *)y, dot_out, nullptr);
        default: return spmv_n_launch<uint16_t>(c, A->n_rows, A->pntr, A->indx, (const uint16_t *)A->vals, 1.0f, (const float *)x, 0.0f, (float *)y, dot_out, nullptr);
    }
}

int hgb_csr_pattern_grad(hgb_csr *A, double alpha, const void *lam, const void *u, void *grad) {
    if (!A || !lam || !u || !grad) return fail(HGB_ERR_ARG, "csr_pattern_grad: bad arguments");
    if (A->dtype != HGB_F64 && A->dtype != HGB_F32) return fail(HGB_ERR_UNSUPPORTED, "csr_pattern_grad: F64 or F32 matrices");
    hgb_ctx *c = A->ctx;
    DeviceGuard g(c->device);
    if (A->n_rows == 0) return HGB_OK;
    int gr = std::max(1, std::min((A->n_rows + 255) / 256, c->num_sms * 8));
    if (A->dtype == HGB_F64)
        pattern_grad_kernel<double><<<gr, 256, 0, c->stream>>>(A->n_rows, A->pntr, A->indx, alpha, (const double *)lam, (const double *)u, (double *)grad);
    else
        pattern_grad_kernel<float><<<gr, 256, 0, c->stream>>>(A->n_rows, A->pntr, A->indx, (float)alpha, (const float *)lam, (const float *)u, (float *)grad);
    return launch_check("pattern_grad_kernel");
}

int hgb_csr_destroy(hgb_csr *A) {
    if (!A) return HGB_OK;
    DeviceGuard g(A->ctx->device);
    if (A->has_T) A->T.release();
    delete A;
    return HGB_OK;
}

}  // extern "C"
