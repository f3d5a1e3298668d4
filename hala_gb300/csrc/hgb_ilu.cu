// ILU(0) factorisation and sparse triangular solves for sm_103a.
//
// Both are sync-free: no grid-wide barrier, no per-level launch.  Work is handed out through an
// atomic ticket in an order where everything a row depends on was handed out earlier, so a warp
// only ever waits on warps that are already running, and each wait is bounded.
//
//  * Factorisation (and the forward level sets): warps take chunks of 32 consecutive rows in
//    natural order and process them row by row; a row waits on the completion flags of the rows
//    named by its strictly-lower entries.  The update order of every entry is the pivot order of
//    factorize_ilu_array (sparse/hala_sparse_utils.hpp:229-255), with separately rounded multiply
//    and subtract, so the factor is bit-identical to the reference CPU factor.
//  * Triangular solves: rows are grouped by level into tasks of up to 32 rows of ONE level; a
//    lane owns a row, reads its entries in the reference's order and waits on the solution
//    entries it needs.  A solution entry not yet produced holds a signalling-NaN pattern, so the
//    value is its own ready flag (one L2 round trip per dependency).
#include "hgb_internal.cuh"
#include "hgb_kernels.cuh"
#include "hgb_bsolve.cuh"
#include "hgb_complex.cuh"

#include <algorithm>
#include <cstdlib>
#include <string>
#include <thread>
#include <vector>

namespace hgb {

// ------------------------------------------------------------------ schedule ------------
struct Schedule {
    int n = 0, nlevels = 0, ntasks = 0;
    int *level = nullptr;   // [n]
    int *perm = nullptr;    // [n] rows grouped by level
    int2 *tasks = nullptr;  // [ntasks] (offset into perm, row count <= 32), level-major
    int *ticket = nullptr;  // [2] ticket and exit counter, self-resetting
    void release() {
        cudaFree(level);
        cudaFree(perm);
        cudaFree(tasks);
        cudaFree(ticket);
        level = perm = nullptr;
        tasks = nullptr;
        ticket = nullptr;
    }
};

__device__ __forceinline__ int ld_relaxed_int(const int *p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_int(int *p, int v) {
    asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// bounded wait until lev[j] >= 0; acquire so that data published before the flag is visible
__device__ __forceinline__ int wait_level(const int *lev, int j, int *err) {
    int v = ld_acquire(lev + j);
    int spins = 0;
    while (v < 0) {
        if (++spins > kSpinLimit) {
            atomicOr(err, DEV_ERR_TIMEOUT);
            return 0;
        }
        v = ld_acquire(lev + j);
    }
    return v;
}

// Level sets over the pattern: lower: deps are entries [pntr_i, diag_i) and rows are taken in
// ascending order; upper: deps (diag_i, pntr_{i+1}) and rows in descending order.
// lev[] starts at -1 everywhere; a row's level is its published completion flag.
__global__ void __launch_bounds__(256) levels_kernel(int n, const int *__restrict__ pntr,
                                                     const int *__restrict__ indx,
                                                     const int *__restrict__ diag, int lower, int *lev,
                                                     int *ticket, int *err) {
    __shared__ int chunk_lev[8][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nchunks = (n + 31) / 32;
    for (;;) {
        int c = 0;
        if (lane == 0) c = atomicAdd(ticket, 1);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (c >= nchunks) break;
        // chunk c covers processing positions [32c, 32c+32)
        for (int k = 0; k < 32; k++) {
            int pos = c * 32 + k;
            if (pos >= n) break;
            int row = lower ? pos : n - 1 - pos;
            int a = lower ? __ldg(pntr + row) : __ldg(diag + row) + 1;
            int b = lower ? __ldg(diag + row) : __ldg(pntr + row + 1);
            int m = -1;
            for (int p = a + lane; p < b; p += 32) {
                int j = __ldg(indx + p);
                int jpos = lower ? j : n - 1 - j;
                int lj = (jpos >= c * 32) ? chunk_lev[w][jpos - c * 32] : wait_level(lev, j, err);
                m = max(m, lj);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0) {
                chunk_lev[w][k] = m + 1;
                st_release(lev + row, m + 1);
            }
            __syncwarp();
        }
    }
    // last CTA out resets the ticket for the next launch
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(ticket + 1, 1) == (int)gridDim.x - 1) {
            ticket[0] = 0;
            ticket[1] = 0;
        }
    }
}


template <typename T> __device__ __forceinline__ T ld_val(const T *p) { return ld_relaxed(p); }

// Row-wise IKJ ILU(0) in place on f (a copy of the matrix values) + forward level sets.
template <typename T>
__global__ void __launch_bounds__(256) ilu_factor_kernel(int n, const int *__restrict__ pntr,
                                                         const int *__restrict__ indx,
                                                         const int *__restrict__ diag, T *f, int *lev,
                                                         int *ticket, int *err) {
    __shared__ int chunk_lev[8][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nchunks = (n + 31) / 32;
    for (;;) {
        int c = 0;
        if (lane == 0) c = atomicAdd(ticket, 1);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (c >= nchunks) break;
        for (int k = 0; k < 32; k++) {
            const int i = c * 32 + k;
            if (i >= n) break;
            const int a = __ldg(pntr + i), b = __ldg(pntr + i + 1), d = __ldg(diag + i);
            int m = -1;
            for (int p = a; p < d; p++) {          // pivots in ascending column order
                const int kr = __ldg(indx + p);
                int lk;
                if (kr >= c * 32) lk = chunk_lev[w][kr - c * 32];
                else lk = wait_level(lev, kr, err);   // every lane waits: acquire per lane
                m = max(m, lk);
                const int dk = __ldg(diag + kr), ek = __ldg(pntr + kr + 1);
                const T ukk = ld_val(f + dk);
                // owner lane of position p scales a_ik; everyone gets l from it
                const int owner = (p - a) & 31;
                T l = T(0);
                if (lane == owner) {
                    l = div_rn(f[p], ukk);
                    f[p] = l;
                    if (ukk == T(0)) atomicOr(err, DEV_ERR_ZERO_PIVOT);
                }
                l = __shfl_sync(0xffffffffu, l, owner);
                // a_iq -= l * a_kq for q > p with column present in row k's upper part
                for (int q = p + 1 + ((lane - (p + 1 - a)) & 31); q < b; q += 32) {
                    const int jc = __ldg(indx + q);
                    int lo = dk + 1, hi = ek - 1, pos = -1;
                    while (lo <= hi) {
                        int mid = (lo + hi) >> 1;
                        int cm = __ldg(indx + mid);
                        if (cm == jc) { pos = mid; break; }
                        if (cm < jc) lo = mid + 1; else hi = mid - 1;
                    }
                    if (pos >= 0) f[q] = sub_rn(f[q], mul_rn(l, ld_val(f + pos)));
                }
                __syncwarp();
            }
            if (lane == ((d - a) & 31) && ld_val(f + d) == T(0)) atomicOr(err, DEV_ERR_ZERO_PIVOT);
            __threadfence();
            __syncwarp();
            if (lane == 0) {
                chunk_lev[w][k] = m + 1;
                st_release(lev + i, m + 1);
            }
            __syncwarp();
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(ticket + 1, 1) == (int)gridDim.x - 1) {
            ticket[0] = 0;
            ticket[1] = 0;
        }
    }
}

__global__ void max_level_kernel(int n, const int *__restrict__ lev, int *out) {
    int m = -1;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = max(m, lev[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void level_hist_kernel(int n, const int *__restrict__ lev, int *cnt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) atomicAdd(cnt + lev[i], 1);
}

__global__ void task_count_kernel(int nl, const int *__restrict__ cnt, int *tcnt) {
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < nl; l += gridDim.x * blockDim.x) tcnt[l] = (cnt[l] + 31) / 32;
}

__global__ void level_scatter_kernel(int n, int lower, const int *__restrict__ lev, const int *__restrict__ lptr,
                                     int *cursor, int *perm) {
    // rows visited in the solve's order so that warp-aggregated slots come out roughly ordered
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int row = lower ? t : n - 1 - t;
        int l = lev[row];
        perm[lptr[l] + atomicAdd(cursor + l, 1)] = row;
    }
}

__global__ void task_fill_kernel(int nl, const int *__restrict__ cnt, const int *__restrict__ lptr,
                                 const int *__restrict__ tptr, int2 *tasks) {
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < nl; l += gridDim.x * blockDim.x) {
        int c = cnt[l], t0 = tptr[l];
        for (int t = 0; 32 * t < c; t++) tasks[t0 + t] = make_int2(lptr[l] + 32 * t, min(32, c - 32 * t));
    }
}

// Build the schedule from a completed level array (S.level filled, S.n set).
static int build_schedule(hgb_ctx *c, Schedule &S, int lower) {
    const int n = S.n;
    int *dmax = nullptr;
    HGB_CUDA(cudaMalloc(&dmax, sizeof(int) * 2));
    HGB_CUDA(cudaMemsetAsync(dmax, 0xff, sizeof(int), c->stream));
    int g = std::max(1, std::min((n + 255) / 256, c->num_sms * 8));
    max_level_kernel<<<g, 256, 0, c->stream>>>(n, S.level, dmax);
    int mx = -1;
    HGB_CUDA(cudaMemcpyAsync(&mx, dmax, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    const int nl = mx + 1;
    S.nlevels = nl;
    int *cnt = nullptr, *lptr = nullptr, *tcnt = nullptr, *tptr = nullptr, *scratch = nullptr;
    size_t nb = (size_t)(nl + 1 + 1023) / 1024 + 2;
    HGB_CUDA(cudaMalloc(&cnt, sizeof(int) * (nl + 1)));
    HGB_CUDA(cudaMalloc(&lptr, sizeof(int) * (nl + 1)));
    HGB_CUDA(cudaMalloc(&tcnt, sizeof(int) * (nl + 1)));
    HGB_CUDA(cudaMalloc(&tptr, sizeof(int) * (nl + 1)));
    HGB_CUDA(cudaMalloc(&scratch, sizeof(int) * nb));
    HGB_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * (nl + 1), c->stream));
    level_hist_kernel<<<g, 256, 0, c->stream>>>(n, S.level, cnt);
    HGB_TRY(exclusive_scan(c, cnt, lptr, nl + 1, scratch + nb - 1, scratch));
    int gl = std::max(1, std::min((nl + 255) / 256, c->num_sms * 8));
    task_count_kernel<<<gl, 256, 0, c->stream>>>(nl, cnt, tcnt);
    HGB_CUDA(cudaMemsetAsync(tcnt + nl, 0, sizeof(int), c->stream));
    HGB_TRY(exclusive_scan(c, tcnt, tptr, nl + 1, scratch + nb - 1, scratch));
    int ntasks = 0;
    HGB_CUDA(cudaMemcpyAsync(&ntasks, tptr + nl, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    S.ntasks = ntasks;
    HGB_CUDA(cudaMalloc(&S.perm, sizeof(int) * n));
    HGB_CUDA(cudaMalloc(&S.tasks, sizeof(int2) * std::max(ntasks, 1)));
    HGB_CUDA(cudaMemsetAsync(tcnt, 0, sizeof(int) * (nl + 1), c->stream));
    level_scatter_kernel<<<g, 256, 0, c->stream>>>(n, lower, S.level, lptr, tcnt, S.perm);
    task_fill_kernel<<<gl, 256, 0, c->stream>>>(nl, cnt, lptr, tptr, S.tasks);
    HGB_TRY(launch_check("build_schedule"));
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    cudaFree(dmax);
    cudaFree(cnt);
    cudaFree(lptr);
    cudaFree(tcnt);
    cudaFree(tptr);
    cudaFree(scratch);
    return HGB_OK;
}

static int alloc_schedule(hgb_ctx *c, Schedule &S, int n) {
    S.n = n;
    HGB_CUDA(cudaMalloc(&S.level, sizeof(int) * n));
    HGB_CUDA(cudaMalloc(&S.ticket, sizeof(int) * 2));
    HGB_CUDA(cudaMemsetAsync(S.level, 0xff, sizeof(int) * n, c->stream));
    HGB_CUDA(cudaMemsetAsync(S.ticket, 0, sizeof(int) * 2, c->stream));
    return HGB_OK;
}

static int sync_grid(hgb_ctx *c, int work_items, int per_block) {
    int g = (work_items + per_block - 1) / per_block;
    return std::max(1, std::min(g, c->num_sms * 8));
}

// Levels of one solve direction over (pntr, indx, diag), then the schedule.
static int analyse(hgb_ctx *c, int n, const int *pntr, const int *indx, const int *diag, int lower, Schedule &S) {
    HGB_TRY(alloc_schedule(c, S, n));
    levels_kernel<<<sync_grid(c, (n + 31) / 32, 8), 256, 0, c->stream>>>(n, pntr, indx, diag, lower, S.level,
                                                                         S.ticket, c->err);
    HGB_TRY(launch_check("levels_kernel"));
    HGB_TRY(collect_dev_error(c));
    return build_schedule(c, S, lower);
}

// ------------------------------------------------------------ triangular solve ---------
enum SolveMode : int {
    MODE_ILU = 0,    // acc = in_i ; acc -= v * x_j ...   (apply_ilu_array, utils:263-276)
    MODE_TRSV = 1    // s = 0 ; s += v * x_j ... ; acc = alpha*in_i - s  (sparse_trsv_array)
};

struct SolveArgs {
    int ntasks;
    const int2 *tasks;
    const int *perm;
    int *ticket;
    const int *pntr, *indx, *diag;   // diag[i] = position of the diagonal entry of row i
    const int *map;                  // optional value gather (transposed view), may be null
    const double *piv;               // optional FP64 pivots (division in FP64), may be null
    int lower, unit, mode, rev;
    int *err;
    const int *skip;                 // optional device flag: the launch is a no-op when set
};

// Polls up to 8 pending solution entries together (one L2 round trip when they are ready).
template <typename X>
__device__ __forceinline__ void wait_values(const X *out, const int (&jj)[8], X (&xv)[8], int cnt, int *err) {
    unsigned pending = 0;
#pragma unroll
    for (int k = 0; k < 8; k++)
        if (k < cnt) {
            xv[k] = ld_relaxed(out + jj[k]);
            if (Pending<X>::is(xv[k])) pending |= 1u << k;
        }
    int spins = 0;
    while (pending) {
        ++spins;
        if (spins > kSpinLimit || ((spins & 4095) == 0 && (*(volatile int *)err & DEV_ERR_TIMEOUT))) {
            atomicOr(err, DEV_ERR_TIMEOUT);
#pragma unroll
            for (int k = 0; k < 8; k++)
                if (pending & (1u << k)) xv[k] = Pending<X>::canon(Pending<X>::value());
            return;
        }
#pragma unroll
        for (int k = 0; k < 8; k++)
            if (pending & (1u << k)) {
                xv[k] = ld_relaxed(out + jj[k]);
                if (!Pending<X>::is(xv[k])) pending &= ~(1u << k);
            }
    }
}

template <typename V, typename X>
__global__ void __launch_bounds__(256) trsv_kernel(SolveArgs A, const V *__restrict__ vals, X alpha,
                                                   const X *in, X *out, X *pend_a, X *pend_b) {
    if (A.skip && *A.skip) return;
    const int lane = threadIdx.x & 31;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(A.ticket, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= A.ntasks) break;
        const int2 task = __ldg(A.tasks + t);
        if (lane < task.y) {
            const int row = __ldg(A.perm + task.x + lane);
            const int d = __ldg(A.diag + row);
            int a, b;
            if (A.lower) { a = __ldg(A.pntr + row); b = d; }
            else { a = d + 1; b = __ldg(A.pntr + row + 1); }
            const X xin = in[row];
            const X dval = A.unit ? X(1) : Val<V>::get(__ldg(vals + (A.map ? __ldg(A.map + d) : d)));
            X acc = (A.mode == MODE_ILU) ? xin : X(0);
            const int len = b - a;
            for (int k0 = 0; k0 < len; k0 += 8) {
                const int cnt = min(8, len - k0);
                int jj[8];
                X vv[8], xv[8];
#pragma unroll
                for (int k = 0; k < 8; k++)
                    if (k < cnt) {
                        const int p = A.rev ? b - 1 - (k0 + k) : a + k0 + k;
                        jj[k] = __ldg(A.indx + p);
                        vv[k] = Val<V>::get(__ldg(vals + (A.map ? __ldg(A.map + p) : p)));
                    }
                wait_values<X>(out, jj, xv, cnt, A.err);
#pragma unroll
                for (int k = 0; k < 8; k++)
                    if (k < cnt) {
                        if (A.mode == MODE_ILU) acc = sub_rn(acc, mul_rn(vv[k], xv[k]));
                        else acc = add_rn(acc, mul_rn(vv[k], xv[k]));
                    }
            }
            if (A.mode == MODE_TRSV) acc = sub_rn(mul_rn(alpha, xin), acc);
            if (!A.unit) {
                if (A.piv) acc = (X)__ddiv_rn((double)acc, __ldg(A.piv + row));
                else acc = div_rn(acc, dval);
            }
            st_relaxed(out + row, Pending<X>::canon(acc));
            if (pend_a) pend_a[row] = Pending<X>::value();
            if (pend_b) pend_b[row] = Pending<X>::value();
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(A.ticket + 1, 1) == (int)gridDim.x - 1) {
            A.ticket[0] = 0;
            A.ticket[1] = 0;
        }
    }
}

template <typename X>
__global__ void fill_pending_kernel(long n, X *p) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        p[i] = Pending<X>::value();
}

template <typename X>
static int fill_pending(hgb_ctx *c, long n, X *p) {
    if (n <= 0) return HGB_OK;
    fill_pending_kernel<X><<<std::max(1, (int)std::min<long>((n + 255) / 256, c->num_sms * 8)), 256, 0, c->stream>>>(n, p);
    return launch_check("fill_pending_kernel");
}

// CTAs (of 8 warps) per SM for the global-level sync-free solves: more warps hold tasks further
// ahead of the wavefront, all of them polling L2.
constexpr int kTrsvBlocksPerSm = 4;

template <typename V, typename X>
static int launch_solve(hgb_ctx *c, const Schedule &S, SolveArgs A, const V *vals, X alpha, const X *in, X *out,
                        X *pend_a, X *pend_b) {
    if (S.n == 0) return HGB_OK;
    A.ntasks = S.ntasks;
    A.tasks = S.tasks;
    A.perm = S.perm;
    A.ticket = S.ticket;
    A.err = c->err;
    int blocks = std::max(1, std::min((S.ntasks + 7) / 8, c->num_sms * kTrsvBlocksPerSm));
    trsv_kernel<V, X><<<blocks, 256, 0, c->stream>>>(A, vals, alpha, in, out, pend_a, pend_b);
    return launch_check("trsv_kernel");
}

// bf16 conversion of the factor for the bf16-store variant
__global__ void f64_to_store_kernel(long n, const double *__restrict__ src, float *f32, uint16_t *b16) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        float v = (float)src[i];
        if (f32) f32[i] = v;
        if (b16) {
            uint32_t u = __float_as_uint(v);
            uint16_t r;
            if ((u & 0x7fffffffu) > 0x7f800000u) r = (uint16_t)((u >> 16) | 0x40u);
            else r = (uint16_t)((u + 0x7fffu + ((u >> 16) & 1u)) >> 16);
            b16[i] = r;
        }
    }
}

__global__ void gather_pivots_kernel(int n, const int *__restrict__ diag, const double *__restrict__ f, double *piv) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) piv[i] = f[diag[i]];
}

template <typename T>
__global__ void gather_kernel(long n, const int *__restrict__ map, const T *__restrict__ src, T *dst) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        dst[i] = src[map[i]];
}

}  // namespace hgb

using namespace hgb;

// ======================================================================= ILU object =====
struct hgb_ilu {
    hgb_ctx *ctx = nullptr;
    int n = 0, nnz = 0;
    const int *pntr = nullptr, *indx = nullptr;
    hgb_dtype fdtype = HGB_F64, store = HGB_F64;
    void *fvals = nullptr;      // factor in the factorisation precision
    void *svals = nullptr;      // factor in the store precision (== fvals when equal)
    double *piv = nullptr;      // FP64 pivots for the F32/BF16 stores of an FP64 factor
    int *diag = nullptr;
    Schedule L, U;
    void *tmp = nullptr;        // forward-solve output, kept in the pending state between applies
    bool tmp_ready = false;
    unsigned tmp_epoch = 0;     // context error epoch at the last refill of tmp
    // transposed view (built on first trans='T' apply)
    bool has_T = false;
    Transpose T;
    int *diagT = nullptr;
    void *svalsT = nullptr;
    double *pivT = nullptr;     // same pivots as piv (diagonal entries are their own transpose)
    Schedule LT, UT;
    // block-local level schedules (hgb_bsolve.cu); the global-level kernel is the fallback
    bool use_bs = false, use_bsT = false;
    BlockSolve BL, BU, BLT, BUT;
    hgb_zilu *z = nullptr;      // the complex factor (C128 / C64); none of the fields above is used then
    // host-buffer creation: the object owns its device copies of the pattern and the values
    int *own_pntr = nullptr, *own_indx = nullptr;
    void *own_vals = nullptr;
};

namespace hgb {

static size_t vsize(hgb_dtype t) {
    return t == HGB_C128 ? 16 : (t == HGB_F64 || t == HGB_C64) ? 8 : (t == HGB_F32 ? 4 : 2);
}
static size_t xsize(hgb_dtype store) { return store == HGB_BF16 ? 4 : vsize(store); }

static void ilu_free(hgb_ilu *M) {
    if (!M) return;
    if (M->svals && M->svals != M->fvals) cudaFree(M->svals);
    cudaFree(M->fvals);
    cudaFree(M->piv);
    cudaFree(M->diag);
    cudaFree(M->tmp);
    M->L.release();
    M->U.release();
    if (M->has_T) {
        M->T.release();
        cudaFree(M->diagT);
        cudaFree(M->svalsT);
        M->LT.release();
        M->UT.release();
    }
    M->BL.release();
    M->BU.release();
    M->BLT.release();
    M->BUT.release();
    cudaFree(M->own_pntr);
    cudaFree(M->own_indx);
    cudaFree(M->own_vals);
    zilu_destroy(M->z);
    delete M;
}

template <typename V, typename X>
static int ilu_apply_n(hgb_ilu *M, const void *x, void *r, const int *skip) {
    hgb_ctx *c = M->ctx;
    X *tmp = (X *)M->tmp;
    if (!M->tmp_ready) {
        HGB_TRY(fill_pending<X>(c, M->n, tmp));
        M->tmp_ready = true;
        M->tmp_epoch = c->error_epoch;
    }
    if (M->use_bs) {
        // forward: unit lower, tmp <- L^-1 x (r reset to pending); backward: r <- U^-1 tmp
        HGB_TRY(bsolve_launch<V, X>(c, M->BL, MODE_ILU, 1, X(1), (const X *)x, tmp, (X *)r, skip));
        HGB_TRY(bsolve_launch<V, X>(c, M->BU, MODE_ILU, 0, X(1), tmp, (X *)r, tmp, skip));
        return HGB_OK;
    }
    SolveArgs A{};
    A.pntr = M->pntr;
    A.indx = M->indx;
    A.diag = M->diag;
    A.map = nullptr;
    A.piv = M->piv;
    A.skip = skip;
    A.mode = MODE_ILU;
    A.rev = 0;
    // forward: unit lower, tmp <- L^-1 x ; the row's slot of r is reset to pending for the backward solve
    A.lower = 1;
    A.unit = 1;
    HGB_TRY(launch_solve<V, X>(c, M->L, A, (const V *)M->svals, X(1), (const X *)x, tmp, (X *)r, nullptr));
    // backward: r <- U^-1 tmp ; tmp goes back to pending for the next apply
    A.lower = 0;
    A.unit = 0;
    HGB_TRY(launch_solve<V, X>(c, M->U, A, (const V *)M->svals, X(1), tmp, (X *)r, tmp, nullptr));
    return HGB_OK;
}

static int ilu_build_T(hgb_ilu *M) {
    hgb_ctx *c = M->ctx;
    HGB_TRY(build_transpose(c, M->n, M->n, M->nnz, M->pntr, M->indx, M->T));
    HGB_CUDA(cudaMalloc(&M->diagT, sizeof(int) * M->n));
    int st = hgb_diag_index(c, M->n, M->nnz, M->T.pntr, M->T.row, M->diagT);
    if (st) return st;
    size_t vs = vsize(M->store);
    HGB_CUDA(cudaMalloc(&M->svalsT, vs * std::max(M->nnz, 1)));
    int g = std::max(1, std::min((M->nnz + 255) / 256, c->num_sms * 8));
    if (vs == 8) gather_kernel<double><<<g, 256, 0, c->stream>>>(M->nnz, M->T.map, (const double *)M->svals, (double *)M->svalsT);
    else if (vs == 4) gather_kernel<float><<<g, 256, 0, c->stream>>>(M->nnz, M->T.map, (const float *)M->svals, (float *)M->svalsT);
    else gather_kernel<uint16_t><<<g, 256, 0, c->stream>>>(M->nnz, M->T.map, (const uint16_t *)M->svals, (uint16_t *)M->svalsT);
    HGB_TRY(launch_check("gather_kernel"));
    // U^T is the lower triangle of the transposed pattern, L^T its upper triangle
    HGB_TRY(analyse(c, M->n, M->T.pntr, M->T.row, M->diagT, 1, M->LT));
    HGB_TRY(analyse(c, M->n, M->T.pntr, M->T.row, M->diagT, 0, M->UT));
    if (M->use_bs) {
        const int R = bsolve_rows(c, (int)xsize(M->store), M->n);
        int st = bsolve_analyse(c, M->n, M->nnz, M->T.pntr, M->T.row, M->diagT, 1, 0, R, (int)xsize(M->store), M->BLT);
        if (!st) st = bsolve_analyse(c, M->n, M->nnz, M->T.pntr, M->T.row, M->diagT, 0, 1, R, (int)xsize(M->store), M->BUT);
        if (!st) st = bsolve_load_values(c, M->BLT, M->svalsT, (int)vsize(M->store), M->piv);
        if (!st) st = bsolve_load_values(c, M->BUT, M->svalsT, (int)vsize(M->store), nullptr);
        if (st == HGB_OK) M->use_bsT = true;
        else if (st != HGB_ERR_UNSUPPORTED) return st;
    }
    M->has_T = true;
    return HGB_OK;
}

// (LU)^-T x = L^-T (U^-T x): U^T w = x (lower, non-unit), then L^T r = w (upper, unit, entries
// visited in descending original row), both with the sum-then-subtract order of the reference's
// transposed triangular solve (sparse_trsv_array 'T', utils:318-335).
template <typename V, typename X>
static int ilu_apply_t(hgb_ilu *M, const void *x, void *r, const int *skip) {
    hgb_ctx *c = M->ctx;
    if (!M->has_T) HGB_TRY(ilu_build_T(M));
    X *tmp = (X *)M->tmp;
    if (!M->tmp_ready) {
        HGB_TRY(fill_pending<X>(c, M->n, tmp));
        M->tmp_ready = true;
        M->tmp_epoch = c->error_epoch;
    }
    if (M->use_bsT) {
        HGB_TRY(bsolve_launch<V, X>(c, M->BLT, MODE_TRSV, 0, X(1), (const X *)x, tmp, (X *)r, skip));
        HGB_TRY(bsolve_launch<V, X>(c, M->BUT, MODE_TRSV, 1, X(1), tmp, (X *)r, tmp, skip));
        return HGB_OK;
    }
    SolveArgs A{};
    A.pntr = M->T.pntr;
    A.indx = M->T.row;
    A.diag = M->diagT;
    A.map = nullptr;
    A.piv = M->piv;
    A.skip = skip;
    A.mode = MODE_TRSV;
    A.lower = 1;
    A.unit = 0;
    A.rev = 0;
    HGB_TRY(launch_solve<V, X>(c, M->LT, A, (const V *)M->svalsT, X(1), (const X *)x, tmp, (X *)r, nullptr));
    A.lower = 0;
    A.unit = 1;
    A.rev = 1;
    HGB_TRY(launch_solve<V, X>(c, M->UT, A, (const V *)M->svalsT, X(1), tmp, (X *)r, tmp, nullptr));
    return HGB_OK;
}

}  // namespace hgb

// ================================================================ triangular object =====
struct hgb_tri {
    hgb_ctx *ctx = nullptr;
    int n = 0, nnz = 0;
    char uplo = 'L', diagc = 'N';
    const int *pntr = nullptr, *indx = nullptr;
    const void *vals = nullptr;
    hgb_dtype dtype = HGB_F64;
    int *diag = nullptr;
    Schedule S;
    hgb_ztri *z = nullptr;     // the complex triangle (C128 / C64)
    bool has_T = false;
    Transpose T;
    int *diagT = nullptr;
    Schedule ST;
    void *bcopy = nullptr;     // staging when b aliases x
};

extern "C" {

static int ilu_check_args(hgb_ctx *c, int n, int nnz, const void *pntr, const void *indx, const void *vals,
                          hgb_dtype vals_dtype, hgb_dtype store) {
    if (!c || n <= 0 || nnz < n || !pntr || !indx || !vals) return fail(HGB_ERR_ARG, "ilu0_create: bad arguments (n=%d nnz=%d)", n, nnz);
    if (vals_dtype == HGB_C128 || vals_dtype == HGB_C64) {
        if (store != vals_dtype) return fail(HGB_ERR_UNSUPPORTED, "ilu0_create: a complex factor is stored in its own precision");
        return HGB_OK;
    }
    if (vals_dtype != HGB_F64 && vals_dtype != HGB_F32) return fail(HGB_ERR_ARG, "ilu0_create: vals dtype must be F64, F32, C128 or C64");
    if (store != HGB_F64 && store != HGB_F32 && store != HGB_BF16) return fail(HGB_ERR_ARG, "ilu0_create: store dtype");
    if (vals_dtype == HGB_F32 && store != HGB_F32) return fail(HGB_ERR_UNSUPPORTED, "ilu0_create: an F32 factor is stored as F32");
    return HGB_OK;
}

// The device part of ILU(0) creation.  plan: when given, the block-solve schedules were planned on
// the host already (from host arrays); otherwise they are planned here from D2H copies.
static int ilu_create_device(hgb_ctx *c, int n, int nnz, const int *pntr, const int *indx, const void *vals,
                             hgb_dtype vals_dtype, hgb_dtype store, hgb_ilu *M, int *zero_pivot_out,
                             BsPlanPair *plan) {
    HGB_TRY(csr_check(c, n, n, nnz, pntr, indx));
    M->ctx = c;
    M->n = n;
    M->nnz = nnz;
    M->pntr = pntr;
    M->indx = indx;
    M->fdtype = vals_dtype;
    M->store = store;
    int st = HGB_OK;
    int zero_pivot = 0;
    do {
        if (cudaMalloc(&M->diag, sizeof(int) * n) != cudaSuccess) { st = cuda_fail(cudaGetLastError(), "ilu0_create"); break; }
        if ((st = hgb_diag_index(c, n, nnz, pntr, indx, M->diag))) break;
        size_t fs = vsize(vals_dtype);
        if (cudaMalloc(&M->fvals, fs * nnz) != cudaSuccess) { st = cuda_fail(cudaGetLastError(), "ilu0_create"); break; }
        if (cudaMemcpyAsync(M->fvals, vals, fs * nnz, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) { st = cuda_fail(cudaGetLastError(), "ilu0_create"); break; }
        if ((st = alloc_schedule(c, M->L, n))) break;
        int blocks = sync_grid(c, (n + 31) / 32, 8);
        if (vals_dtype == HGB_F64)
            ilu_factor_kernel<double><<<blocks, 256, 0, c->stream>>>(n, pntr, indx, M->diag, (double *)M->fvals, M->L.level, M->L.ticket, c->err);
        else
            ilu_factor_kernel<float><<<blocks, 256, 0, c->stream>>>(n, pntr, indx, M->diag, (float *)M->fvals, M->L.level, M->L.ticket, c->err);
        if ((st = launch_check("ilu_factor_kernel"))) break;
        st = collect_dev_error(c);
        if (st == HGB_ERR_ZERO_PIVOT) { zero_pivot = 1; st = HGB_OK; }
        if (st) break;
        if ((st = build_schedule(c, M->L, 1))) break;
        if ((st = analyse(c, n, pntr, indx, M->diag, 0, M->U))) break;
        // store precision
        if (store == vals_dtype) {
            M->svals = M->fvals;
        } else {
            if (cudaMalloc(&M->svals, vsize(store) * nnz) != cudaSuccess) { st = cuda_fail(cudaGetLastError(), "ilu0_create"); break; }
            if (cudaMalloc(&M->piv, sizeof(double) * n) != cudaSuccess) { st = cuda_fail(cudaGetLastError(), "ilu0_create"); break; }
            int gg = std::max(1, std::min((nnz + 255) / 256, c->num_sms * 8));
            f64_to_store_kernel<<<gg, 256, 0, c->stream>>>(nnz, (const double *)M->fvals,
                                                          store == HGB_F32 ? (float *)M->svals : nullptr,
                                                          store == HGB_BF16 ? (uint16_t *)M->svals : nullptr);
            gather_pivots_kernel<<<std::max(1, std::min((n + 255) / 256, c->num_sms * 8)), 256, 0, c->stream>>>(n, M->diag, (const double *)M->fvals, M->piv);
            if ((st = launch_check("ilu store conversion"))) break;
        }
        if (cudaMalloc(&M->tmp, xsize(store) * n) != cudaSuccess) { st = cuda_fail(cudaGetLastError(), "ilu0_create"); break; }
        {   // block-local schedules; patterns they cannot hold fall back to the global-level solve
            int bs = HGB_OK;
            BsPlanPair *own = nullptr;
            if (!plan) {   // planned here, from host copies of the pattern
                const int R = bsolve_rows(c, (int)xsize(store), n);
                std::vector<int> hp(n + 1), hi(nnz), hd(n);
                if (cudaMemcpyAsync(hp.data(), pntr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
                    cudaMemcpyAsync(hi.data(), indx, sizeof(int) * (size_t)nnz, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
                    cudaMemcpyAsync(hd.data(), M->diag, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
                    cudaStreamSynchronize(c->stream) != cudaSuccess) {
                    st = cuda_fail(cudaGetLastError(), "ilu0_create");
                    break;
                }
                bs = bsolve_plan_pair(c, n, nnz, hp.data(), hi.data(), hd.data(), R, (int)xsize(store), &own);
                plan = own;
            }
            if (!bs) bs = bsolve_upload_pair(plan, M->BL, M->BU);
            bsolve_plan_pair_free(own);
            if (!bs) bs = bsolve_load_values(c, M->BL, M->svals, (int)vsize(store), nullptr);
            if (!bs) bs = bsolve_load_values(c, M->BU, M->svals, (int)vsize(store), M->piv);
            if (bs == HGB_OK) M->use_bs = true;
            else if (bs != HGB_ERR_UNSUPPORTED) { st = bs; break; }
        }
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) { st = cuda_fail(cudaGetLastError(), "ilu0_create"); break; }
    } while (0);
    if (zero_pivot_out) *zero_pivot_out = zero_pivot;
    return st;
}

// complex factors: the level-synchronous factorisation and sweeps of hgb_complex.cu
static int ilu_create_complex(hgb_ctx *c, int n, int nnz, const int *pntr, const int *indx, const void *vals,
                              hgb_dtype dt, hgb_ilu *M, int *zero_pivot) {
    M->ctx = c;
    M->n = n;
    M->nnz = nnz;
    M->pntr = pntr;
    M->indx = indx;
    M->fdtype = M->store = dt;
    return zilu_create(c, n, nnz, pntr, indx, vals, dt == HGB_C128 ? 8 : 4, &M->z, zero_pivot);
}

int hgb_ilu0_create(hgb_ctx *c, int n, int nnz, const int *pntr, const int *indx, const void *vals,
                    hgb_dtype vals_dtype, hgb_dtype store, char policy, hgb_ilu **out) {
    (void)policy;
    if (!out) return fail(HGB_ERR_ARG, "ilu0_create: null output");
    *out = nullptr;
    HGB_TRY(ilu_check_args(c, n, nnz, pntr, indx, vals, vals_dtype, store));
    DeviceGuard g(c->device);
    hgb_ilu *M = new hgb_ilu();
    int zero_pivot = 0;
    const int st = (vals_dtype == HGB_C128 || vals_dtype == HGB_C64)
                       ? ilu_create_complex(c, n, nnz, pntr, indx, vals, vals_dtype, M, &zero_pivot)
                       : ilu_create_device(c, n, nnz, pntr, indx, vals, vals_dtype, store, M, &zero_pivot, nullptr);
    if (st) {
        ilu_free(M);
        return st;
    }
    *out = M;
    if (zero_pivot) return fail(HGB_ERR_ZERO_PIVOT, "ILU(0) met an exactly zero pivot");
    return HGB_OK;
}

// Host-side structure check and diagonal index of a host CSR (the host planning reads the arrays
// directly, so they are validated first): pntr monotone from 0 to nnz, columns in range and strictly
// increasing in each row, every diagonal present.
static int host_csr_diag(int n, int nnz, const int *pntr, const int *indx, std::vector<int> &diag) {
    if (pntr[0] != 0 || pntr[n] != nnz) return fail(HGB_ERR_CSR, "ilu0_create_host: pntr[0] = %d, pntr[n] = %d (nnz %d)", pntr[0], pntr[n], nnz);
    diag.assign(n, -1);
    for (int i = 0; i < n; i++) {
        const int a = pntr[i], e = pntr[i + 1];
        if (e < a || e > nnz) return fail(HGB_ERR_CSR, "ilu0_create_host: row %d has pntr %d..%d", i, a, e);
        int prev = -1;
        for (int q = a; q < e; q++) {
            const int col = indx[q];
            if (col <= prev || col >= n) return fail(HGB_ERR_CSR, "ilu0_create_host: row %d column %d", i, col);
            if (col == i) diag[i] = q;
            prev = col;
        }
        if (diag[i] < 0) return fail(HGB_ERR_CSR, "ilu0_create_host: row %d has no diagonal entry", i);
    }
    return HGB_OK;
}

int hgb_ilu0_create_host(hgb_ctx *c, int n, int nnz, const int *pntr_h, const int *indx_h, const void *vals_h,
                         hgb_dtype vals_dtype, hgb_dtype store, char policy, hgb_ilu **out) {
    (void)policy;
    if (!out) return fail(HGB_ERR_ARG, "ilu0_create_host: null output");
    *out = nullptr;
    HGB_TRY(ilu_check_args(c, n, nnz, pntr_h, indx_h, vals_h, vals_dtype, store));
    DeviceGuard g(c->device);
    std::vector<int> diag;
    HGB_TRY(host_csr_diag(n, nnz, pntr_h, indx_h, diag));
    hgb_ilu *M = new hgb_ilu();
    const size_t vs = vsize(vals_dtype);
    if (cudaMalloc(&M->own_pntr, sizeof(int) * (n + 1)) != cudaSuccess ||
        cudaMalloc(&M->own_indx, sizeof(int) * (size_t)nnz) != cudaSuccess ||
        cudaMalloc(&M->own_vals, vs * (size_t)nnz) != cudaSuccess) {
        const int st = cuda_fail(cudaGetLastError(), "ilu0_create_host");
        ilu_free(M);
        return st;
    }
    // the pattern and the values go to the device on the context's copy stream, from a helper
    // thread (pageable sources make cudaMemcpyAsync wait on the host), while this thread plans the
    // triangular schedules from the host arrays
    int copy_status = HGB_OK;
    std::string copy_msg;
    std::thread copier([&] {
        DeviceGuard gc(c->device);
        copy_status = h2d_chunked(c, c->copy, M->own_pntr, pntr_h, sizeof(int) * (n + 1));
        if (!copy_status) copy_status = h2d_chunked(c, c->copy, M->own_indx, indx_h, sizeof(int) * (size_t)nnz);
        if (!copy_status) copy_status = h2d_chunked(c, c->copy, M->own_vals, vals_h, vs * (size_t)nnz);
        if (!copy_status && cudaStreamSynchronize(c->copy) != cudaSuccess)
            copy_status = cuda_fail(cudaGetLastError(), "ilu0_create_host copy");
        if (copy_status) copy_msg = hgb_last_error();
    });
    const bool cplx = (vals_dtype == HGB_C128 || vals_dtype == HGB_C64);
    BsPlanPair *plan = nullptr;
    const int pst = cplx ? HGB_ERR_UNSUPPORTED
                         : bsolve_plan_pair(c, n, nnz, pntr_h, indx_h, diag.data(),
                                            bsolve_rows(c, (int)xsize(store), n), (int)xsize(store), &plan);
    copier.join();
    int st = copy_status ? fail(copy_status, "%s", copy_msg.c_str()) : HGB_OK;
    int zero_pivot = 0;
    // a pattern the block solve cannot hold leaves plan null: the device path plans (and falls back) itself
    if (!st && pst && pst != HGB_ERR_UNSUPPORTED) st = pst;
    if (!st && cplx) st = ilu_create_complex(c, n, nnz, M->own_pntr, M->own_indx, M->own_vals, vals_dtype, M, &zero_pivot);
    else if (!st) st = ilu_create_device(c, n, nnz, M->own_pntr, M->own_indx, M->own_vals, vals_dtype, store, M,
                                         &zero_pivot, plan);
    bsolve_plan_pair_free(plan);
    if (st) {
        ilu_free(M);
        return st;
    }
    *out = M;
    if (zero_pivot) return fail(HGB_ERR_ZERO_PIVOT, "ILU(0) met an exactly zero pivot");
    return HGB_OK;
}

int hgb_ilu0_apply(hgb_ilu *M, char trans, const void *x, void *r) {
    return hgb::ilu_apply_internal(M, trans, x, r, nullptr);
}

}  // extern "C"

namespace hgb {
int ilu_apply_internal(hgb_ilu *M, char trans, const void *x, void *r, const int *skip) {
    if (!M || !x || !r) return fail(HGB_ERR_ARG, "ilu0_apply: bad arguments");
    DeviceGuard g(M->ctx->device);
    if (M->tmp_epoch != M->ctx->error_epoch) M->tmp_ready = false;   // an earlier launch failed
    bool nt = (trans == 'N' || trans == 'n');
    bool tt = (trans == 'T' || trans == 't' || trans == 'C' || trans == 'c');
    if (!nt && !tt) return fail(HGB_ERR_ARG, "ilu0_apply: trans '%c'", trans);
    if (M->z) {
        HGB_TRY(zilu_apply(M->z, trans, x, r));
        return collect_dev_error(M->ctx);
    }
    switch (M->store) {
        case HGB_F64: return nt ? ilu_apply_n<double, double>(M, x, r, skip) : ilu_apply_t<double, double>(M, x, r, skip);
        case HGB_F32: return nt ? ilu_apply_n<float, float>(M, x, r, skip) : ilu_apply_t<float, float>(M, x, r, skip);
        default: return nt ? ilu_apply_n<uint16_t, float>(M, x, r, skip) : ilu_apply_t<uint16_t, float>(M, x, r, skip);
    }
}
}  // namespace hgb

extern "C" {

int hgb_ilu0_export(hgb_ilu *M, void *factor_vals, int *diag) {
    if (!M) return fail(HGB_ERR_ARG, "ilu0_export: null handle");
    hgb_ctx *c = M->ctx;
    DeviceGuard g(c->device);
    if (M->z) {
        HGB_TRY(zilu_export(M->z, factor_vals, diag));
    } else {
        if (factor_vals) HGB_CUDA(cudaMemcpyAsync(factor_vals, M->fvals, vsize(M->fdtype) * M->nnz, cudaMemcpyDeviceToDevice, c->stream));
        if (diag) HGB_CUDA(cudaMemcpyAsync(diag, M->diag, sizeof(int) * M->n, cudaMemcpyDeviceToDevice, c->stream));
    }
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    return HGB_OK;
}

int hgb_ilu0_levels(hgb_ilu *M, char uplo, int *level, int *nlevels) {
    if (!M) return fail(HGB_ERR_ARG, "ilu0_levels: null handle");
    if (M->z) return fail(HGB_ERR_UNSUPPORTED, "ilu0_levels: real factors");
    hgb_ctx *c = M->ctx;
    DeviceGuard g(c->device);
    const Schedule &S = (uplo == 'L' || uplo == 'l') ? M->L : M->U;
    if (level) HGB_CUDA(cudaMemcpyAsync(level, S.level, sizeof(int) * M->n, cudaMemcpyDeviceToDevice, c->stream));
    if (nlevels) *nlevels = S.nlevels;
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    return HGB_OK;
}

int hgb_ilu0_destroy(hgb_ilu *M) {
    if (!M) return HGB_OK;
    DeviceGuard g(M->ctx->device);
    ilu_free(M);
    return HGB_OK;
}

// ----------------------------------------------------------------- triangular ----------
int hgb_tri_create(hgb_ctx *c, char uplo, char diagc, int n, int nnz, const int *pntr, const int *indx,
                   const void *vals, hgb_dtype dtype, hgb_tri **out) {
    if (!out) return fail(HGB_ERR_ARG, "tri_create: null output");
    *out = nullptr;
    if (!c || n <= 0 || nnz < 0 || !pntr || !indx || !vals) return fail(HGB_ERR_ARG, "tri_create: bad arguments");
    bool lower = (uplo == 'L' || uplo == 'l');
    if (!lower && uplo != 'U' && uplo != 'u') return fail(HGB_ERR_ARG, "tri_create: uplo '%c'", uplo);
    if (diagc != 'U' && diagc != 'u' && diagc != 'N' && diagc != 'n') return fail(HGB_ERR_ARG, "tri_create: diag '%c'", diagc);
    if (dtype != HGB_F64 && dtype != HGB_F32 && dtype != HGB_C128 && dtype != HGB_C64)
        return fail(HGB_ERR_UNSUPPORTED, "tri_create: F64, F32, C128 or C64 values");
    DeviceGuard g(c->device);
    HGB_TRY(csr_check(c, n, n, nnz, pntr, indx));
    if (dtype == HGB_C128 || dtype == HGB_C64) {
        hgb_ztri *z = nullptr;
        HGB_TRY(ztri_create(c, lower ? 'L' : 'U', diagc, n, nnz, pntr, indx, vals, dtype == HGB_C128 ? 8 : 4, &z));
        hgb_tri *T = new hgb_tri();
        T->ctx = c;
        T->n = n;
        T->nnz = nnz;
        T->dtype = dtype;
        T->z = z;
        *out = T;
        return HGB_OK;
    }
    hgb_tri *T = new hgb_tri();
    T->ctx = c;
    T->n = n;
    T->nnz = nnz;
    T->uplo = lower ? 'L' : 'U';
    T->diagc = (diagc == 'U' || diagc == 'u') ? 'U' : 'N';
    T->pntr = pntr;
    T->indx = indx;
    T->vals = vals;
    T->dtype = dtype;
    int st = HGB_OK;
    do {
        if (cudaMalloc(&T->diag, sizeof(int) * n) != cudaSuccess) { st = cuda_fail(cudaGetLastError(), "tri_create"); break; }
        if ((st = hgb_diag_index(c, n, nnz, pntr, indx, T->diag))) break;
        if ((st = analyse(c, n, pntr, indx, T->diag, lower ? 1 : 0, T->S))) break;
    } while (0);
    if (st) {
        cudaFree(T->diag);
        T->S.release();
        delete T;
        return st;
    }
    *out = T;
    return HGB_OK;
}

}  // extern "C"

namespace hgb {
template <typename V>
static int tri_solve_t(hgb_tri *T, char trans, double alpha, const void *b, void *x) {
    using X = V;
    hgb_ctx *c = T->ctx;
    bool nt = (trans == 'N' || trans == 'n');
    const X *bin = (const X *)b;
    if (b == x) {
        if (!T->bcopy) HGB_CUDA(cudaMalloc(&T->bcopy, sizeof(X) * T->n));
        HGB_CUDA(cudaMemcpyAsync(T->bcopy, b, sizeof(X) * T->n, cudaMemcpyDeviceToDevice, c->stream));
        bin = (const X *)T->bcopy;
    }
    HGB_TRY(fill_pending<X>(c, T->n, (X *)x));
    SolveArgs A{};
    A.piv = nullptr;
    A.mode = MODE_TRSV;
    A.unit = (T->diagc == 'U') ? 1 : 0;
    bool lower = (T->uplo == 'L');
    if (nt) {
        A.pntr = T->pntr;
        A.indx = T->indx;
        A.diag = T->diag;
        A.map = nullptr;
        A.lower = lower ? 1 : 0;
        A.rev = 0;
        return launch_solve<V, X>(c, T->S, A, (const V *)T->vals, (X)alpha, bin, (X *)x, nullptr, nullptr);
    }
    if (!T->has_T) {
        HGB_TRY(build_transpose(c, T->n, T->n, T->nnz, T->pntr, T->indx, T->T));
        HGB_CUDA(cudaMalloc(&T->diagT, sizeof(int) * T->n));
        HGB_TRY(hgb_diag_index(c, T->n, T->nnz, T->T.pntr, T->T.row, T->diagT));
        // op(L)=L^T is upper (rows descending); op(U)=U^T is lower (rows ascending)
        HGB_TRY(analyse(c, T->n, T->T.pntr, T->T.row, T->diagT, lower ? 0 : 1, T->ST));
        T->has_T = true;
    }
    A.pntr = T->T.pntr;
    A.indx = T->T.row;
    A.diag = T->diagT;
    A.map = T->T.map;
    A.lower = lower ? 0 : 1;
    A.rev = lower ? 1 : 0;     // contributions arrive in descending row order for L^T
    return launch_solve<V, X>(c, T->ST, A, (const V *)T->vals, (X)alpha, bin, (X *)x, nullptr, nullptr);
}
}  // namespace hgb

extern "C" {

int hgb_tri_solve(hgb_tri *T, char trans, double alpha, const void *b, void *x) {
    if (!T || !b || !x) return fail(HGB_ERR_ARG, "tri_solve: bad arguments");
    if (trans != 'N' && trans != 'n' && trans != 'T' && trans != 't' && trans != 'C' && trans != 'c')
        return fail(HGB_ERR_ARG, "tri_solve: trans '%c'", trans);
    DeviceGuard g(T->ctx->device);
    if (T->z) {
        const double a2[2] = {alpha, 0.0};
        const float a1[2] = {(float)alpha, 0.0f};
        HGB_TRY(ztri_solve(T->z, trans, T->dtype == HGB_C128 ? (const void *)a2 : (const void *)a1, b, x));
        return collect_dev_error(T->ctx);
    }
    int st = (T->dtype == HGB_F64) ? tri_solve_t<double>(T, trans, alpha, b, x) : tri_solve_t<float>(T, trans, alpha, b, x);
    if (st) return st;
    return collect_dev_error(T->ctx);
}

int hgb_tri_destroy(hgb_tri *T) {
    if (!T) return HGB_OK;
    DeviceGuard g(T->ctx->device);
    ztri_destroy(T->z);
    cudaFree(T->diag);
    cudaFree(T->bcopy);
    T->S.release();
    if (T->has_T) {
        T->T.release();
        cudaFree(T->diagT);
        T->ST.release();
    }
    delete T;
    return HGB_OK;
}

}  // extern "C"

// internal accessors for the fused solvers
namespace hgb {
hgb_dtype ilu_store(const hgb_ilu *M) { return M->store; }
int ilu_n(const hgb_ilu *M) { return M->n; }
size_t ilu_xbytes(const hgb_ilu *M) { return M->store == HGB_BF16 ? 4 : vsize(M->store); }
hgb_zilu *ilu_zfactor(const hgb_ilu *M) { return M->z; }
}  // namespace hgb
