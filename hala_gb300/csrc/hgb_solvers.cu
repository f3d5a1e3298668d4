// Fused Krylov solvers over the SpMV / ILU kernels.
//
// CG / PCG follow solve_cg_core (hex/solvers/hala_solvers_cg.hpp:92-156) step for step, but the
// scalars never leave the device: <p,Ap> is reduced in the SpMV epilogue, ||r||^2 in the x/r
// update, and the convergence decision is taken on the device.  One iteration is six launches
// (SpMV+dot, update+norm, L solve, U solve, <r,z>, p update); ITERS_PER_GRAPH iterations are
// captured once into a CUDA graph and replayed, every launch of an iteration after convergence
// being a no-op, so the host synchronises once per graph replay instead of three times per
// iteration as the reference does (cublasDdot / cublasDnrm2 in host pointer mode).
#include "hgb_internal.cuh"
#include "hgb_kernels.cuh"
#include "hgb_complex.cuh"

#include <algorithm>
#include <cstddef>
#include <cmath>
#include <vector>

namespace hgb {

constexpr int kItersPerGraph = 16;

// Elements a thread takes per round in the CG vector kernels, their loads issued together: the
// kernels are short and latency-bound (about 14 elements per thread at 128^3), so one element per
// round left a thread waiting on one memory round trip per element.
template <typename X, int NARR = 2> __host__ __device__ constexpr int ew_unroll() {
    return (sizeof(X) == 8 ? 4 : 8) / (NARR > 2 ? 2 : 1);   // NARR: vectors read per element
}
// their grids are num_sms x 4 CTAs of 256 threads: the register budget keeps all four resident
// (unbounded, the batched loads took up to 86 registers and the grid ran in two waves)
constexpr int kEwThreads = 256, kEwCtasPerSm = 4;

// <p, Ap>: the SpMV's per-CTA parts summed in one order in every CTA (pap_n > 0), or the value
// its grid reduction stored (pap_n == 0: the transposed product)
__device__ __forceinline__ double parts_sum(const double *part, int np, double stored) {
    if (np == 0) return stored;
    __shared__ double res;
    double v[1] = {0.0};
    for (int b = threadIdx.x; b < np; b += blockDim.x) v[0] += part[b];
    block_sum<1>(v);
    if (threadIdx.x == 0) res = v[0];
    __syncthreads();
    return res;
}

template <typename X>
__global__ void __launch_bounds__(kEwThreads, kEwCtasPerSm) cg_update_kernel(long n, const SolverScalars *__restrict__ s_in, SolverScalars *s,
                                 const X *__restrict__ p, const X *__restrict__ Ap, X *__restrict__ x,
                                 X *__restrict__ r, double *partials, unsigned *counter, const double *pap_part,
                                 int pap_n) {
    if (s_in->done) return;
    const double pap = parts_sum(pap_part, pap_n, s_in->pap);
    // a = <r,z> / <p,Ap>; x += a p; r -= a Ap  (axpy(a,p,x), axpy(-a,Ap,r))
    const X a = (X)(s_in->zr / pap);
    const X ma = -a;
    DotAcc<X> rr;
    constexpr int U = ew_unroll<X, 4>();
    const long T = (long)gridDim.x * blockDim.x;
    for (long base = blockIdx.x * (long)blockDim.x + threadIdx.x; base < n; base += T * U) {
        X pv[U], av[U], xv[U], rv[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long i = base + u * T;
            if (i < n) {
                pv[u] = p[i];
                av[u] = Ap[i];
                xv[u] = x[i];
                rv[u] = r[i];
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long i = base + u * T;
            if (i < n) {
                x[i] = add_rn(xv[u], mul_rn(a, pv[u]));
                const X ri = add_rn(rv[u], mul_rn(ma, av[u]));
                r[i] = ri;
                rr.add(ri, ri);
            }
        }
    }
    double acc[1] = {rr.get()};
    grid_sum<1>(acc, partials, counter, [&](double (&v)[1]) {
        s->pap = pap;
        s->rr = v[0];
        s->it += 1;
        s->done = (s->it >= s->max_iter) || (v[0] < s->tol2) || !(v[0] == v[0]);
    });
}

template <typename X>
__global__ void __launch_bounds__(kEwThreads, kEwCtasPerSm) cg_rz_kernel(long n, SolverScalars *s, const X *__restrict__ r, const X *__restrict__ z,
                             double *partials, unsigned *counter, int init) {
    if (!init && s->done) return;
    DotAcc<X> rz, rr;
    constexpr int U = ew_unroll<X>();
    const long T = (long)gridDim.x * blockDim.x;
    for (long base = blockIdx.x * (long)blockDim.x + threadIdx.x; base < n; base += T * U) {
        X rv[U], zv[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long i = base + u * T;
            if (i < n) {
                rv[u] = r[i];
                zv[u] = z[i];
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            if (base + u * T < n) {
                rz.add(rv[u], zv[u]);
                if (init) rr.add(rv[u], rv[u]);
            }
        }
    }
    double acc[2] = {rz.get(), rr.get()};
    grid_sum<2>(acc, partials, counter, [&](double (&v)[2]) {
        s->nzr = s->zr;      // previous <r,z>, used by the p update
        s->zr = v[0];
        if (init) {
            s->rr = v[1];
            s->r0 = sqrt(v[1]);
            if (s->rel > 0.0) {
                double t = s->rel * s->r0;
                s->tol2 = fmax(s->tol2, t * t);
            }
        }
    });
}

// p = (zr_new / zr_old) p + z   (scal(a, p); axpy(1, z, p))
template <typename X>
__global__ void __launch_bounds__(kEwThreads, kEwCtasPerSm) cg_p_kernel(long n, const SolverScalars *__restrict__ s, X *__restrict__ p, const X *__restrict__ z) {
    if (s->done) return;
    const X bta = (X)(s->zr / s->nzr);
    constexpr int U = ew_unroll<X>();
    const long T = (long)gridDim.x * blockDim.x;
    for (long base = blockIdx.x * (long)blockDim.x + threadIdx.x; base < n; base += T * U) {
        X pv[U], zv[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long i = base + u * T;
            if (i < n) {
                pv[u] = p[i];
                zv[u] = z[i];
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long i = base + u * T;
            if (i < n) p[i] = add_rn(mul_rn(bta, pv[u]), zv[u]);
        }
    }
}

__global__ void cg_init_kernel(SolverScalars *s, double tol2, double rel, int max_iter) {
    s->it = 1;
    s->done = 0;
    s->max_iter = max_iter;
    s->tol2 = tol2;
    s->rel = rel;
    s->zr = 0.0;
    s->nzr = 0.0;
    s->pap = 0.0;
    s->rr = 0.0;
}

template <typename X>
__global__ void copy_kernel(long n, const X *__restrict__ a, X *__restrict__ b) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) b[i] = a[i];
}

__global__ void f64_to_f32_kernel(long n, const double *__restrict__ a, float *__restrict__ b) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) b[i] = (float)a[i];
}

__global__ void add_f32_to_f64_kernel(long n, const float *__restrict__ d, double *__restrict__ x) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) x[i] += (double)d[i];
}

__global__ void zero_f32_kernel(long n, float *d) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) d[i] = 0.0f;
}

// r = b - A x in FP64 and ||r||^2 -> result slot (the refinement residual)
__global__ void residual_norm_kernel(long n, const double *__restrict__ r, double *partials, unsigned *counter,
                                     double *out) {
    double acc[1] = {0.0};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        acc[0] += r[i] * r[i];
    grid_sum<1>(acc, partials, counter, [&](double (&v)[1]) { *out = v[0]; });
}

static inline int ew_grid(hgb_ctx *c, long n) {
    return std::max(1, (int)std::min<long>((n + 255) / 256, (long)c->num_sms * 4));
}

// Workspace of one fused CG run (X = vector type).
template <typename X>
struct CgWork {
    X *r = nullptr, *z = nullptr, *p = nullptr, *Ap = nullptr;
    hgb_ctx *c = nullptr;
    int alloc(hgb_ctx *ctx, long n, bool need_z) {
        c = ctx;
        if (ws_alloc(c, &r, n) || ws_alloc(c, &p, n) || ws_alloc(c, &Ap, n) || (need_z && ws_alloc(c, &z, n)))
            return cuda_fail(cudaErrorMemoryAllocation, "cg workspace");
        return HGB_OK;
    }
    void release() {
        if (!c) return;
        ws_free(c, r);
        ws_free(c, z);
        ws_free(c, p);
        ws_free(c, Ap);
    }
};

// y = alpha op(A) x + beta y with an optional fused <x, y>: into *dot, or (nparts, 'N' only) as
// per-CTA parts left for the consuming kernel (*nparts: their count; 0 when *dot was written)
template <typename V, typename X>
static int spmv_A(hgb_ctx *c, hgb_csr *A, X alpha, const X *x, X beta, X *y, double *dot, const int *skip,
                  bool trans = false, int *nparts = nullptr) {
    if (trans) {
        if (nparts) *nparts = 0;
        return spmv_t_fused_launch<V>(A, alpha, x, beta, y, x, dot, skip);
    }
    return spmv_n_launch<V>(c, csr_rows(A), csr_pntr(A), csr_indx(A), (const V *)csr_vals(A), alpha, x, beta, y,
                            nparts ? nullptr : dot, skip, nparts);
}
template <>
int spmv_A<uint16_t, float>(hgb_ctx *c, hgb_csr *A, float alpha, const float *x, float beta, float *y, double *dot,
                           const int *skip, bool trans, int *nparts) {
    if (trans) return fail(HGB_ERR_UNSUPPORTED, "transposed product of a bf16 matrix");
    return spmv_n_launch<uint16_t>(c, csr_rows(A), csr_pntr(A), csr_indx(A), (const uint16_t *)csr_vals(A), alpha, x,
                                   beta, y, nparts ? nullptr : dot, skip, nparts);
}

// One CG iteration: the launches captured into the graph.
template <typename V, typename X>
static int cg_iteration(hgb_ctx *c, hgb_csr *A, hgb_ilu *M, CgWork<X> &w, X *x, long n, bool trans) {
    SolverScalars *s = c->scal;
    const int *done = &s->done;
    int np = 0;
    HGB_TRY(spmv_A<V, X>(c, A, X(1), w.p, X(0), w.Ap, &s->pap, done, trans, &np));
    cg_update_kernel<X><<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, s, s, w.p, w.Ap, x, w.r, c->partials,
                                                                           c->counter, c->partials + kSpmvPartsOffset, np);
    X *z = M ? w.z : w.r;
    if (M) HGB_TRY(ilu_apply_internal(M, trans ? 'T' : 'N', w.r, w.z, done));
    cg_rz_kernel<X><<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, s, w.r, z, c->partials, c->counter, 0);
    cg_p_kernel<X><<<ew_grid(c, n), 256, 0, c->stream>>>(n, s, w.p, z);
    return launch_check("cg iteration");
}

// ------------------------------------------------------------------ persistent CG -------
// Unpreconditioned CG on a system whose matrix and vectors stay in L2 (the 256^2 Poisson class):
// there the graph-replayed iteration is bound by its launches and their reductions' tails
// (about 27 us per iteration for six launches), not by bytes.  One cooperative launch runs up to
// kCgpChunk iterations with two grid barriers each: after the x / r update (||r||^2 complete, and
// r in memory for the next product) and after the direction update (<p, Ap> complete).  The
// product is taken of r, s = A r, and the new direction's product follows by the recurrence
// Ap = beta Ap + s beside p = beta p + r, so no barrier waits for the new p (a launch starts
// with Ap = A p).  Every CTA keeps its rows for the whole launch, writes one partial per reduction
// and, after the barrier, sums all CTAs' partials in the same order, so every CTA takes the same
// decision with the same bits and no CTA waits on a single finisher.  The updates are the graph
// path's (DotAcc partials per thread, separately rounded, the product in the context's SpMV
// mode), with z = r, so <r, z> is ||r||^2; the Ap recurrence rounds differently from A p, so the
// iteration count can differ from the graph path's by a few.  Barriers are bounded: a barrier
// that runs out of polls sets DEV_ERR_TIMEOUT and every CTA returns.
constexpr int kCgpThreads = 256;
constexpr int kCgpChunk = 4096;                 // iterations per launch (the barrier counter stays small)
constexpr long kCgpMaxRows = 1L << 20;          // larger systems take the graph path
constexpr size_t kCgpMaxBytes = 48u << 20;      // matrix + vectors resident in L2 (129 MB)

// acc += v * x: separately rounded (the exact SpMV mode) or one fused multiply-add
template <bool EXACT, typename X>
__device__ __forceinline__ X cgp_acc(X acc, X v, X x) {
    return EXACT ? add_rn(acc, mul_rn(v, x)) : fma(v, x, acc);
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// One reduction of the persistent CG: the CTA's partial of v (warp sums, then warp 0), the
// arrival of every CTA (a grid barrier, bounded), then the sum of all G partials in one fixed
// order (lane b takes partials b, b + 32, ..., then the warp's butterfly), the same bits in every
// CTA.  Two CTA barriers: the first orders every thread's earlier global writes before warp 0's
// release, the second publishes the sum.  False when the wait ran out (DEV_ERR_TIMEOUT set).
__device__ __forceinline__ bool cgp_reduce(double v, double *part, unsigned *count, unsigned target, int *err,
                                           double &sum) {
    __shared__ double wsh[32], res;
    __shared__ int ok;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum(v);
    if (lane == 0) wsh[wid] = v;
    __syncthreads();
    if (wid == 0) {
        const double t = warp_sum(lane < (int)(blockDim.x >> 5) ? wsh[lane] : 0.0);
        if (lane == 0) {
            part[blockIdx.x] = t;
            // release at GPU scope, cumulative over the CTA's writes that the bar.sync ordered before it
            asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(count) : "memory");
        }
        // every lane polls (one coalesced load), so each lane's own acquire orders its loads below
        int spins = 0, good = 1;
        while (!__all_sync(0xFFFFFFFFu, ld_acquire_u32(count) >= target)) {
            if (++spins > kSpinLimit || ((spins & 1023) == 0 && (*(volatile int *)err & DEV_ERR_TIMEOUT))) {
                good = 0;
                break;
            }
        }
        good = __all_sync(0xFFFFFFFFu, good);
        double acc = 0.0;
        if (good)
            for (int b = lane; b < (int)gridDim.x; b += 32) acc += __ldcg(part + b);
        acc = warp_sum(acc);
        if (lane == 0) {
            if (!good) atomicOr(err, DEV_ERR_TIMEOUT);
            res = acc;
            ok = good;
        }
    }
    __syncthreads();
    sum = res;
    return ok != 0;
}

// RPT > 0: thread t owns rows t, t + stride, ... (RPT of them: 1, 2 or 4) for the whole launch and keeps their
// x, r, p and (rows of at most kCgpMaxE entries) their matrix entries in registers: an iteration
// then reads only the neighbours' p from L2.  RPT = 0: the rows are walked with grid-stride loops
// and every vector lives in memory (systems too large for one register-resident row set).
constexpr int kCgpMaxE = 8;

template <typename V, typename X, bool EXACT, int RPT>
__global__ void __launch_bounds__(kCgpThreads)
cg_persistent_kernel(long n, const int *__restrict__ pntr, const int *__restrict__ indx, const V *__restrict__ vals,
                     X *x, X *r, X *p, X *Ap, SolverScalars *s, double *part, unsigned *count, int *err) {
    const int G = gridDim.x;
    if (s->done) return;
    double zr = s->zr, rrv = s->rr;
    int it = s->it;
    const int max_iter = s->max_iter;
    const double tol2 = s->tol2;
    double *partA = part, *partB = part + G;
    const long t0 = (long)blockIdx.x * blockDim.x + threadIdx.x, stride = (long)G * blockDim.x;
    unsigned target = 0;
    bool done = false;
    constexpr int K = RPT > 0 ? RPT : 1;
    long row[K];
    int beg[K], len[K], ci[K][kCgpMaxE];
    X cv[K][kCgpMaxE], xr[K], rr[K], pr[K];
    if (RPT > 0) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            row[k] = t0 + k * stride;
            len[k] = 0;
            beg[k] = 0;
            if (row[k] < n) {
                beg[k] = pntr[row[k]];
                len[k] = pntr[row[k] + 1] - beg[k];
                xr[k] = x[row[k]];
                rr[k] = r[row[k]];
                pr[k] = p[row[k]];
#pragma unroll
                for (int e = 0; e < kCgpMaxE; e++)
                    if (e < len[k]) {
                        ci[k][e] = indx[beg[k] + e];
                        cv[k][e] = Val<V>::get(vals[beg[k] + e]);
                    }
            }
        }
    }
    // row k of this thread (RPT > 0) or row i (RPT = 0) times the vector v, whose entries other
    // CTAs wrote during this launch (__ldcg: from L2)
    auto row_product = [&](int k, long i, const X *v) -> X {
        X acc = X(0);
        if (RPT > 0 && len[k] <= kCgpMaxE) {
            X xv[kCgpMaxE];
#pragma unroll
            for (int e = 0; e < kCgpMaxE; e++)
                if (e < len[k]) xv[e] = __ldcg(v + ci[k][e]);
#pragma unroll
            for (int e = 0; e < kCgpMaxE; e++)
                if (e < len[k]) acc = cgp_acc<EXACT, X>(acc, cv[k][e], xv[e]);
        } else {
            const int jb = RPT > 0 ? beg[k] : pntr[i], je = RPT > 0 ? beg[k] + len[k] : pntr[i + 1];
            for (int j = jb; j < je; j++) acc = cgp_acc<EXACT, X>(acc, Val<V>::get(vals[j]), __ldcg(v + indx[j]));
        }
        return acc;
    };
    // q = A p for the direction the launch starts from, and <p, q>
    X qr[K];
    double pAp;
    {
        DotAcc<X> pq;
        if (RPT > 0) {
#pragma unroll
            for (int k = 0; k < K; k++)
                if (row[k] < n) {
                    qr[k] = row_product(k, row[k], p);
                    pq.add(pr[k], qr[k]);
                }
        } else {
            for (long i = t0; i < n; i += stride) {
                const X q = row_product(0, i, p);
                Ap[i] = q;
                pq.add(p[i], q);
            }
        }
        target += G;
        if (!cgp_reduce(pq.get(), partA, count, target, err, pAp)) return;
    }
    for (int c = 0; c < kCgpChunk; c++) {
        // a = <r,z> / <p,Ap>; x += a p; r -= a Ap; ||r||^2 (r to memory: the next product reads it)
        const X a = (X)(zr / pAp), ma = -a;
        DotAcc<X> rrd;
        if (RPT > 0) {
#pragma unroll
            for (int k = 0; k < K; k++) {
                if (row[k] >= n) continue;
                xr[k] = add_rn(xr[k], mul_rn(a, pr[k]));
                rr[k] = add_rn(rr[k], mul_rn(ma, qr[k]));
                r[row[k]] = rr[k];
                rrd.add(rr[k], rr[k]);
            }
        } else {
            for (long i = t0; i < n; i += stride) {
                x[i] = add_rn(x[i], mul_rn(a, p[i]));
                const X ri = add_rn(r[i], mul_rn(ma, Ap[i]));
                r[i] = ri;
                rrd.add(ri, ri);
            }
        }
        target += G;
        if (!cgp_reduce(rrd.get(), partB, count, target, err, rrv)) return;
        it++;
        done = (it >= max_iter) || (rrv < tol2) || !(rrv == rrv);
        if (done) break;
        // z = r: <r, z> = ||r||^2; p = (zr_new / zr_old) p + z and, with s = A r, the product of the
        // new direction by the same recurrence: Ap = (zr_new / zr_old) Ap + s.  So the product reads
        // r, complete at the barrier above, and no barrier waits for the new p.
        const X bta = (X)(rrv / zr);
        DotAcc<X> pq;
        if (RPT > 0) {
#pragma unroll
            for (int k = 0; k < K; k++) {
                if (row[k] >= n) continue;
                const X sk = row_product(k, row[k], r);
                pr[k] = add_rn(mul_rn(bta, pr[k]), rr[k]);
                qr[k] = add_rn(mul_rn(bta, qr[k]), sk);
                pq.add(pr[k], qr[k]);
            }
        } else {
            for (long i = t0; i < n; i += stride) {
                const X si = row_product(0, i, r);
                const X pi = add_rn(mul_rn(bta, p[i]), r[i]);
                const X qi = add_rn(mul_rn(bta, Ap[i]), si);
                p[i] = pi;
                Ap[i] = qi;
                pq.add(pi, qi);
            }
        }
        zr = rrv;
        target += G;
        if (!cgp_reduce(pq.get(), partA, count, target, err, pAp)) return;
    }
    if (RPT > 0) {
#pragma unroll
        for (int k = 0; k < K; k++)
            if (row[k] < n) {
                x[row[k]] = xr[k];
                r[row[k]] = rr[k];
                p[row[k]] = pr[k];
            }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        s->it = it;
        s->rr = rrv;
        s->nzr = s->zr;
        s->zr = zr;
        s->done = done ? 1 : 0;
    }
}

// Launch shape of the persistent CG: {grid, rows per thread (0: grid-stride)}; grid 0 when no
// co-resident grid exists.  Every CTA costs each barrier one more arrival on the counter and each
// reduction one more part, every row of a thread one more serial stretch of its phase: one row per
// thread up to one CTA per SM, two up to two CTAs per SM, four up to two, else grid-stride loops.
// (256^2 Poisson: 11.1 us per iteration with two rows per thread on 128 CTAs, 13.2 with four on 64.)
struct CgpShape {
    int grid = 0, rpt = 0;
};
template <typename V, typename X, bool EXACT>
static CgpShape cgp_shape(hgb_ctx *c, long n) {
    CgpShape sh;
    int nb[4] = {0, 0, 0, 0};
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb[0], cg_persistent_kernel<V, X, EXACT, 0>, kCgpThreads, 0) ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb[1], cg_persistent_kernel<V, X, EXACT, 1>, kCgpThreads, 0) ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb[2], cg_persistent_kernel<V, X, EXACT, 2>, kCgpThreads, 0) ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb[3], cg_persistent_kernel<V, X, EXACT, 4>, kCgpThreads, 0)) {
        cudaGetLastError();
        return sh;
    }
    const long g1 = (n + kCgpThreads - 1) / kCgpThreads;
    const long g2 = (n + 2L * kCgpThreads - 1) / (2L * kCgpThreads), g4 = (n + 4L * kCgpThreads - 1) / (4L * kCgpThreads);
    if (g1 <= std::min<long>((long)nb[1] * c->num_sms, (long)c->num_sms)) return CgpShape{(int)g1, 1};
    if (g2 <= std::min<long>((long)nb[2] * c->num_sms, 2L * c->num_sms)) return CgpShape{(int)g2, 2};
    if (g4 <= std::min<long>((long)nb[3] * c->num_sms, 2L * c->num_sms)) return CgpShape{(int)g4, 4};
    // about four rows per thread: fewer CTAs make cheaper barriers, the data are in L2 anyway
    const long want = std::max<long>(1, (n + 4L * kCgpThreads - 1) / (4L * kCgpThreads));
    sh.grid = (int)std::min<long>(want, (long)nb[0] * c->num_sms);
    sh.rpt = 0;
    return sh;
}

template <typename V, typename X>
static bool cgp_eligible(hgb_csr *A, hgb_ilu *M, bool trans) {
    const long n = csr_rows(A);
    const size_t bytes = (size_t)csr_nnz(A) * (sizeof(V) + 4) + (size_t)(n + 1) * 4 + (size_t)n * sizeof(X) * 5;
    return !M && !trans && n > 0 && n <= kCgpMaxRows && bytes <= kCgpMaxBytes;
}

template <typename V, typename X, bool EXACT>
static const void *cgp_kernel(int rpt) {
    return rpt == 1   ? (const void *)cg_persistent_kernel<V, X, EXACT, 1>
           : rpt == 2 ? (const void *)cg_persistent_kernel<V, X, EXACT, 2>
           : rpt == 4 ? (const void *)cg_persistent_kernel<V, X, EXACT, 4>
                      : (const void *)cg_persistent_kernel<V, X, EXACT, 0>;
}

// Runs the loop of an initialised CgWork (r, p, the scalars' zr / it / tol2) to the end.
template <typename V, typename X>
static int cgp_run(hgb_ctx *c, hgb_csr *A, CgWork<X> &w, X *x, long n, long long *launches, SolverScalars &hs) {
    const bool exact = (c->spmv_mode == HGB_SPMV_EXACT);
    const CgpShape sh = exact ? cgp_shape<V, X, true>(c, n) : cgp_shape<V, X, false>(c, n);
    const int G = sh.grid;
    if (G < 1) return fail(HGB_ERR_UNSUPPORTED, "persistent cg: no co-resident grid");
    double *part = nullptr;
    unsigned *count = nullptr;
    int st = HGB_OK;
    if (ws_alloc(c, &part, 2 * (size_t)G) || ws_alloc(c, &count, 1)) st = cuda_fail(cudaErrorMemoryAllocation, "persistent cg");
    const int *pntr = csr_pntr(A), *indx = csr_indx(A);
    const V *vals = (const V *)csr_vals(A);
    SolverScalars *s = c->scal;
    int *err = c->err;
    X *r = w.r, *p = w.p, *Ap = w.Ap;
    void *args[] = {&n, &pntr, &indx, &vals, &x, &r, &p, &Ap, &s, &part, &count, &err};
    while (!st) {
        if (cudaMemsetAsync(count, 0, sizeof(unsigned), c->stream) != cudaSuccess) {
            st = cuda_fail(cudaGetLastError(), "persistent cg");
            break;
        }
        const void *fn = exact ? cgp_kernel<V, X, true>(sh.rpt) : cgp_kernel<V, X, false>(sh.rpt);
        if (cudaLaunchCooperativeKernel(fn, dim3(G), dim3(kCgpThreads), args, 0, c->stream) != cudaSuccess) {
            st = cuda_fail(cudaGetLastError(), "persistent cg launch");
            break;
        }
        *launches += 1;
        if (cudaMemcpyAsync(c->host_result, s, sizeof(SolverScalars), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
            cudaStreamSynchronize(c->stream) != cudaSuccess) {
            st = cuda_fail(cudaGetLastError(), "persistent cg sync");
            break;
        }
        memcpy(&hs, c->host_result, sizeof(SolverScalars));
        if ((st = collect_dev_error(c))) break;
        if (hs.done) break;
    }
    ws_free(c, part);
    ws_free(c, count);
    return st;
}

// Runs CG on (A, M) for b -> x (x holds the initial guess).  zero_x0: skip r = b - A x.
// kernels per captured CG iteration: SpMV+dot, update+norm, [L solve, U solve], <r,z>, p update
static int cg_launches_per_iter(bool precond) { return precond ? 6 : 4; }

template <typename V, typename X>
static int cg_run(hgb_ctx *c, hgb_csr *A, hgb_ilu *M, const X *b, X *x, double tol2, double rel, int max_iter,
                  bool zero_x0, int *iters, double *rr_out, long long *launches, bool trans = false) {
    const long n = csr_rows(A);
    CaptureStream cs(c);
    CgWork<X> w;
    int st = w.alloc(c, n, M != nullptr);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    SolverScalars hs{};
    do {
        if (st) break;
        SolverScalars *s = c->scal;
        cg_init_kernel<<<1, 1, 0, c->stream>>>(s, tol2, rel, max_iter);
        *launches += 1 + (zero_x0 ? 0 : 1) + (M ? 2 : 0) + 2;   // init, SpMV, L/U solves, copy, <r,z>
        // r = b - A x  (r = b; r += -1 * A x)
        if (cudaMemcpyAsync(w.r, b, sizeof(X) * n, cudaMemcpyDeviceToDevice, c->stream)) { st = cuda_fail(cudaGetLastError(), "cg"); break; }
        if (trans && (st = csr_ensure_transpose(A))) break;
        if (!zero_x0 && (st = spmv_A<V, X>(c, A, X(-1), x, X(1), w.r, nullptr, nullptr, trans))) break;
        X *z = M ? w.z : w.r;
        if (M && (st = ilu_apply_internal(M, trans ? 'T' : 'N', w.r, w.z, nullptr))) break;
        copy_kernel<X><<<ew_grid(c, n), 256, 0, c->stream>>>(n, z, w.p);
        cg_rz_kernel<X><<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, s, w.r, z, c->partials, c->counter, 1);
        if ((st = launch_check("cg init"))) break;
        if (cgp_eligible<V, X>(A, M, trans)) {   // small, L2-resident, unpreconditioned: one persistent launch
            st = cgp_run<V, X>(c, A, w, x, n, launches, hs);
            break;
        }
        // capture ITERS_PER_GRAPH iterations
        cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
        if (cudaStreamBeginCapture(c->stream, mode)) { st = cuda_fail(cudaGetLastError(), "begin capture"); break; }
        for (int k = 0; k < kItersPerGraph && !st; k++) st = cg_iteration<V, X>(c, A, M, w, x, n, trans);
        cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
        if (st) break;
        if (ce != cudaSuccess) { st = cuda_fail(ce, "end capture"); break; }
        if (cudaGraphInstantiate(&exec, graph, 0)) { st = cuda_fail(cudaGetLastError(), "graph instantiate"); break; }
        for (;;) {
            if (cudaGraphLaunch(exec, c->stream)) { st = cuda_fail(cudaGetLastError(), "graph launch"); break; }
            *launches += (long long)kItersPerGraph * cg_launches_per_iter(M != nullptr);
            if (cudaMemcpyAsync(c->host_result, s, sizeof(SolverScalars), cudaMemcpyDeviceToHost, c->stream)) { st = cuda_fail(cudaGetLastError(), "cg"); break; }
            if (cudaStreamSynchronize(c->stream)) { st = cuda_fail(cudaGetLastError(), "cg sync"); break; }
            memcpy(&hs, c->host_result, sizeof(SolverScalars));
            if (hs.done) break;
        }
    } while (0);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    w.release();
    if (st) return st;
    HGB_TRY(collect_dev_error(c));
    *iters = hs.it;
    *rr_out = hs.rr;
    return HGB_OK;
}

static int true_residual(hgb_ctx *c, hgb_csr *A64, const double *b, const double *x, double *r, double *res,
                         long long *launches, bool trans = false) {
    *launches += 2;
    const long n = csr_rows(A64);
    HGB_CUDA(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
    if (trans) HGB_TRY(csr_ensure_transpose(A64));
    HGB_TRY(spmv_A<double, double>(c, A64, -1.0, x, 1.0, r, nullptr, nullptr, trans));
    residual_norm_kernel<<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, r, c->partials, c->counter, c->result);
    HGB_TRY(launch_check("residual_norm_kernel"));
    HGB_CUDA(cudaMemcpyAsync(c->host_result, c->result, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    *res = sqrt(c->host_result[0]);
    return HGB_OK;
}

}  // namespace hgb

using namespace hgb;

extern "C" {

int hgb_cg_solve(hgb_ctx *c, hgb_csr *A, hgb_ilu *M, const void *b, void *x, double tol, int max_iter,
                 hgb_solve_info *info) {
    return hgb_cg_solve_op(c, A, M, 'N', b, x, tol, max_iter, info);
}

int hgb_cg_solve_op(hgb_ctx *c, hgb_csr *A, hgb_ilu *M, char trans, const void *b, void *x, double tol, int max_iter,
                    hgb_solve_info *info) {
    if (!c || !A || !b || !x) return fail(HGB_ERR_ARG, "cg_solve: bad arguments");
    const bool tr = (trans == 'T' || trans == 't' || trans == 'C' || trans == 'c');
    if (!tr && trans != 'N' && trans != 'n') return fail(HGB_ERR_ARG, "cg_solve: trans '%c'", trans);
    if (csr_rows(A) != csr_cols(A)) return fail(HGB_ERR_ARG, "cg_solve: square matrix required");
    if (max_iter < 1) return fail(HGB_ERR_ARG, "cg_solve: max_iter < 1");
    DeviceGuard g(c->device);
    hgb_dtype dt = csr_dtype(A);
    if (M) {
        if (ilu_n(M) != csr_rows(A)) return fail(HGB_ERR_ARG, "cg_solve: preconditioner size");
        if (!ilu_matches(ilu_store(M), dt)) return fail(HGB_ERR_ARG, "cg_solve: preconditioner precision does not match the matrix");
    }
    if (dt == HGB_C128 || dt == HGB_C64) {
        if (tr) return fail(HGB_ERR_UNSUPPORTED, "cg_solve: transposed complex solves");
        return zcg_solve(c, A, M ? ilu_zfactor(M) : nullptr, b, x, tol, max_iter, info);
    }
    int it = 0;
    double rr = 0.0;
    double tol2 = tol * tol;
    long long launches = 0;
    int st;
    if (dt == HGB_F64) st = cg_run<double, double>(c, A, M, (const double *)b, (double *)x, tol2, 0.0, max_iter, false, &it, &rr, &launches, tr);
    else if (dt == HGB_F32) st = cg_run<float, float>(c, A, M, (const float *)b, (float *)x, tol2, 0.0, max_iter, false, &it, &rr, &launches, tr);
    else st = cg_run<uint16_t, float>(c, A, M, (const float *)b, (float *)x, tol2, 0.0, max_iter, false, &it, &rr, &launches, tr);
    if (st) return st;
    if (info) {
        info->iterations = it;
        info->outer = 0;
        info->residual = sqrt(rr);
        info->true_residual = -1.0;
        info->kernel_launches = launches;
    }
    return HGB_OK;
}

int hgb_ir_pcg_solve(hgb_ctx *c, hgb_csr *A64, hgb_csr *Ai, hgb_ilu *Mi, const double *b, double *x, double tol,
                     double inner_rtol, int max_inner, int max_outer, hgb_solve_info *info) {
    return hgb_ir_pcg_solve_op(c, A64, Ai, Mi, 'N', b, x, tol, inner_rtol, max_inner, max_outer, info);
}

int hgb_ir_pcg_solve_op(hgb_ctx *c, hgb_csr *A64, hgb_csr *Ai, hgb_ilu *Mi, char trans, const double *b, double *x,
                        double tol, double inner_rtol, int max_inner, int max_outer, hgb_solve_info *info) {
    if (!c || !A64 || !Ai || !b || !x) return fail(HGB_ERR_ARG, "ir_pcg: bad arguments");
    const bool tr = (trans == 'T' || trans == 't' || trans == 'C' || trans == 'c');
    if (!tr && trans != 'N' && trans != 'n') return fail(HGB_ERR_ARG, "ir_pcg: trans '%c'", trans);
    if (tr && csr_dtype(Ai) == HGB_BF16) return fail(HGB_ERR_UNSUPPORTED, "ir_pcg: transposed solve with a bf16 matrix");
    if (csr_dtype(A64) != HGB_F64) return fail(HGB_ERR_ARG, "ir_pcg: the outer matrix must be F64");
    if (!real_inner(csr_dtype(Ai))) return fail(HGB_ERR_ARG, "ir_pcg: the inner matrix must be F32 or BF16");
    if (Mi && !real_inner(ilu_store(Mi))) return fail(HGB_ERR_ARG, "ir_pcg: the inner preconditioner must store F32 or BF16");
    const long n = csr_rows(A64);
    if (csr_rows(Ai) != n || csr_cols(A64) != n) return fail(HGB_ERR_ARG, "ir_pcg: sizes");
    if (max_inner < 1 || max_outer < 0 || !(inner_rtol > 0.0)) return fail(HGB_ERR_ARG, "ir_pcg: limits");
    DeviceGuard g(c->device);
    double *r64 = nullptr;
    float *r32 = nullptr, *d32 = nullptr;
    int st = HGB_OK;
    int total = 0, outer = 0;
    double res = 0.0;
    long long launches = 0;
    do {
        if (ws_alloc(c, &r64, n) || ws_alloc(c, &r32, n) || ws_alloc(c, &d32, n)) {
            st = cuda_fail(cudaErrorMemoryAllocation, "ir_pcg workspace");
            break;
        }
        for (;;) {
            if ((st = true_residual(c, A64, b, x, r64, &res, &launches, tr))) break;
            if (res < tol || res == 0.0 || outer >= max_outer || !(res == res)) break;   // 0: x is exact
            f64_to_f32_kernel<<<ew_grid(c, n), 256, 0, c->stream>>>(n, r64, r32);
            zero_f32_kernel<<<ew_grid(c, n), 256, 0, c->stream>>>(n, d32);
            int it = 0;
            double rr = 0.0;
            launches += 3;   // residual cast, zero, update
            // reduce this sweep's residual only as far as the target needs (with a factor 2 of
            // margin), never by less than inner_rtol: the last sweep stops early
            const double rel = std::min(0.5, std::max(inner_rtol, 0.5 * tol / res));
            if (csr_dtype(Ai) == HGB_F32)
                st = cg_run<float, float>(c, Ai, Mi, r32, d32, 0.0, rel, max_inner, true, &it, &rr, &launches, tr);
            else
                st = cg_run<uint16_t, float>(c, Ai, Mi, r32, d32, 0.0, rel, max_inner, true, &it, &rr, &launches);
            if (st) break;
            total += it;
            add_f32_to_f64_kernel<<<ew_grid(c, n), 256, 0, c->stream>>>(n, d32, x);
            if ((st = launch_check("ir update"))) break;
            outer++;
        }
    } while (0);
    ws_free(c, r64);
    ws_free(c, r32);
    ws_free(c, d32);
    if (st) return st;
    if (info) {
        info->iterations = total;
        info->outer = outer;
        info->residual = res;
        info->true_residual = res;
        info->kernel_launches = launches;
    }
    if (!(res < tol || res == 0.0)) return fail(HGB_ERR_NOT_CONVERGED, "ir_pcg: ||b-Ax|| = %g after %d sweeps (tol %g)", res, outer, tol);
    return HGB_OK;
}

}  // extern "C"

// ============================================== mixed PCG with reliable updates =======
// One FP32 ILU(0)-PCG (solve_cg_core's order, hex/solvers/hala_solvers_cg.hpp:92-156) on the
// correction d, with FP64 reliable updates (van der Vorst and Ye, "Residual replacement
// strategies for Krylov subspace iterative methods for the convergence of true residuals",
// SIAM J. Sci. Comput. 22 (2000)): when ||r|| falls below delta times its largest value since
// the last update (or below tol, or at the iteration limit), x += d in FP64, r = b - A x in FP64
// and the iteration continues from the new residual with the same search direction, or restarts
// (beta = 0) when that update reduced the FP64 residual less than twice.  Unlike a
// restarted refinement, the Krylov space is kept, so the iterations stay those of FP64 PCG.
// No reference counterpart.  One iteration is nine launches, three of them (the update) no-ops
// except in update iterations; kItersPerGraph iterations are one CUDA graph.
namespace hgb {

__global__ void ru_init_kernel(SolverScalars *s, double tol2, double delta2, double rr, int max_iter) {
    s->it = 0;
    s->done = 0;
    s->max_iter = max_iter;
    s->tol2 = tol2;
    s->rel = 0.0;
    s->zr = s->nzr = s->pap = 0.0;
    s->rr = rr;
    s->rmax2 = rr;
    s->delta2 = delta2;
    s->ru_skip = 1;
    s->updates = 0;
    s->last2 = rr;
    s->restart = 0;
}

// a = <r,z>/<p,Ap>; d += a p; r -= a Ap; ||r||^2; decide whether this iteration updates
__global__ void __launch_bounds__(kEwThreads, kEwCtasPerSm) ru_step_kernel(long n, SolverScalars *s, const float *__restrict__ p, const float *__restrict__ Ap,
                               float *__restrict__ d, float *__restrict__ r, double *partials, unsigned *counter,
                               const double *pap_part, int pap_n) {
    if (s->done) return;
    const double pap = parts_sum(pap_part, pap_n, s->pap);
    const float a = (float)(s->zr / pap);
    const float ma = -a;
    DotAcc<float> rr;
    constexpr int U = ew_unroll<float, 4>();
    const long T = (long)gridDim.x * blockDim.x;
    for (long base = blockIdx.x * (long)blockDim.x + threadIdx.x; base < n; base += T * U) {
        float pv[U], av[U], dv[U], rv[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long i = base + u * T;
            if (i < n) {
                pv[u] = p[i];
                av[u] = Ap[i];
                dv[u] = d[i];
                rv[u] = r[i];
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long i = base + u * T;
            if (i < n) {
                d[i] = __fadd_rn(dv[u], __fmul_rn(a, pv[u]));
                const float ri = __fadd_rn(rv[u], __fmul_rn(ma, av[u]));
                r[i] = ri;
                rr.add(ri, ri);
            }
        }
    }
    double acc[1] = {rr.get()};
    grid_sum<1>(acc, partials, counter, [&](double (&v)[1]) {
        const double rr = v[0];
        s->pap = pap;
        s->rr = rr;
        s->it += 1;
        s->rmax2 = fmax(s->rmax2, rr);
        const bool upd = (rr < s->delta2 * s->rmax2) || (rr < s->tol2) || !(rr == rr) || (s->it >= s->max_iter);
        s->ru_skip = upd ? 0 : 1;
        s->restart = 0;
    });
}

// x += d (FP64); d = 0; r64 = b   (the FP64 product follows)
__global__ void ru_fold_kernel(long n, const SolverScalars *__restrict__ s, const double *__restrict__ b,
                               float *__restrict__ d, double *__restrict__ x, double *__restrict__ r64) {
    if (s->ru_skip) return;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        x[i] += (double)d[i];
        d[i] = 0.0f;
        r64[i] = b[i];
    }
}

// r = (float) r64; ||r64||^2; the stopping test on the FP64 residual
__global__ void ru_replace_kernel(long n, SolverScalars *s, const double *__restrict__ r64, float *__restrict__ r,
                                  double *partials, unsigned *counter) {
    if (s->ru_skip) return;
    double acc[1] = {0.0};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double v = r64[i];
        r[i] = (float)v;
        acc[0] += v * v;
    }
    grid_sum<1>(acc, partials, counter, [&](double (&v)[1]) {
        const double rr = v[0];
        s->rr = rr;
        s->rmax2 = rr;
        s->updates += 1;
        s->done = (rr < s->tol2) || !(rr == rr) || (s->it >= s->max_iter);
        s->ru_skip = 1;
        // an update that reduced ||r|| less than twice: the kept directions are stale (FP32
        // recurrences on an ill-conditioned operator), restart from the new residual
        s->restart = rr > 0.25 * s->last2;
        s->last2 = rr;
    });
}

// p = beta p + z with beta = <r,z> / <r,z>_old, or p = z after a restart
__global__ void __launch_bounds__(kEwThreads, kEwCtasPerSm) ru_p_kernel(long n, const SolverScalars *__restrict__ s, float *__restrict__ p,
                            const float *__restrict__ z) {
    if (s->done) return;
    const float bta = s->restart ? 0.0f : (float)(s->zr / s->nzr);
    constexpr int U = ew_unroll<float>();
    const long T = (long)gridDim.x * blockDim.x;
    for (long base = blockIdx.x * (long)blockDim.x + threadIdx.x; base < n; base += T * U) {
        float pv[U], zv[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long i = base + u * T;
            if (i < n) {
                pv[u] = p[i];
                zv[u] = z[i];
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long i = base + u * T;
            if (i < n) p[i] = __fadd_rn(__fmul_rn(bta, pv[u]), zv[u]);
        }
    }
}

template <typename V>
static int ru_iteration(hgb_ctx *c, hgb_csr *A64, hgb_csr *Ai, hgb_ilu *M, CgWork<float> &w, float *d, double *x,
                        double *r64, const double *b, long n, bool trans) {
    SolverScalars *s = c->scal;
    const int *done = &s->done;
    int np = 0;
    HGB_TRY(spmv_A<V, float>(c, Ai, 1.0f, w.p, 0.0f, w.Ap, &s->pap, done, trans, &np));
    ru_step_kernel<<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, s, w.p, w.Ap, d, w.r, c->partials, c->counter,
                                                                      c->partials + kSpmvPartsOffset, np);
    ru_fold_kernel<<<ew_grid(c, n), 256, 0, c->stream>>>(n, s, b, d, x, r64);
    HGB_TRY(spmv_A<double, double>(c, A64, -1.0, x, 1.0, r64, nullptr, &s->ru_skip, trans));
    ru_replace_kernel<<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, s, r64, w.r, c->partials, c->counter);
    float *z = M ? w.z : w.r;
    if (M) HGB_TRY(ilu_apply_internal(M, trans ? 'T' : 'N', w.r, w.z, done));
    cg_rz_kernel<float><<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, s, w.r, z, c->partials, c->counter, 0);
    ru_p_kernel<<<ew_grid(c, n), 256, 0, c->stream>>>(n, s, w.p, z);
    return launch_check("ru iteration");
}

static int ru_launches_per_iter(bool precond) { return precond ? 9 : 7; }

template <typename V>
static int ru_run(hgb_ctx *c, hgb_csr *A64, hgb_csr *Ai, hgb_ilu *M, const double *b, double *x, double tol,
                  double delta, int max_iter, int *iters, int *updates, double *res, long long *launches,
                  bool trans = false) {
    const long n = csr_rows(A64);
    CaptureStream cs(c);
    CgWork<float> w;
    float *d = nullptr;
    double *r64 = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    SolverScalars hs{};
    int st = w.alloc(c, n, M != nullptr);
    do {
        if (st) break;
        if (ws_alloc(c, &d, n) || ws_alloc(c, &r64, n)) {
            st = cuda_fail(cudaErrorMemoryAllocation, "ru_pcg workspace");
            break;
        }
        double rn = 0.0;
        if (trans && (st = csr_ensure_transpose(Ai))) break;
        if ((st = true_residual(c, A64, b, x, r64, &rn, launches, trans))) break;
        *iters = 0;
        *updates = 0;
        *res = rn;
        if (rn < tol || rn == 0.0 || !(rn == rn) || max_iter < 1) break;   // 0: x is exact
        SolverScalars *s = c->scal;
        ru_init_kernel<<<1, 1, 0, c->stream>>>(s, tol * tol, delta * delta, rn * rn, max_iter);
        f64_to_f32_kernel<<<ew_grid(c, n), 256, 0, c->stream>>>(n, r64, w.r);
        zero_f32_kernel<<<ew_grid(c, n), 256, 0, c->stream>>>(n, d);
        float *z = M ? w.z : w.r;
        if (M && (st = ilu_apply_internal(M, trans ? 'T' : 'N', w.r, w.z, nullptr))) break;
        copy_kernel<float><<<ew_grid(c, n), 256, 0, c->stream>>>(n, z, w.p);
        // <r,z> of the first direction (the rr slot keeps the FP64 residual)
        cg_rz_kernel<float><<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, s, w.r, z, c->partials, c->counter, 0);
        *launches += 5 + (M ? 2 : 0);
        if ((st = launch_check("ru init"))) break;
        if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal)) { st = cuda_fail(cudaGetLastError(), "begin capture"); break; }
        for (int k = 0; k < kItersPerGraph && !st; k++) st = ru_iteration<V>(c, A64, Ai, M, w, d, x, r64, b, n, trans);
        cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
        if (st) break;
        if (ce != cudaSuccess) { st = cuda_fail(ce, "end capture"); break; }
        if (cudaGraphInstantiate(&exec, graph, 0)) { st = cuda_fail(cudaGetLastError(), "graph instantiate"); break; }
        for (;;) {
            if (cudaGraphLaunch(exec, c->stream)) { st = cuda_fail(cudaGetLastError(), "graph launch"); break; }
            *launches += (long long)kItersPerGraph * ru_launches_per_iter(M != nullptr);
            if (cudaMemcpyAsync(c->host_result, s, sizeof(SolverScalars), cudaMemcpyDeviceToHost, c->stream) ||
                cudaStreamSynchronize(c->stream)) { st = cuda_fail(cudaGetLastError(), "ru_pcg sync"); break; }
            memcpy(&hs, c->host_result, sizeof(SolverScalars));
            if (hs.done) break;
        }
        *iters = hs.it;
        *updates = hs.updates;
        *res = sqrt(hs.rr);
    } while (0);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    w.release();
    ws_free(c, d);
    ws_free(c, r64);
    if (st) return st;
    return collect_dev_error(c);
}

}  // namespace hgb

extern "C" int hgb_ru_pcg_solve(hgb_ctx *c, hgb_csr *A64, hgb_csr *Ai, hgb_ilu *Mi, const double *b, double *x,
                                double tol, double delta, int max_iter, hgb_solve_info *info) {
    return hgb_ru_pcg_solve_op(c, A64, Ai, Mi, 'N', b, x, tol, delta, max_iter, info);
}

extern "C" int hgb_ru_pcg_solve_op(hgb_ctx *c, hgb_csr *A64, hgb_csr *Ai, hgb_ilu *Mi, char trans, const double *b,
                                   double *x, double tol, double delta, int max_iter, hgb_solve_info *info) {
    if (!c || !A64 || !Ai || !b || !x) return fail(HGB_ERR_ARG, "ru_pcg: bad arguments");
    const bool tr = (trans == 'T' || trans == 't' || trans == 'C' || trans == 'c');
    if (!tr && trans != 'N' && trans != 'n') return fail(HGB_ERR_ARG, "ru_pcg: trans '%c'", trans);
    if (tr && csr_dtype(Ai) == HGB_BF16) return fail(HGB_ERR_UNSUPPORTED, "ru_pcg: transposed solve with a bf16 matrix");
    if (csr_dtype(A64) != HGB_F64) return fail(HGB_ERR_ARG, "ru_pcg: the outer matrix must be F64");
    if (!real_inner(csr_dtype(Ai))) return fail(HGB_ERR_ARG, "ru_pcg: the inner matrix must be F32 or BF16");
    if (Mi && !real_inner(ilu_store(Mi))) return fail(HGB_ERR_ARG, "ru_pcg: the preconditioner must store F32 or BF16");
    const long n = csr_rows(A64);
    if (csr_rows(Ai) != n || csr_cols(A64) != n || csr_cols(Ai) != n || (Mi && ilu_n(Mi) != n))
        return fail(HGB_ERR_ARG, "ru_pcg: sizes");
    if (max_iter < 0 || !(delta > 0.0 && delta < 1.0)) return fail(HGB_ERR_ARG, "ru_pcg: limits (0 < delta < 1)");
    DeviceGuard g(c->device);
    int it = 0, upd = 0;
    double res = 0.0;
    long long launches = 0;
    int st = (csr_dtype(Ai) == HGB_F32)
                 ? ru_run<float>(c, A64, Ai, Mi, b, x, tol, delta, max_iter, &it, &upd, &res, &launches, tr)
                 : ru_run<uint16_t>(c, A64, Ai, Mi, b, x, tol, delta, max_iter, &it, &upd, &res, &launches);
    if (st) return st;
    if (info) {
        info->iterations = it;
        info->outer = upd;
        info->residual = res;
        info->true_residual = res;
        info->kernel_launches = launches;
    }
    if (!(res < tol || res == 0.0)) return fail(HGB_ERR_NOT_CONVERGED, "ru_pcg: ||b-Ax|| = %g after %d iterations (tol %g)", res, it, tol);
    return HGB_OK;
}

// ===================================================================== GMRES ===========
// solve_gmres (hex/solvers/hala_solvers_gmres.hpp:127-230), device resident.  The reference
// reads the projection coefficients back to the host in every inner iteration (:67-72) and
// rotates on the host; here the Hessenberg columns, the Givens rotations, the residual estimate
// and the back substitution (tpsv) live in a GmresState in device memory and are updated by the
// last CTA of the projection's grid reduction.  Inner iteration j of a cycle always projects
// against j+1 basis vectors, so one whole restart cycle is captured once into a CUDA graph; the
// launches of iterations after the inner stop are no-ops, and the host reads the state once per
// cycle.  The arithmetic of the rotations, of tpsv and of the x update is the reference's
// operation for operation (explicitly rounded, no contraction); the inner products are parallel.
namespace hgb {

constexpr int kGmresMaxRestart = 512;   // the Hessenberg factor (1 MB) lives in device memory

struct GmresState {
    // header (read by the host after every cycle)
    double tol;          // threshold on the preconditioned residual estimate
    double rel;          // > 0: tol = max(tol, rel * first estimate) (inner solves of a refinement)
    double inner_res, outer_res;
    double inv;          // reciprocal of the norm of the vector being appended
    int k, stop, done, wcol, upd, total, outer, max_outer, restart, first;
    // rotations and the triangular factor
    double Z[kGmresMaxRestart + 1];
    double C[kGmresMaxRestart], S[kGmresMaxRestart];
    double H[kGmresMaxRestart * (kGmresMaxRestart + 1) / 2];
};

__device__ __forceinline__ void gm_rotg(double &a, double &b, double &c, double &s) {
    double roe = (fabs(a) > fabs(b)) ? a : b;
    double scale = __dadd_rn(fabs(a), fabs(b)), r, z;
    if (scale == 0.0) {
        c = 1.0; s = 0.0; r = 0.0; z = 0.0;
    } else {
        double as = __ddiv_rn(a, scale), bs = __ddiv_rn(b, scale);
        r = __dmul_rn(scale, __dsqrt_rn(__dadd_rn(__dmul_rn(as, as), __dmul_rn(bs, bs))));
        if (roe < 0.0) r = -r;
        c = __ddiv_rn(a, r);
        s = __ddiv_rn(b, r);
        z = 1.0;
        if (fabs(a) > fabs(b)) z = s;
        if (fabs(b) >= fabs(a) && c != 0.0) z = __ddiv_rn(1.0, c);
    }
    a = r;
    b = z;
}

__device__ __forceinline__ void gm_rot(double &x, double &y, double c, double s) {
    double t = __dadd_rn(__dmul_rn(c, x), __dmul_rn(s, y));
    y = __dsub_rn(__dmul_rn(c, y), __dmul_rn(s, x));
    x = t;
}

__global__ void gm_init_kernel(GmresState *st, double tol, double rel, int max_outer, int restart) {
    st->tol = tol;
    st->rel = rel;
    st->inner_res = 0.0;
    st->outer_res = tol + 1.0;
    st->inv = 0.0;
    st->k = 0;
    st->stop = 1;
    st->done = !(max_outer > 0);
    st->wcol = -1;
    st->upd = 0;
    st->total = 0;
    st->outer = 0;
    st->max_outer = max_outer;
    st->restart = restart;
    st->first = 1;
}

__global__ void gm_begin_kernel(GmresState *st) {
    st->k = 0;
    st->upd = 0;
    st->wcol = -1;
    st->stop = 1;
}

template <typename X>
__global__ void gm_copy_kernel(long n, const int *skip, const X *__restrict__ a, X *__restrict__ b) {
    if (*skip) return;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) b[i] = a[i];
}

// beta = ||P^-1 (b - A x)||: the first estimate of the cycle (Z[0]); basis vector 0 follows
template <typename X>
__global__ void gm_start_kernel(long n, GmresState *st, const X *__restrict__ r, double *partials,
                                unsigned *counter) {
    if (st->done) return;
    double acc[1] = {0.0};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        acc[0] += (double)r[i] * (double)r[i];
    grid_sum<1>(acc, partials, counter, [&](double (&v)[1]) {
        double beta = __dsqrt_rn(v[0]);
        if (st->first) {
            st->first = 0;
            if (st->rel > 0.0) st->tol = fmax(st->tol, st->rel * beta);
        }
        st->total += 1;
        st->inner_res = beta;
        st->Z[0] = beta;
        bool go = beta > st->tol;
        st->stop = !go;
        st->wcol = go ? 0 : -1;
        st->inv = __ddiv_rn(1.0, beta);
    });
}

// r *= inv; W[:, wcol] = r   (scal(1/nrm, r) and the copy into the basis)
template <typename X>
__global__ void gm_scale_kernel(long n, const GmresState *__restrict__ st, X *__restrict__ r, X *__restrict__ W) {
    const int col = st->wcol;
    if (col < 0) return;
    const X a = (X)st->inv;
    X *w = W + (long)col * n;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        X v = mul_rn(r[i], a);
        r[i] = v;
        w[i] = v;
    }
}

// cf[0..k] = W[:, 0..k]^T r   (krylov_project's gemv 'T', :67-70), for the k1 columns from W and cf
// on (one group of up to 64 columns per launch)
template <typename X, int KMAX>
__global__ void gm_dots_kernel(long n, int k1, const GmresState *__restrict__ st, const X *__restrict__ W,
                               const X *__restrict__ r, double *cf, double *partials, unsigned *counter) {
    if (st->stop) return;
    double acc[KMAX];
#pragma unroll
    for (int j = 0; j < KMAX; j++) acc[j] = 0.0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double ri = (double)r[i];
#pragma unroll
        for (int j = 0; j < KMAX; j++)
            if (j < k1) acc[j] += (double)W[(long)j * n + i] * ri;
    }
    grid_sum<KMAX>(acc, partials, counter, [&](double (&s)[KMAX]) {
        for (int j = 0; j < k1; j++) cf[j] = s[j];
    });
}

// r -= W cf (krylov_project's gemv 'N', :71-76), ||r||, then in the last CTA the Givens step of
// solve_gmres (:190-216) for column k of the Hessenberg matrix.
template <typename X>
__global__ void gm_update_kernel(long n, int k, GmresState *st, const X *__restrict__ W, const double *__restrict__ cf,
                                 X *__restrict__ r, double *partials, unsigned *counter) {
    if (st->stop) return;
    double acc[1] = {0.0};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        X ri = r[i];
        for (int j = 0; j <= k; j++) ri = add_rn(ri, mul_rn((X)-cf[j], W[(long)j * n + i]));
        r[i] = ri;
        acc[0] += (double)ri * (double)ri;
    }
    grid_sum<1>(acc, partials, counter, [&](double (&v)[1]) {
        const double nrm = __dsqrt_rn(v[0]);
        // the previous rotations applied to the new column in order, carrying h[i + 1] in a register
        double *Hk = st->H + (long)k * (k + 1) / 2;
        double hi = cf[0];
        for (int i = 0; i < k; i++) {
            double hn = cf[i + 1];
            gm_rot(hi, hn, st->C[i], st->S[i]);
            Hk[i] = hi;
            hi = hn;
        }
        double beta = nrm, ic, is;
        gm_rotg(hi, beta, ic, is);
        Hk[k] = hi;
        st->S[k] = is;
        st->C[k] = ic;
        const double res = fabs(__dmul_rn(is, st->Z[k]));
        st->inner_res = res;
        st->total += 1;
        st->k = k + 1;
        const bool expand = (res > st->tol) && (k + 1 < st->restart);
        if (expand) {
            st->Z[k + 1] = 0.0;
            gm_rot(st->Z[k], st->Z[k + 1], ic, is);
            st->wcol = k + 1;
            st->inv = __ddiv_rn(1.0, nrm);
        } else {
            st->wcol = -1;
            st->stop = 1;
        }
    });
}

// End of a cycle: tpsv('U','N','N', k, H, Z) (:219-223), the restart bookkeeping (:225-229)
__global__ void gm_end_kernel(GmresState *st) {
    if (st->done) return;
    const int nz = st->k;
    if (nz > 0) {
        long kk = (long)nz * (nz + 1) / 2 - 1;
        for (int j = nz - 1; j >= 0; j--) {
            if (st->Z[j] != 0.0) {
                st->Z[j] = __ddiv_rn(st->Z[j], st->H[kk]);
                const double tt = st->Z[j];
                long q = kk - 1;
                for (int i = j - 1; i >= 0; i--, q--) st->Z[i] = __dsub_rn(st->Z[i], __dmul_rn(tt, st->H[q]));
            }
            kk -= j + 1;
        }
        st->upd = 1;
    }
    st->outer += 1;
    st->outer_res = st->inner_res;
    st->done = !(st->outer_res > st->tol && st->outer < st->max_outer);
}

// x += W[:, 0..k-1] Z   (krylov_combine, :53-60), column by column in the reference's order
template <typename X>
__global__ void gm_xupdate_kernel(long n, const GmresState *__restrict__ st, const X *__restrict__ W, X *__restrict__ x) {
    if (!st->upd) return;
    const int nz = st->k;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        X xi = x[i];
        for (int j = 0; j < nz; j++) xi = add_rn(xi, mul_rn((X)st->Z[j], W[(long)j * n + i]));
        x[i] = xi;
    }
}

template <typename X>
static int gm_dots_launch(hgb_ctx *c, long n, int k1, const GmresState *st, const X *W, const X *r, double *cf) {
    // up to 64 partial sums per CTA: the grid stays below the SpMV parts of the context's partials
    const int grid = std::min(reduce_grid(c, n, 256 * 8), (int)(kSpmvPartsOffset / 64));
    for (int j0 = 0; j0 < k1; j0 += 64) {   // groups of up to 64 columns, one grid reduction each
        const int kk = std::min(64, k1 - j0);
        const X *Wj = W + (long)j0 * n;
        double *cj = cf + j0;
        if (kk <= 8) gm_dots_kernel<X, 8><<<grid, 256, 0, c->stream>>>(n, kk, st, Wj, r, cj, c->partials, c->counter);
        else if (kk <= 16) gm_dots_kernel<X, 16><<<grid, 256, 0, c->stream>>>(n, kk, st, Wj, r, cj, c->partials, c->counter);
        else if (kk <= 32) gm_dots_kernel<X, 32><<<grid, 256, 0, c->stream>>>(n, kk, st, Wj, r, cj, c->partials, c->counter);
        else gm_dots_kernel<X, 64><<<grid, 256, 0, c->stream>>>(n, kk, st, Wj, r, cj, c->partials, c->counter);
        HGB_TRY(launch_check("gm_dots_kernel"));
    }
    return HGB_OK;
}

// Runs restarted GMRES on (A, M) for b -> x (x holds the initial guess).  tol: absolute threshold
// on the preconditioned residual estimate; rel > 0 also stops at rel * the first estimate;
// max_outer: restart cycles.
template <typename V, typename X>
static int gmres_run(hgb_ctx *c, hgb_csr *A, hgb_ilu *M, int restart, const X *b, X *x, double tol, double rel,
                     int max_outer, int *total, int *outer, double *res, long long *launches) {
    const long n = csr_rows(A);
    CaptureStream cs(c);
    X *t = nullptr, *r = nullptr, *W = nullptr;
    double *cf = nullptr;
    GmresState *st = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const int pre = M ? 2 : 1;          // ILU: L and U sweeps; none: a copy
    const long long per_cycle = 6 + pre + (long long)restart * (4 + pre);
    int rc = HGB_OK;
    do {
        if (ws_alloc(c, &t, n) || ws_alloc(c, &r, n) || ws_alloc(c, &W, (size_t)n * restart) ||
            ws_alloc(c, &cf, kGmresMaxRestart + 1) || ws_alloc(c, &st, 1)) {
            rc = cuda_fail(cudaErrorMemoryAllocation, "gmres workspace");
            break;
        }
        gm_init_kernel<<<1, 1, 0, c->stream>>>(st, tol, rel, max_outer, restart);
        *launches += 1;
        if ((rc = launch_check("gm_init_kernel"))) break;
        auto precon = [&](const X *in, X *out, const int *skip) -> int {
            if (M) return ilu_apply_internal(M, 'N', in, out, skip);
            gm_copy_kernel<X><<<ew_grid(c, n), 256, 0, c->stream>>>(n, skip, in, out);
            return launch_check("gm_copy_kernel");
        };
        if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal)) { rc = cuda_fail(cudaGetLastError(), "begin capture"); break; }
        do {
            // t = b - A x ; r = P^-1 t ; beta = ||r|| ; W[:,0] = r / beta
            gm_begin_kernel<<<1, 1, 0, c->stream>>>(st);
            gm_copy_kernel<X><<<ew_grid(c, n), 256, 0, c->stream>>>(n, &st->done, b, t);
            if ((rc = spmv_A<V, X>(c, A, X(-1), x, X(1), t, nullptr, &st->done))) break;
            if ((rc = precon(t, r, &st->done))) break;
            gm_start_kernel<X><<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, st, r, c->partials, c->counter);
            gm_scale_kernel<X><<<ew_grid(c, n), 256, 0, c->stream>>>(n, st, r, W);
            for (int k = 0; k < restart && !rc; k++) {
                if ((rc = spmv_A<V, X>(c, A, X(1), r, X(0), t, nullptr, &st->stop))) break;
                if ((rc = precon(t, r, &st->stop))) break;
                if ((rc = gm_dots_launch<X>(c, n, k + 1, st, W, r, cf))) break;
                gm_update_kernel<X><<<reduce_grid(c, n, 256 * 4), 256, 0, c->stream>>>(n, k, st, W, cf, r, c->partials,
                                                                                       c->counter);
                gm_scale_kernel<X><<<ew_grid(c, n), 256, 0, c->stream>>>(n, st, r, W);
            }
            if (rc) break;
            gm_end_kernel<<<1, 1, 0, c->stream>>>(st);
            gm_xupdate_kernel<X><<<ew_grid(c, n), 256, 0, c->stream>>>(n, st, W, x);
            rc = launch_check("gmres cycle");
        } while (0);
        cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
        if (rc) break;
        if (ce != cudaSuccess) { rc = cuda_fail(ce, "end capture"); break; }
        if (cudaGraphInstantiate(&exec, graph, 0)) { rc = cuda_fail(cudaGetLastError(), "graph instantiate"); break; }
        GmresState hs{};
        const size_t head = offsetof(GmresState, Z);
        for (;;) {
            if (cudaGraphLaunch(exec, c->stream)) { rc = cuda_fail(cudaGetLastError(), "graph launch"); break; }
            *launches += per_cycle;
            if (cudaMemcpyAsync(c->host_result, st, head, cudaMemcpyDeviceToHost, c->stream) ||
                cudaStreamSynchronize(c->stream)) { rc = cuda_fail(cudaGetLastError(), "gmres"); break; }
            memcpy(&hs, c->host_result, head);
            if (hs.done) break;
        }
        *total = hs.total;
        *outer = hs.outer;
        *res = hs.inner_res;
    } while (0);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    ws_free(c, t);
    ws_free(c, r);
    ws_free(c, W);
    ws_free(c, cf);
    ws_free(c, st);
    if (rc) return rc;
    return collect_dev_error(c);
}

}  // namespace hgb

extern "C" int hgb_gmres_solve(hgb_ctx *c, hgb_csr *A, hgb_ilu *M, int restart, const void *bv, void *xv, double tol,
                               int max_iter, hgb_solve_info *info) {
    if (!c || !A || !bv || !xv || restart < 1 || restart > kGmresMaxRestart)
        return fail(HGB_ERR_ARG, "gmres: bad arguments (restart 1..%d)", kGmresMaxRestart);
    if (csr_rows(A) != csr_cols(A)) return fail(HGB_ERR_ARG, "gmres: square matrix required");
    const hgb_dtype dt = csr_dtype(A);
    if (M) {
        if (ilu_n(M) != csr_rows(A)) return fail(HGB_ERR_ARG, "gmres: preconditioner size");
        if (!ilu_matches(ilu_store(M), dt)) return fail(HGB_ERR_ARG, "gmres: preconditioner precision does not match the matrix");
    }
    DeviceGuard g(c->device);
    if (dt == HGB_C128 || dt == HGB_C64)
        return zgmres_solve(c, A, M ? ilu_zfactor(M) : nullptr, restart, bv, xv, tol, max_iter, info);
    int total = 0, outer = 0;
    double res = 0.0;
    long long launches = 0;
    int st;
    if (dt == HGB_F64)
        st = gmres_run<double, double>(c, A, M, restart, (const double *)bv, (double *)xv, tol, 0.0, max_iter, &total, &outer, &res, &launches);
    else if (dt == HGB_F32)
        st = gmres_run<float, float>(c, A, M, restart, (const float *)bv, (float *)xv, tol, 0.0, max_iter, &total, &outer, &res, &launches);
    else
        st = gmres_run<uint16_t, float>(c, A, M, restart, (const float *)bv, (float *)xv, tol, 0.0, max_iter, &total, &outer, &res, &launches);
    if (st) return st;
    if (info) {
        info->iterations = total;
        info->outer = outer;
        info->residual = res;
        info->true_residual = -1.0;
        info->kernel_launches = launches;
    }
    return HGB_OK;
}

// Mixed-precision GMRES: FP64 iterative refinement around an FP32-vector GMRES(restart) with an
// FP32 or BF16 matrix and ILU(0) (no reference counterpart; the inner solver is solve_gmres).
extern "C" int hgb_ir_gmres_solve(hgb_ctx *c, hgb_csr *A64, hgb_csr *Ai, hgb_ilu *Mi, int restart, const double *b,
                                  double *x, double tol, double inner_rtol, int max_inner, int max_outer,
                                  hgb_solve_info *info) {
    if (!c || !A64 || !Ai || !b || !x || restart < 1 || restart > kGmresMaxRestart)
        return fail(HGB_ERR_ARG, "ir_gmres: bad arguments (restart 1..%d)", kGmresMaxRestart);
    if (csr_dtype(A64) != HGB_F64) return fail(HGB_ERR_ARG, "ir_gmres: the outer matrix must be F64");
    if (!real_inner(csr_dtype(Ai))) return fail(HGB_ERR_ARG, "ir_gmres: the inner matrix must be F32 or BF16");
    if (Mi && !real_inner(ilu_store(Mi))) return fail(HGB_ERR_ARG, "ir_gmres: the inner preconditioner must store F32 or BF16");
    const long n = csr_rows(A64);
    if (csr_rows(Ai) != n || csr_cols(A64) != n || csr_cols(Ai) != n || (Mi && ilu_n(Mi) != n))
        return fail(HGB_ERR_ARG, "ir_gmres: sizes");
    if (max_inner < 1 || max_outer < 0 || !(inner_rtol > 0.0)) return fail(HGB_ERR_ARG, "ir_gmres: limits");
    DeviceGuard g(c->device);
    double *r64 = nullptr;
    float *r32 = nullptr, *d32 = nullptr;
    int st = HGB_OK;
    int total = 0, outer = 0;
    double res = 0.0;
    long long launches = 0;
    const int cycles = (max_inner + restart - 1) / restart;
    do {
        if (ws_alloc(c, &r64, n) || ws_alloc(c, &r32, n) || ws_alloc(c, &d32, n)) {
            st = cuda_fail(cudaErrorMemoryAllocation, "ir_gmres workspace");
            break;
        }
        for (;;) {
            if ((st = true_residual(c, A64, b, x, r64, &res, &launches))) break;
            if (res < tol || res == 0.0 || outer >= max_outer || !(res == res)) break;   // 0: x is exact
            f64_to_f32_kernel<<<ew_grid(c, n), 256, 0, c->stream>>>(n, r64, r32);
            zero_f32_kernel<<<ew_grid(c, n), 256, 0, c->stream>>>(n, d32);
            launches += 3;   // residual cast, zero, update
            // as the refinement CG: this sweep reduces its (preconditioned) residual as far as the
            // target needs with a factor 2 of margin, never by less than inner_rtol
            const double rel = std::min(0.5, std::max(inner_rtol, 0.5 * tol / res));
            int it = 0, cyc = 0;
            double ires = 0.0;
            if (csr_dtype(Ai) == HGB_F32)
                st = gmres_run<float, float>(c, Ai, Mi, restart, r32, d32, 0.0, rel, cycles, &it, &cyc, &ires, &launches);
            else
                st = gmres_run<uint16_t, float>(c, Ai, Mi, restart, r32, d32, 0.0, rel, cycles, &it, &cyc, &ires, &launches);
            if (st) break;
            total += it;
            add_f32_to_f64_kernel<<<ew_grid(c, n), 256, 0, c->stream>>>(n, d32, x);
            if ((st = launch_check("ir update"))) break;
            outer++;
        }
    } while (0);
    ws_free(c, r64);
    ws_free(c, r32);
    ws_free(c, d32);
    if (st) return st;
    if (info) {
        info->iterations = total;
        info->outer = outer;
        info->residual = res;
        info->true_residual = res;
        info->kernel_launches = launches;
    }
    if (!(res < tol || res == 0.0)) return fail(HGB_ERR_NOT_CONVERGED, "ir_gmres: ||b-Ax|| = %g after %d sweeps (tol %g)", res, outer, tol);
    return HGB_OK;
}

// ========================================================== host-buffer (mixed) solve ====
extern "C" int hgb_mixed_cg_solve(hgb_ctx *c, int n, int nnz, const int *pntr_h, const int *indx_h, const double *vals_h,
                                  hgb_ilu *M, const double *b_h, double *x_h, double tol, int max_iter,
                                  hgb_solve_info *info) {
    if (!c || n <= 0 || nnz < 0 || !pntr_h || !indx_h || !vals_h || !b_h || !x_h) return fail(HGB_ERR_ARG, "mixed_cg: bad arguments");
    DeviceGuard g(c->device);
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    size_t op = 0, oi = op + al(sizeof(int) * (n + 1)), ov = oi + al(sizeof(int) * (size_t)nnz);
    size_t ob = ov + al(sizeof(double) * (size_t)nnz), ox = ob + al(sizeof(double) * n), total = ox + al(sizeof(double) * n);
    if (c->arena_bytes < total) {
        cudaFree(c->arena);
        c->arena = nullptr;
        c->arena_bytes = 0;
        HGB_CUDA(cudaMalloc(&c->arena, total));
        c->arena_bytes = total;
    }
    char *base = (char *)c->arena;
    int *dp = (int *)(base + op), *di = (int *)(base + oi);
    double *dv = (double *)(base + ov), *db = (double *)(base + ob), *dx = (double *)(base + ox);
    // the loads (gpu_engine::load, wax/hala_lib_extensions.hpp:137-146) in chunks on the copy stream,
    // ordered after the caller's earlier work on the context's stream and before the solve
    HGB_CUDA(cudaEventRecord(c->ev_in, c->stream));
    HGB_CUDA(cudaStreamWaitEvent(c->copy, c->ev_in, 0));
    HGB_TRY(h2d_chunked(c, c->copy, dp, pntr_h, sizeof(int) * (n + 1)));
    HGB_TRY(h2d_chunked(c, c->copy, di, indx_h, sizeof(int) * (size_t)nnz));
    HGB_TRY(h2d_chunked(c, c->copy, dv, vals_h, sizeof(double) * (size_t)nnz));
    HGB_TRY(h2d_chunked(c, c->copy, db, b_h, sizeof(double) * n));
    HGB_TRY(h2d_chunked(c, c->copy, dx, x_h, sizeof(double) * n));
    HGB_CUDA(cudaEventRecord(c->ev_out, c->copy));
    HGB_CUDA(cudaStreamWaitEvent(c->stream, c->ev_out, 0));
    hgb_csr *A = nullptr;
    HGB_TRY(hgb_csr_create(c, n, n, nnz, dp, di, dv, HGB_F64, &A));
    int st = hgb_cg_solve(c, A, M, db, dx, tol, max_iter, info);
    hgb_csr_destroy(A);
    if (st) return st;
    HGB_CUDA(cudaMemcpyAsync(x_h, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    return HGB_OK;
}

namespace hgb {
__global__ void f64_to_inner_kernel(long n, const double *__restrict__ a, float *f32, uint16_t *b16) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        float v = (float)a[i];
        if (f32) f32[i] = v;
        if (b16) {
            uint32_t u = __float_as_uint(v);
            b16[i] = ((u & 0x7fffffffu) > 0x7f800000u) ? (uint16_t)((u >> 16) | 0x40u)
                                                      : (uint16_t)((u + 0x7fffu + ((u >> 16) & 1u)) >> 16);
        }
    }
}
}  // namespace hgb

// Host-buffer mixed solves: pntr/indx/vals (FP64) and b/x are loaded into the context's arena, the
// inner matrix is converted on the device to Mi's store precision, the solver runs on the device
// copies and x is read back (also when the solve did not converge).
template <typename Solve>
static int mixed_host_solve(hgb_ctx *c, const char *what, int n, int nnz, const int *pntr_h, const int *indx_h,
                            const double *vals_h, hgb_ilu *Mi, const double *b_h, double *x_h, hgb_solve_info *info,
                            Solve solve) {
    if (!c || n <= 0 || nnz < 0 || !pntr_h || !indx_h || !vals_h || !b_h || !x_h || !Mi)
        return fail(HGB_ERR_ARG, "%s: bad arguments", what);
    if (!real_inner(ilu_store(Mi))) return fail(HGB_ERR_ARG, "%s: the preconditioner must store F32 or BF16", what);
    DeviceGuard g(c->device);
    // the inner operator is FP32 whatever the factor's store: BF16 values shift the operator (on the
    // 128^3 system the rounded diagonal moves it by nine times its smallest eigenvalue) and the
    // refinement's fixed point with it, while a BF16 factor only changes the preconditioner
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    size_t op = 0, oi = op + al(sizeof(int) * (n + 1)), ov = oi + al(sizeof(int) * (size_t)nnz);
    size_t ow = ov + al(sizeof(double) * (size_t)nnz), ob = ow + al(sizeof(float) * (size_t)nnz);
    size_t ox = ob + al(sizeof(double) * n), total = ox + al(sizeof(double) * n);
    if (c->arena_bytes < total) {
        cudaFree(c->arena);
        c->arena = nullptr;
        c->arena_bytes = 0;
        HGB_CUDA(cudaMalloc(&c->arena, total));
        c->arena_bytes = total;
    }
    char *base = (char *)c->arena;
    int *dp = (int *)(base + op), *di = (int *)(base + oi);
    double *dv = (double *)(base + ov), *db = (double *)(base + ob), *dx = (double *)(base + ox);
    void *dw = base + ow;
    // The loads in chunks on the copy stream, overlapped with the conversion of the values to the
    // inner precision on the context's stream: each chunk of values is converted as soon as it has
    // landed, while the next chunks are in flight.
    HGB_CUDA(cudaEventRecord(c->ev_in, c->stream));
    HGB_CUDA(cudaStreamWaitEvent(c->copy, c->ev_in, 0));
    HGB_TRY(h2d_chunked(c, c->copy, dp, pntr_h, sizeof(int) * (n + 1)));
    HGB_TRY(h2d_chunked(c, c->copy, di, indx_h, sizeof(int) * (size_t)nnz));
    constexpr long kChunk = 1L << 21;   // values per conversion chunk (16 MB of FP64)
    for (long o = 0; o < nnz; o += kChunk) {
        const long m = std::min(kChunk, (long)nnz - o);
        HGB_TRY(h2d_chunked(c, c->copy, dv + o, vals_h + o, sizeof(double) * (size_t)m));
        HGB_CUDA(cudaEventRecord(c->ev_out, c->copy));
        HGB_CUDA(cudaStreamWaitEvent(c->stream, c->ev_out, 0));   // waits on this record, not later ones
        f64_to_inner_kernel<<<ew_grid(c, m), 256, 0, c->stream>>>(
            m, dv + o, (float *)dw + o, nullptr);
        HGB_TRY(launch_check("f64_to_inner_kernel"));
    }
    HGB_TRY(h2d_chunked(c, c->copy, db, b_h, sizeof(double) * n));
    HGB_TRY(h2d_chunked(c, c->copy, dx, x_h, sizeof(double) * n));
    HGB_CUDA(cudaEventRecord(c->ev_out, c->copy));
    HGB_CUDA(cudaStreamWaitEvent(c->stream, c->ev_out, 0));
    hgb_csr *A64 = nullptr, *Ai = nullptr;
    HGB_TRY(hgb_csr_create(c, n, n, nnz, dp, di, dv, HGB_F64, &A64));
    int st = hgb_csr_create(c, n, n, nnz, dp, di, dw, HGB_F32, &Ai);
    if (!st) st = solve(A64, Ai, db, dx);
    hgb_csr_destroy(A64);
    hgb_csr_destroy(Ai);
    if (info) info->kernel_launches += 1;
    if (st && st != HGB_ERR_NOT_CONVERGED) return st;
    HGB_CUDA(cudaMemcpyAsync(x_h, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    return st;
}

extern "C" int hgb_mixed_ir_pcg_solve(hgb_ctx *c, int n, int nnz, const int *pntr_h, const int *indx_h,
                                      const double *vals_h, hgb_ilu *Mi, const double *b_h, double *x_h,
                                      double tol, double inner_rtol, int max_inner, int max_outer,
                                      hgb_solve_info *info) {
    return mixed_host_solve(c, "mixed_ir_pcg", n, nnz, pntr_h, indx_h, vals_h, Mi, b_h, x_h, info,
                            [&](hgb_csr *A64, hgb_csr *Ai, const double *db, double *dx) {
                                return hgb_ir_pcg_solve(c, A64, Ai, Mi, db, dx, tol, inner_rtol, max_inner, max_outer,
                                                        info);
                            });
}

extern "C" int hgb_mixed_ru_pcg_solve(hgb_ctx *c, int n, int nnz, const int *pntr_h, const int *indx_h,
                                      const double *vals_h, hgb_ilu *Mi, const double *b_h, double *x_h,
                                      double tol, double delta, int max_iter, hgb_solve_info *info) {
    return mixed_host_solve(c, "mixed_ru_pcg", n, nnz, pntr_h, indx_h, vals_h, Mi, b_h, x_h, info,
                            [&](hgb_csr *A64, hgb_csr *Ai, const double *db, double *dx) {
                                return hgb_ru_pcg_solve(c, A64, Ai, Mi, db, dx, tol, delta, max_iter, info);
                            });
}
