// Batched CG for many independent sparse SPD systems of uneven size, in ONE persistent launch.
//
// The batch is a block-diagonal CSR (global column indices) with system row offsets sys_ptr.
// Work items are handed out by an atomic ticket, largest systems first: a "large" item is one
// system solved by the whole CTA, a "small" item packs up to (threads/32) systems, one per warp,
// each solved with warp-synchronous reductions only.  Per system: FP32 CG on vectors held in
// shared memory (matrix streamed from L2/HBM), FP64 iterative refinement against the FP64
// residual of the FP32-stored matrix, stopping at ||b - A x|| <= rtol ||b|| per system.
// The block size and the warp/CTA threshold are chosen by hgb_batch_autotune, which times the
// candidates on the batch and caches the choice in a small text file.
#include "hgb_internal.cuh"
#include "hgb_kernels.cuh"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace hgb {

constexpr int kBatchSmem = 64 * 1024;    // per CTA: 4 float vectors of up to 4096 rows
constexpr int kBatchUnroll = 4;          // matrix entries whose loads are issued together

struct BatchArgs {
    int nitems;
    const int *item_sys;     // [nitems * wpb] system ids (-1 padding); large items use slot 0
    const int *item_large;   // [nitems]
    const int *sys_ptr;      // [S + 1]
    const int *pntr, *indx;
    const float *vals;
    const double *b;
    double *x;
    int *iters;              // [S] total inner iterations (may be null)
    double *relres;          // [S] final ||b - Ax|| / ||b|| (may be null)
    double rtol, inner_rtol;
    int max_inner, max_outer;
    int *ticket;             // [2] self-resetting
    int *err;
};

struct WarpGroup {
    __device__ int rank() const { return threadIdx.x & 31; }
    __device__ int size() const { return 32; }
    __device__ void sync() const { __syncwarp(); }
    __device__ double sum(double v) const { return warp_sum(v); }
};

struct CtaGroup {
    double *red;   // >= 33 doubles of shared memory
    __device__ int rank() const { return threadIdx.x; }
    __device__ int size() const { return blockDim.x; }
    __device__ void sync() const { __syncthreads(); }
    __device__ double sum(double v) const {
        v = warp_sum(v);
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        if (lane == 0) red[w] = v;
        __syncthreads();
        if (w == 0) {
            double t = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
            t = warp_sum(t);
            if (lane == 0) red[32] = t;
        }
        __syncthreads();
        return red[32];
    }
};

// One system: rows [r0, r0+n) of the batch; sm holds 4 float vectors of n entries.
template <class G>
__device__ void solve_system(const G &g, const BatchArgs &A, int s, float *sm) {
    const int r0 = A.sys_ptr[s], n = A.sys_ptr[s + 1] - r0;
    float *r = sm, *p = sm + n, *q = sm + 2 * n, *d = sm + 3 * n;
    const int t0 = g.rank(), ts = g.size();
    double bb = 0.0;
    for (int i = t0; i < n; i += ts) bb += A.b[r0 + i] * A.b[r0 + i];
    const double bnorm = sqrt(g.sum(bb));
    const double target = A.rtol * bnorm;
    int total = 0;
    double res = 0.0;
    for (int outer = 0;; outer++) {
        // FP64 residual of the stored (FP32) matrix: r = b - A x
        double rr = 0.0;
        for (int i = t0; i < n; i += ts) {
            const int row = r0 + i;
            double acc = A.b[row];
            const int kb = __ldg(A.pntr + row), ke = __ldg(A.pntr + row + 1);
            for (int k = kb; k < ke; k += kBatchUnroll) {
                float vv[kBatchUnroll];
                double xv[kBatchUnroll];
#pragma unroll
                for (int u = 0; u < kBatchUnroll; u++)
                    if (k + u < ke) {
                        vv[u] = __ldg(A.vals + k + u);
                        xv[u] = A.x[__ldg(A.indx + k + u)];
                    }
#pragma unroll
                for (int u = 0; u < kBatchUnroll; u++)
                    if (k + u < ke) acc -= (double)vv[u] * xv[u];
            }
            r[i] = (float)acc;
            d[i] = 0.0f;
            rr += acc * acc;
        }
        res = sqrt(g.sum(rr));
        if (!(res > target) || outer >= A.max_outer || !(res == res)) break;
        // inner FP32 CG on A d = r from d = 0 (solve_cg_core's order, identity preconditioner)
        double rz = 0.0;
        for (int i = t0; i < n; i += ts) {
            p[i] = r[i];
            rz += (double)r[i] * r[i];
        }
        g.sync();
        rz = g.sum(rz);
        const double stop2 = A.inner_rtol * A.inner_rtol * rz;
        for (int it = 0; it < A.max_inner; it++) {
            double pq = 0.0;
            for (int i = t0; i < n; i += ts) {
                const int row = r0 + i;
                const int kb = __ldg(A.pntr + row), ke = __ldg(A.pntr + row + 1);
                float acc = 0.0f;
                // entries kBatchUnroll at a time, their loads issued together (the row's matrix
                // comes from L2: one round trip per group, not per entry); the sum keeps the order
                for (int k = kb; k < ke; k += kBatchUnroll) {
                    float vv[kBatchUnroll];
                    int cc[kBatchUnroll];
#pragma unroll
                    for (int u = 0; u < kBatchUnroll; u++)
                        if (k + u < ke) {
                            vv[u] = __ldg(A.vals + k + u);
                            cc[u] = __ldg(A.indx + k + u);
                        }
#pragma unroll
                    for (int u = 0; u < kBatchUnroll; u++)
                        if (k + u < ke) acc += vv[u] * p[cc[u] - r0];
                }
                q[i] = acc;
                pq += (double)p[i] * acc;
            }
            pq = g.sum(pq);
            const float a = (float)(rz / pq);
            double nr = 0.0;
            for (int i = t0; i < n; i += ts) {
                d[i] += a * p[i];
                float ri = r[i] - a * q[i];
                r[i] = ri;
                nr += (double)ri * ri;
            }
            nr = g.sum(nr);
            total++;
            if (nr < stop2 || !(nr == nr)) break;
            const float beta = (float)(nr / rz);
            for (int i = t0; i < n; i += ts) p[i] = r[i] + beta * p[i];
            rz = nr;
            g.sync();
        }
        for (int i = t0; i < n; i += ts) A.x[r0 + i] += (double)d[i];
        g.sync();
        __threadfence_block();
    }
    if (g.rank() == 0) {
        if (A.iters) A.iters[s] = total;
        if (A.relres) A.relres[s] = bnorm > 0 ? res / bnorm : res;
    }
    g.sync();
}

// every column of a system's rows must fall inside that system (block-diagonal batch)
__global__ void batch_check_kernel(int S, const int *__restrict__ sys_ptr, const int *__restrict__ pntr,
                                   const int *__restrict__ indx, int *err) {
    for (int s = blockIdx.x; s < S; s += gridDim.x) {
        const int r0 = sys_ptr[s], r1 = sys_ptr[s + 1];
        for (int row = r0 + threadIdx.x; row < r1; row += blockDim.x)
            for (int k = pntr[row]; k < pntr[row + 1]; k++) {
                int c = indx[k];
                if (c < r0 || c >= r1) { atomicOr(err, DEV_ERR_CSR); break; }
            }
    }
}

static bool same_args(const BatchArgs &a, const BatchArgs &b) {
    return a.nitems == b.nitems && a.item_sys == b.item_sys && a.item_large == b.item_large &&
           a.sys_ptr == b.sys_ptr && a.pntr == b.pntr && a.indx == b.indx && a.vals == b.vals && a.b == b.b &&
           a.x == b.x && a.iters == b.iters && a.relres == b.relres && a.rtol == b.rtol &&
           a.inner_rtol == b.inner_rtol && a.max_inner == b.max_inner && a.max_outer == b.max_outer &&
           a.ticket == b.ticket && a.err == b.err;
}

__global__ void batch_cg_kernel(BatchArgs A) {
    extern __shared__ __align__(16) float bsm[];
    __shared__ double red[33];
    __shared__ int item;
    const int wpb = blockDim.x >> 5, w = threadIdx.x >> 5;
    for (;;) {
        if (threadIdx.x == 0) item = atomicAdd(A.ticket, 1);
        __syncthreads();
        const int it = item;
        __syncthreads();
        if (it >= A.nitems) break;
        if (A.item_large[it]) {
            CtaGroup g{red};
            solve_system(g, A, A.item_sys[it * wpb], bsm);
        } else {
            const int s = A.item_sys[it * wpb + w];
            if (s >= 0) {
                WarpGroup g;
                const int per_warp = kBatchSmem / (int)sizeof(float) / wpb;
                solve_system(g, A, s, bsm + w * per_warp);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(A.ticket + 1, 1) == (int)gridDim.x - 1) {
            A.ticket[0] = 0;
            A.ticket[1] = 0;
        }
    }
}

}  // namespace hgb

using namespace hgb;

struct hgb_batch {
    hgb_ctx *ctx = nullptr;
    int S = 0, n_total = 0, nnz = 0;
    const int *sys_ptr = nullptr, *pntr = nullptr, *indx = nullptr;
    const float *vals = nullptr;
    std::vector<int> sizes;          // host copy of the system sizes
    hgb_batch_config cfg{256, 256};
    int nitems = 0;
    int *item_sys = nullptr, *item_large = nullptr, *ticket = nullptr;
    // graph of the single launch, keyed by the vectors it was captured with
    cudaGraphExec_t exec = nullptr;
    BatchArgs captured{};
};

namespace hgb {

static int batch_plan(hgb_batch *B, hgb_batch_config cfg) {
    hgb_ctx *c = B->ctx;
    const int wpb = cfg.block_threads / 32;
    const int warp_cap = kBatchSmem / (int)sizeof(float) / wpb / 4;   // rows per warp system
    const int cta_cap = kBatchSmem / (int)sizeof(float) / 4;
    int warp_max = std::min(cfg.warp_max_n, warp_cap);
    std::vector<int> order(B->S);
    for (int s = 0; s < B->S; s++) order[s] = s;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return B->sizes[a] > B->sizes[b]; });
    std::vector<int> isys, ilarge;
    size_t k = 0;
    for (; k < order.size() && B->sizes[order[k]] > warp_max; k++) {
        if (B->sizes[order[k]] > cta_cap) return fail(HGB_ERR_UNSUPPORTED, "batch: system of %d rows > %d", B->sizes[order[k]], cta_cap);
        isys.push_back(order[k]);
        for (int j = 1; j < wpb; j++) isys.push_back(-1);
        ilarge.push_back(1);
    }
    while (k < order.size()) {
        for (int j = 0; j < wpb; j++) isys.push_back(k < order.size() ? order[k++] : -1);
        ilarge.push_back(0);
    }
    cudaFree(B->item_sys);
    cudaFree(B->item_large);
    B->item_sys = B->item_large = nullptr;
    B->nitems = (int)ilarge.size();
    HGB_CUDA(cudaMalloc(&B->item_sys, sizeof(int) * std::max<size_t>(isys.size(), 1)));
    HGB_CUDA(cudaMalloc(&B->item_large, sizeof(int) * std::max<size_t>(ilarge.size(), 1)));
    HGB_CUDA(cudaMemcpy(B->item_sys, isys.data(), sizeof(int) * isys.size(), cudaMemcpyHostToDevice));
    HGB_CUDA(cudaMemcpy(B->item_large, ilarge.data(), sizeof(int) * ilarge.size(), cudaMemcpyHostToDevice));
    B->cfg = cfg;
    if (B->exec) {
        cudaGraphExecDestroy(B->exec);
        B->exec = nullptr;
    }
    (void)c;
    return HGB_OK;
}

static int batch_launch(hgb_batch *B, const BatchArgs &A, cudaStream_t st) {
    hgb_ctx *c = B->ctx;
    int per_sm = 0;
    HGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_cg_kernel, B->cfg.block_threads, kBatchSmem));
    int grid = std::max(1, std::min(B->nitems, c->num_sms * std::max(per_sm, 1)));
    batch_cg_kernel<<<grid, B->cfg.block_threads, kBatchSmem, st>>>(A);
    return launch_check("batch_cg_kernel");
}

static BatchArgs batch_args(hgb_batch *B, const double *b, double *x, double rtol, double inner_rtol, int max_inner,
                            int max_outer, int *iters, double *relres) {
    BatchArgs A{};
    A.nitems = B->nitems;
    A.item_sys = B->item_sys;
    A.item_large = B->item_large;
    A.sys_ptr = B->sys_ptr;
    A.pntr = B->pntr;
    A.indx = B->indx;
    A.vals = B->vals;
    A.b = b;
    A.x = x;
    A.iters = iters;
    A.relres = relres;
    A.rtol = rtol;
    A.inner_rtol = inner_rtol;
    A.max_inner = max_inner;
    A.max_outer = max_outer;
    A.ticket = B->ticket;
    A.err = B->ctx->err;
    return A;
}

}  // namespace hgb

extern "C" {

int hgb_batch_create(hgb_ctx *c, int num_systems, const int *sys_ptr, int n_total, int nnz, const int *pntr,
                     const int *indx, const float *vals, hgb_batch **out) {
    if (!out) return fail(HGB_ERR_ARG, "batch_create: null output");
    *out = nullptr;
    if (!c || num_systems <= 0 || n_total <= 0 || nnz < 0 || !sys_ptr || !pntr || !indx || !vals)
        return fail(HGB_ERR_ARG, "batch_create: bad arguments");
    DeviceGuard g(c->device);
    HGB_TRY(csr_check(c, n_total, n_total, nnz, pntr, indx));
    std::vector<int> sp(num_systems + 1);
    HGB_CUDA(cudaMemcpy(sp.data(), sys_ptr, sizeof(int) * (num_systems + 1), cudaMemcpyDeviceToHost));
    if (sp[0] != 0 || sp[num_systems] != n_total) return fail(HGB_ERR_ARG, "batch_create: sys_ptr must span [0, n_total]");
    hgb_batch *B = new hgb_batch();
    B->ctx = c;
    B->S = num_systems;
    B->n_total = n_total;
    B->nnz = nnz;
    B->sys_ptr = sys_ptr;
    B->pntr = pntr;
    B->indx = indx;
    B->vals = vals;
    B->sizes.resize(num_systems);
    for (int s = 0; s < num_systems; s++) {
        B->sizes[s] = sp[s + 1] - sp[s];
        if (B->sizes[s] <= 0) { delete B; return fail(HGB_ERR_ARG, "batch_create: empty system %d", s); }
    }
    int st = HGB_OK;
    batch_check_kernel<<<std::min(num_systems, c->num_sms * 8), 128, 0, c->stream>>>(num_systems, sys_ptr, pntr, indx, c->err);
    st = collect_dev_error(c);
    if (st) {
        delete B;
        return fail(st, "batch_create: a column falls outside its system's rows");
    }
    if (cudaMalloc(&B->ticket, sizeof(int) * 2) || cudaMemset(B->ticket, 0, sizeof(int) * 2)) st = cuda_fail(cudaGetLastError(), "batch_create");
    if (!st) st = cudaFuncSetAttribute(batch_cg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kBatchSmem) ? HGB_ERR_CUDA : HGB_OK;
    if (!st) st = batch_plan(B, B->cfg);
    if (st) {
        hgb_batch_destroy(B);
        return st;
    }
    *out = B;
    return HGB_OK;
}

int hgb_batch_set_config(hgb_batch *B, const hgb_batch_config *cfg) {
    if (!B || !cfg) return fail(HGB_ERR_ARG, "batch_set_config: bad arguments");
    if (cfg->block_threads != 128 && cfg->block_threads != 256 && cfg->block_threads != 512)
        return fail(HGB_ERR_ARG, "batch: block_threads must be 128, 256 or 512");
    if (cfg->warp_max_n < 0) return fail(HGB_ERR_ARG, "batch: warp_max_n < 0");
    DeviceGuard g(B->ctx->device);
    return batch_plan(B, *cfg);
}

int hgb_batch_get_config(hgb_batch *B, hgb_batch_config *cfg) {
    if (!B || !cfg) return fail(HGB_ERR_ARG, "batch_get_config: bad arguments");
    *cfg = B->cfg;
    return HGB_OK;
}

int hgb_batch_cg_solve(hgb_batch *B, const double *b, double *x, double rtol, double inner_rtol, int max_inner,
                       int max_outer, int *iters, double *relres) {
    if (!B || !b || !x || !(rtol > 0) || !(inner_rtol > 0) || max_inner < 1 || max_outer < 0)
        return fail(HGB_ERR_ARG, "batch_cg_solve: bad arguments");
    hgb_ctx *c = B->ctx;
    DeviceGuard g(c->device);
    BatchArgs A = batch_args(B, b, x, rtol, inner_rtol, max_inner, max_outer, iters, relres);
    // the single persistent launch is captured once into a graph and replayed while the
    // vectors and controls stay the same
    bool same = B->exec && same_args(A, B->captured);
    if (!same) {
        if (B->exec) {
            cudaGraphExecDestroy(B->exec);
            B->exec = nullptr;
        }
        CaptureStream cs(c);
        cudaGraph_t graph = nullptr;
        HGB_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        int st = batch_launch(B, A, c->stream);
        cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
        if (st) return st;
        if (ce != cudaSuccess) return cuda_fail(ce, "batch capture");
        cudaError_t ie = cudaGraphInstantiate(&B->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) return cuda_fail(ie, "batch graph instantiate");
        B->captured = A;
    }
    {
        CaptureStream cs(c);
        HGB_CUDA(cudaGraphLaunch(B->exec, c->stream));
    }
    return collect_dev_error(c);
}

int hgb_batch_autotune(hgb_batch *B, const double *b, double *x, double rtol, const char *cache_path,
                       hgb_batch_config *best) {
    if (!B || !b || !x) return fail(HGB_ERR_ARG, "batch_autotune: bad arguments");
    hgb_ctx *c = B->ctx;
    DeviceGuard g(c->device);
    // signature: number of systems and the size histogram in powers of two
    std::ostringstream sig;
    int hist[16] = {0};
    for (int s : B->sizes) {
        int k = 0;
        while ((1 << (k + 1)) <= s && k < 15) k++;
        hist[k]++;
    }
    sig << "S" << B->S << "_rt" << rtol;
    for (int k = 0; k < 16; k++) if (hist[k]) sig << "_" << k << ":" << hist[k];
    if (cache_path) {
        std::ifstream in(cache_path);
        std::string key;
        int bt, wm;
        while (in >> key >> bt >> wm) {
            if (key == sig.str()) {
                hgb_batch_config cfg{bt, wm};
                HGB_TRY(hgb_batch_set_config(B, &cfg));
                if (best) *best = cfg;
                return HGB_OK;
            }
        }
    }
    const int blocks[] = {128, 256, 512};
    const int warp_max[] = {0, 64, 128, 256, 512};
    double best_ms = 1e30;
    hgb_batch_config bcfg = B->cfg;
    cudaEvent_t e0, e1;
    HGB_CUDA(cudaEventCreate(&e0));
    HGB_CUDA(cudaEventCreate(&e1));
    int st = HGB_OK;
    for (int bt : blocks) {
        for (int wm : warp_max) {
            int cap = kBatchSmem / (int)sizeof(float) / (bt / 32) / 4;
            if (wm > cap) continue;
            hgb_batch_config cfg{bt, wm};
            if ((st = hgb_batch_set_config(B, &cfg))) break;
            float best_here = 1e30f;
            for (int rep = 0; rep < 2 && !st; rep++) {
                if (cudaMemsetAsync(x, 0, sizeof(double) * B->n_total, c->stream)) { st = HGB_ERR_CUDA; break; }
                cudaEventRecord(e0, c->stream);
                st = hgb_batch_cg_solve(B, b, x, rtol, 1e-4, 1000, 20, nullptr, nullptr);
                cudaEventRecord(e1, c->stream);
                cudaEventSynchronize(e1);
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                best_here = std::min(best_here, ms);
            }
            if (st) break;
            if (best_here < best_ms) {
                best_ms = best_here;
                bcfg = cfg;
            }
        }
        if (st) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    HGB_TRY(hgb_batch_set_config(B, &bcfg));
    if (best) *best = bcfg;
    if (cache_path) {
        std::ofstream o(cache_path, std::ios::app);
        o << sig.str() << " " << bcfg.block_threads << " " << bcfg.warp_max_n << "\n";
    }
    return HGB_OK;
}

int hgb_batch_destroy(hgb_batch *B) {
    if (!B) return HGB_OK;
    DeviceGuard g(B->ctx->device);
    if (B->exec) cudaGraphExecDestroy(B->exec);
    cudaFree(B->item_sys);
    cudaFree(B->item_large);
    cudaFree(B->ticket);
    delete B;
    return HGB_OK;
}

}  // extern "C"
