// Block-local level-scheduled sparse triangular solve for sm_103a.
//
// Rows are cut, in solve order, into contiguous blocks of R rows; one persistent CTA solves one
// block at a time (blocks handed out by an atomic ticket in solve order, so a CTA only waits on
// blocks already taken by running CTAs).  Inside a block the rows are grouped by LOCAL level
// (levels over the dependencies that stay inside the block): a dependency inside the block is
// read from the block's solution slice in shared memory, a dependency on an earlier block is
// read from global memory, where a not-yet-produced entry holds a signalling-NaN pattern (the
// value is its own ready flag, bounded poll).  A named barrier separates local levels, so most
// dependency hops cost a shared-memory round trip instead of an L2 round trip between SMs.
//
// The per-level data is repacked at analysis time into contiguous chunks (row records, entry
// codes, entry values, diagonal values), streamed into a shared-memory ring by a producer warp
// with TMA bulk copies (cp.async.bulk + mbarrier full/empty pairs) while the consumer warps
// compute.  Entries keep the reference's accumulation order within each row, so results are
// bit-identical to the sequential loops of apply_ilu_array / sparse_trsv_array.
#include "hgb_internal.cuh"
#include "hgb_kernels.cuh"
#include "hgb_bsolve.cuh"

#include <algorithm>
#include <vector>

namespace hgb {

constexpr int kBsStages = 4;
constexpr int kBsConsumers = 128;          // consumer threads (4 warps)
constexpr int kBsThreads = kBsConsumers + 32 + 32 * kBsStages;   // + TMA warp + one prefetch warp per stage
constexpr int kBsCapRows = 128;            // rows per chunk (level piece)
constexpr int kBsCapEnt = 512;             // entries per chunk (padded to 8)

// stage layout: [records | codes | values | diagonal values | prefetched remote values |
//                16-byte chunk descriptor]
template <typename V, typename X>
__host__ __device__ constexpr size_t bs_stage_bytes(size_t dvb) {
    return (size_t)kBsCapRows * 16 + (size_t)kBsCapEnt * 4 + (size_t)kBsCapEnt * sizeof(V) + (size_t)kBsCapRows * dvb +
           (size_t)kBsCapEnt * sizeof(X) + 16;
}

struct BsArgs {
    int nblk;
    const int *blk_chunk;    // [nblk+1] chunk range of each block
    const int4 *chunks;      // {rec_off, nrows, ent_off, nent (padded)}
    const int4 *recs;        // {row, entry offset in chunk, ndeps, smem slot}
    const int *codes;        // >= 0: smem slot of a local dependency; < 0: -(global index + 1)
    const void *vals;        // V
    const void *dvals;       // V or double (pivots)
    int dv_double;           // dvals are FP64 pivots
    int R;                   // rows per block (smem slice)
    int n, lower;            // block b holds rows [row_lo, row_lo + cnt) in both directions
    int mode, unit;
    int *ticket;
    int *err;
    const int *skip;
};

__device__ __forceinline__ void named_bar(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

template <typename V, typename X>
__global__ void __launch_bounds__(kBsThreads, 1)
bsolve_kernel(BsArgs A, X alpha, const X *in, X *out, X *pend_a, X *pend_b) {
    if (A.skip && *A.skip) return;
    extern __shared__ __align__(128) unsigned char smem[];
    const size_t dvb = A.dv_double ? sizeof(double) : sizeof(V);
    const size_t sb = bs_stage_bytes<V, X>(dvb);
    const size_t rv_off = (size_t)kBsCapRows * 16 + (size_t)kBsCapEnt * (4 + sizeof(V)) + (size_t)kBsCapRows * dvb;
    X *xs = (X *)smem;
    unsigned char *ring = smem + (size_t)A.R * sizeof(X);
    __shared__ __align__(8) uint64_t full[kBsStages], ready[kBsStages], empty[kBsStages];
    __shared__ int blk_sh;
    const int tid = threadIdx.x;
    const bool producer = (tid >= kBsConsumers) && (tid < kBsConsumers + 32);
    const bool prefetcher = tid >= kBsConsumers + 32;
    if (tid == 0) {
        for (int s = 0; s < kBsStages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&ready[s], 1);
            mbar_init(&empty[s], 1);
        }
        fence_mbar_init();
    }
    __syncthreads();
    unsigned u0 = 0;   // chunks this CTA has streamed so far (stage / phase bookkeeping)
    for (;;) {
        if (tid == 0) blk_sh = atomicAdd(A.ticket, 1);
        __syncthreads();
        const int b = blk_sh;
        __syncthreads();
        if (b >= A.nblk) break;
        const int c0 = __ldg(A.blk_chunk + b), c1 = __ldg(A.blk_chunk + b + 1);
        if (producer) {
            // descriptors of the next 32 chunks come in one warp-wide load; lane 0 issues the copies
            const int lane = tid & 31;
            for (int cb = c0; cb < c1; cb += 32) {
                int4 mine = make_int4(0, 0, 0, 0);
                if (cb + lane < c1) mine = __ldg(A.chunks + cb + lane);
                const int cnt = min(32, c1 - cb);
                for (int k = 0; k < cnt; k++) {
                    int4 ch;
                    ch.x = __shfl_sync(0xffffffffu, mine.x, k);
                    ch.y = __shfl_sync(0xffffffffu, mine.y, k);
                    ch.z = __shfl_sync(0xffffffffu, mine.z, k);
                    ch.w = __shfl_sync(0xffffffffu, mine.w, k);
                    if (lane == 0) {
                        const unsigned u = u0 + (cb + k - c0);
                        const int s = u % kBsStages;
                        if (u >= kBsStages) mbar_wait(&empty[s], ((u / kBsStages) - 1) & 1, A.err);
                        unsigned char *st = ring + s * sb;
                        *(int4 *)(st + sb - 16) = ch;     // published by the arrive below
                        const uint32_t br = (uint32_t)ch.y * 16, be = (uint32_t)ch.w;
                        const uint32_t bd = (uint32_t)(((ch.y + 7) & ~7) * dvb);
                        // every chunk has >= 1 row, so the transaction count is never zero
                        mbar_arrive_tx(&full[s], br + be * 4 + be * (uint32_t)sizeof(V) + bd);
                        bulk_g2s(st, A.recs + ch.x, br, &full[s]);
                        if (be) {
                            bulk_g2s(st + kBsCapRows * 16, A.codes + ch.z, be * 4, &full[s]);
                            bulk_g2s(st + kBsCapRows * 16 + kBsCapEnt * 4, (const V *)A.vals + ch.z, be * sizeof(V), &full[s]);
                        }
                        bulk_g2s(st + kBsCapRows * 16 + kBsCapEnt * (4 + sizeof(V)),
                                 (const unsigned char *)A.dvals + (size_t)ch.x * dvb, bd, &full[s]);
                    }
                }
            }
        } else if (prefetcher) {
            // warp w owns ring stage w: once the stage's chunk has landed, load the chunk's
            // dependencies on earlier blocks from L2 (16 loads in flight per lane) into the
            // stage, then release it to the consumers.  Values still pending are re-polled there.
            const int w = (tid - kBsConsumers - 32) >> 5, lane = tid & 31;
            for (int c = c0; c < c1; c++) {
                const unsigned u = u0 + (c - c0);
                if ((int)(u % kBsStages) != w) continue;
                mbar_wait(&full[w], (u / kBsStages) & 1, A.err);
                unsigned char *st = ring + w * sb;
                const int4 ch = *(const int4 *)(st + sb - 16);
                const int *code = (const int *)(st + kBsCapRows * 16);
                X *rv = (X *)(st + rv_off);
                X v[kBsCapEnt / 32];
#pragma unroll
                for (int q = 0; q < kBsCapEnt / 32; q++) {
                    const int e = lane + 32 * q;
                    if (e < ch.w) {
                        const int cd = code[e];
                        if (cd < 0) v[q] = ld_relaxed(out + (-cd - 1));
                    }
                }
#pragma unroll
                for (int q = 0; q < kBsCapEnt / 32; q++) {
                    const int e = lane + 32 * q;
                    if (e < ch.w && code[e] < 0) rv[e] = v[q];
                }
                __threadfence_block();
                __syncwarp();
                if (lane == 0) mbar_arrive(&ready[w]);
            }
        } else {
            // the block's right-hand side into its shared solution slice (slot = row - row_lo);
            // a row reads its own slot before overwriting it, dependencies read finished slots
            const int cnt_rows = min(A.R, A.n - b * A.R);
            const int row_lo = A.lower ? b * A.R : A.n - b * A.R - cnt_rows;
#pragma unroll 4
            for (int i = tid; i < cnt_rows; i += kBsConsumers) xs[i] = in[row_lo + i];
            named_bar(1, kBsConsumers);
            for (int c = c0; c < c1; c++) {
                const unsigned u = u0 + (c - c0);
                const int s = u % kBsStages;
                mbar_wait(&ready[s], (u / kBsStages) & 1, A.err);
                const unsigned char *st = ring + s * sb;
                const int4 ch = *(const int4 *)(st + sb - 16);
                const X *rv = (const X *)(st + rv_off);
                const int4 *rec = (const int4 *)st;
                const int *code = (const int *)(st + kBsCapRows * 16);
                const V *val = (const V *)(st + kBsCapRows * 16 + kBsCapEnt * 4);
                const unsigned char *dv = st + kBsCapRows * 16 + kBsCapEnt * (4 + sizeof(V));
                for (int t = tid; t < ch.y; t += kBsConsumers) {
                    const int4 r = rec[t];
                    const X xin = xs[r.w];
                    X acc = (A.mode == 0) ? xin : X(0);
                    for (int k0 = 0; k0 < r.z; k0 += 8) {
                        const int cnt = min(8, r.z - k0);
                        int jj[8];
                        X vv[8], xv[8];
                        unsigned remote = 0;
#pragma unroll
                        for (int k = 0; k < 8; k++)
                            if (k < cnt) {
                                const int cd = code[r.y + k0 + k];
                                vv[k] = Val<V>::get(val[r.y + k0 + k]);
                                if (cd >= 0) {
                                    xv[k] = xs[cd];
                                    jj[k] = 0;
                                } else {
                                    xv[k] = rv[r.y + k0 + k];      // prefetched; pending -> re-poll
                                    jj[k] = -cd - 1;
                                    if (Pending<X>::is(xv[k])) remote |= 1u << k;
                                }
                            }
                        if (remote) {
                            // poll the remote dependencies together (one L2 round trip when ready)
                            int spins = 0;
#pragma unroll
                            for (int k = 0; k < 8; k++)
                                if (remote & (1u << k)) {
                                    xv[k] = ld_relaxed(out + jj[k]);
                                    if (!Pending<X>::is(xv[k])) remote &= ~(1u << k);
                                }
                            while (remote) {
                                if (++spins > kSpinLimit) {
                                    atomicOr(A.err, DEV_ERR_TIMEOUT);
#pragma unroll
                                    for (int k = 0; k < 8; k++)
                                        if (remote & (1u << k)) xv[k] = Pending<X>::canon(Pending<X>::value());
                                    break;
                                }
#pragma unroll
                                for (int k = 0; k < 8; k++)
                                    if (remote & (1u << k)) {
                                        xv[k] = ld_relaxed(out + jj[k]);
                                        if (!Pending<X>::is(xv[k])) remote &= ~(1u << k);
                                    }
                            }
                        }
#pragma unroll
                        for (int k = 0; k < 8; k++)
                            if (k < cnt) {
                                if (A.mode == 0) acc = sub_rn(acc, mul_rn(vv[k], xv[k]));
                                else acc = add_rn(acc, mul_rn(vv[k], xv[k]));
                            }
                    }
                    if (A.mode == 1) acc = sub_rn(mul_rn(alpha, xin), acc);
                    if (!A.unit) {
                        // mixed stores: the FP64 pivot division as one FP64 multiply by the pivot's
                        // FP64 reciprocal (the slow FP64 divide stays out of the sweep)
                        if (A.dv_double) acc = (X)__dmul_rn((double)acc, ((const double *)dv)[t]);
                        else acc = div_rn(acc, Val<V>::get(((const V *)dv)[t]));
                    }
                    acc = Pending<X>::canon(acc);
                    xs[r.w] = acc;
                    st_relaxed(out + r.x, acc);
                    if (pend_a) pend_a[r.x] = Pending<X>::value();
                    if (pend_b) pend_b[r.x] = Pending<X>::value();
                }
                named_bar(1, kBsConsumers);     // this level is complete in shared memory
                if (tid == 0) mbar_arrive(&empty[s]);
            }
        }
        u0 += (unsigned)(c1 - c0);
        __syncthreads();
    }
    // drain: the producer issued nothing beyond the consumed chunks; last CTA resets the ticket
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(A.ticket + 1, 1) == (int)gridDim.x - 1) {
            A.ticket[0] = 0;
            A.ticket[1] = 0;
        }
    }
}

template <typename V>
__global__ void bs_gather_kernel(long n, const int *__restrict__ map, const V *__restrict__ src, V *__restrict__ dst) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        int m = map[i];
        dst[i] = (m >= 0) ? src[m] : V(0);
    }
}

__global__ void bs_gather_piv_kernel(long n, const int *__restrict__ rowmap, const double *__restrict__ piv,
                                     double *__restrict__ dst) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        int r = rowmap[i];
        dst[i] = (r >= 0) ? 1.0 / piv[r] : 1.0;   // FP64 reciprocal of the FP64 pivot
    }
}

void BlockSolve::release() {
    cudaFree(blk_chunk);
    cudaFree(chunks);
    cudaFree(recs);
    cudaFree(codes);
    cudaFree(vals);
    cudaFree(dvals);
    cudaFree(ticket);
    cudaFree(ent_map);
    cudaFree(dv_map);
    cudaFree(dv_row);
    *this = BlockSolve();
}

// Host-side analysis: blocks, local levels, chunks and the packed arrays (structure only; the
// values are gathered on the device through ent_map / dv_map).
int bsolve_analyse(hgb_ctx *c, int n, int nnz, const int *pntr_d, const int *indx_d, const int *diag_d, int lower,
                   int rev, int R, BlockSolve &S) {
    std::vector<int> pntr(n + 1), indx(std::max(nnz, 1)), diag(n);
    HGB_CUDA(cudaMemcpyAsync(pntr.data(), pntr_d, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaMemcpyAsync(indx.data(), indx_d, sizeof(int) * nnz, cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaMemcpyAsync(diag.data(), diag_d, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    const int nblk = (n + R - 1) / R;
    std::vector<int> blk_chunk(1, 0);
    std::vector<int4> chunks;
    std::vector<int4> recs;
    std::vector<int> codes, ent_map, dv_map, dv_row;
    std::vector<int> lev(R), cnt, order;
    auto row_of = [&](int pos) { return lower ? pos : n - 1 - pos; };
    auto pos_of = [&](int row) { return lower ? row : n - 1 - row; };
    for (int b = 0; b < nblk; b++) {
        const int p0 = b * R, p1 = std::min(n, p0 + R);
        const int row_lo = lower ? p0 : n - p1;     // the block's rows are [row_lo, row_lo + p1 - p0)
        int maxlev = 0;
        for (int pos = p0; pos < p1; pos++) {
            const int row = row_of(pos);
            const int a = lower ? pntr[row] : diag[row] + 1;
            const int e = lower ? diag[row] : pntr[row + 1];
            if (e - a > kBsCapEnt) return fail(HGB_ERR_UNSUPPORTED, "row %d has %d dependencies", row, e - a);
            int lv = 0;
            for (int q = a; q < e; q++) {
                const int pj = pos_of(indx[q]);
                if (pj >= p0) lv = std::max(lv, lev[pj - p0] + 1);
            }
            lev[pos - p0] = lv;
            maxlev = std::max(maxlev, lv);
        }
        cnt.assign(maxlev + 2, 0);
        for (int pos = p0; pos < p1; pos++) cnt[lev[pos - p0] + 1]++;
        for (int l = 0; l <= maxlev; l++) cnt[l + 1] += cnt[l];
        order.assign(p1 - p0, 0);
        {
            std::vector<int> cur(cnt.begin(), cnt.end() - 1);
            for (int pos = p0; pos < p1; pos++) order[cur[lev[pos - p0]]++] = pos;
        }
        for (int l = 0; l <= maxlev; l++) {
            int k = cnt[l];
            while (k < cnt[l + 1]) {
                // one chunk: rows of level l while they fit the stage
                const int rec0 = (int)recs.size(), ent0 = (int)codes.size();
                int nr = 0, ne = 0;
                while (k < cnt[l + 1] && nr < kBsCapRows) {
                    const int pos = order[k];
                    const int row = row_of(pos);
                    const int a = lower ? pntr[row] : diag[row] + 1;
                    const int e = lower ? diag[row] : pntr[row + 1];
                    if (ne + (e - a) > kBsCapEnt) break;
                    recs.push_back(make_int4(row, ne, e - a, row - row_lo));
                    for (int q = 0; q < e - a; q++) {
                        const int p = rev ? e - 1 - q : a + q;
                        const int pj = pos_of(indx[p]);
                        codes.push_back(pj >= p0 ? indx[p] - row_lo : -(indx[p] + 1));
                        ent_map.push_back(p);
                    }
                    dv_map.push_back(diag[row]);
                    dv_row.push_back(row);
                    ne += e - a;
                    nr++;
                    k++;
                }
                // pad entries and diagonal values to 16-byte multiples for the bulk copies
                while (codes.size() % 8) { codes.push_back(0); ent_map.push_back(-1); }
                while (dv_map.size() % 8) { dv_map.push_back(-1); dv_row.push_back(-1); }
                while (recs.size() % 8) recs.push_back(make_int4(0, 0, 0, 0));
                chunks.push_back(make_int4(rec0, nr, ent0, (int)codes.size() - ent0));
            }
        }
        blk_chunk.push_back((int)chunks.size());
    }
    S.n = n;
    S.lower = lower;
    S.nblk = nblk;
    S.R = R;
    S.nchunks = (int)chunks.size();
    S.nrec = (int)recs.size();
    S.nent = (int)codes.size();
    HGB_CUDA(cudaMalloc(&S.blk_chunk, sizeof(int) * blk_chunk.size()));
    HGB_CUDA(cudaMalloc(&S.chunks, sizeof(int4) * chunks.size()));
    HGB_CUDA(cudaMalloc(&S.recs, sizeof(int4) * recs.size()));
    HGB_CUDA(cudaMalloc(&S.codes, sizeof(int) * std::max<size_t>(codes.size(), 8)));
    HGB_CUDA(cudaMalloc(&S.ent_map, sizeof(int) * std::max<size_t>(ent_map.size(), 8)));
    HGB_CUDA(cudaMalloc(&S.dv_map, sizeof(int) * dv_map.size()));
    HGB_CUDA(cudaMalloc(&S.dv_row, sizeof(int) * dv_row.size()));
    HGB_CUDA(cudaMalloc(&S.ticket, sizeof(int) * 2));
    HGB_CUDA(cudaMemcpy(S.blk_chunk, blk_chunk.data(), sizeof(int) * blk_chunk.size(), cudaMemcpyHostToDevice));
    HGB_CUDA(cudaMemcpy(S.chunks, chunks.data(), sizeof(int4) * chunks.size(), cudaMemcpyHostToDevice));
    HGB_CUDA(cudaMemcpy(S.recs, recs.data(), sizeof(int4) * recs.size(), cudaMemcpyHostToDevice));
    if (!codes.empty()) {
        HGB_CUDA(cudaMemcpy(S.codes, codes.data(), sizeof(int) * codes.size(), cudaMemcpyHostToDevice));
        HGB_CUDA(cudaMemcpy(S.ent_map, ent_map.data(), sizeof(int) * ent_map.size(), cudaMemcpyHostToDevice));
    }
    HGB_CUDA(cudaMemcpy(S.dv_map, dv_map.data(), sizeof(int) * dv_map.size(), cudaMemcpyHostToDevice));
    HGB_CUDA(cudaMemcpy(S.dv_row, dv_row.data(), sizeof(int) * dv_row.size(), cudaMemcpyHostToDevice));
    HGB_CUDA(cudaMemset(S.ticket, 0, sizeof(int) * 2));
    return HGB_OK;
}

// Gather the values (store precision vsize) and diagonal values (or FP64 pivots) into packed order.
int bsolve_load_values(hgb_ctx *c, BlockSolve &S, const void *svals, int vsize, const double *piv) {
    cudaFree(S.vals);
    cudaFree(S.dvals);
    S.vals = S.dvals = nullptr;
    S.vsize = vsize;
    S.dv_double = piv != nullptr;
    HGB_CUDA(cudaMalloc(&S.vals, (size_t)vsize * std::max(S.nent, 8)));
    HGB_CUDA(cudaMalloc(&S.dvals, (size_t)(piv ? 8 : vsize) * std::max(S.nrec, 8)));
    int g = std::max(1, std::min((S.nent + 255) / 256, c->num_sms * 8));
    int gr = std::max(1, std::min((S.nrec + 255) / 256, c->num_sms * 8));
    if (vsize == 8) {
        bs_gather_kernel<double><<<g, 256, 0, c->stream>>>(S.nent, S.ent_map, (const double *)svals, (double *)S.vals);
        bs_gather_kernel<double><<<gr, 256, 0, c->stream>>>(S.nrec, S.dv_map, (const double *)svals, (double *)S.dvals);
    } else if (vsize == 4) {
        bs_gather_kernel<float><<<g, 256, 0, c->stream>>>(S.nent, S.ent_map, (const float *)svals, (float *)S.vals);
        if (!piv) bs_gather_kernel<float><<<gr, 256, 0, c->stream>>>(S.nrec, S.dv_map, (const float *)svals, (float *)S.dvals);
    } else {
        bs_gather_kernel<uint16_t><<<g, 256, 0, c->stream>>>(S.nent, S.ent_map, (const uint16_t *)svals, (uint16_t *)S.vals);
        if (!piv) bs_gather_kernel<uint16_t><<<gr, 256, 0, c->stream>>>(S.nrec, S.dv_map, (const uint16_t *)svals, (uint16_t *)S.dvals);
    }
    if (piv) bs_gather_piv_kernel<<<gr, 256, 0, c->stream>>>(S.nrec, S.dv_row, piv, (double *)S.dvals);
    return launch_check("bsolve_load_values");
}

template <typename V, typename X>
int bsolve_launch(hgb_ctx *c, const BlockSolve &S, int mode, int unit, X alpha, const X *in, X *out, X *pend_a,
                  X *pend_b, const int *skip) {
    if (S.n == 0) return HGB_OK;
    BsArgs A;
    A.nblk = S.nblk;
    A.blk_chunk = S.blk_chunk;
    A.chunks = S.chunks;
    A.recs = S.recs;
    A.codes = S.codes;
    A.vals = S.vals;
    A.dvals = S.dvals;
    A.dv_double = S.dv_double;
    A.R = S.R;
    A.n = S.n;
    A.lower = S.lower;
    A.mode = mode;
    A.unit = unit;
    A.ticket = S.ticket;
    A.err = c->err;
    A.skip = skip;
    const size_t dvb = S.dv_double ? sizeof(double) : sizeof(V);
    const size_t smem = (size_t)S.R * sizeof(X) + kBsStages * bs_stage_bytes<V, X>(dvb);
    static bool attr[2][3] = {};
    const int xi = sizeof(X) == 8 ? 0 : 1, vi = sizeof(V) == 8 ? 0 : (sizeof(V) == 4 ? 1 : 2);
    if (!attr[xi][vi]) {
        HGB_CUDA(cudaFuncSetAttribute(bsolve_kernel<V, X>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
        attr[xi][vi] = true;
    }
    if (smem > 220 * 1024) return fail(HGB_ERR_UNSUPPORTED, "bsolve: %zu bytes of shared memory", smem);
    const int grid = std::max(1, std::min(S.nblk, c->num_sms));
    bsolve_kernel<V, X><<<grid, kBsThreads, smem, c->stream>>>(A, alpha, in, out, pend_a, pend_b);
    return launch_check("bsolve_kernel");
}

template int bsolve_launch<double, double>(hgb_ctx *, const BlockSolve &, int, int, double, const double *, double *,
                                           double *, double *, const int *);
template int bsolve_launch<float, float>(hgb_ctx *, const BlockSolve &, int, int, float, const float *, float *, float *,
                                         float *, const int *);
template int bsolve_launch<uint16_t, float>(hgb_ctx *, const BlockSolve &, int, int, float, const float *, float *,
                                            float *, float *, const int *);

}  // namespace hgb
