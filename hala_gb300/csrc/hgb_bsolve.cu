// Block-local level-scheduled sparse triangular solve for sm_103a.
//
// Rows are cut, in solve order, into contiguous blocks of at most R rows and kBsStepCap steps.
// One persistent CTA solves one block at a time; blocks are handed out by an atomic ticket in
// solve order, so a CTA only waits on blocks already taken by running CTAs.  Inside a block the
// rows are grouped by LOCAL level (levels over the dependencies that stay inside the block) and
// each level is cut into steps of at most 128 rows.  A dependency inside the block is read from
// the block's solution slice in shared memory.  A dependency on an earlier block is read from
// global memory, where a not-yet-produced entry holds a signalling-NaN pattern: the value is its
// own ready flag (bounded polls).
//
// The CTA has two roles.  128 solver threads take one row each per step.  Every solver thread
// streams its own row packets (three dependency codes and the row's slot, then the values and
// diagonal terms, 16-byte pieces) up to D steps ahead into a private shared-memory ring with
// cp.async, half a ring per commit group, so no handshake between warps sits on that path; a
// named barrier ends each level.  Three (FP64) or four (FP32) fetcher warps take the coming steps
// in turn: a warp polls one value of its step in L2 until it is produced, then loads the first
// dependency on an earlier block of
// every row of the step (re-polling the few not yet produced) and deposits each value in a
// shared-memory ring.  A solver thread therefore waits on shared memory, not on an L2 round trip,
// when it needs a value from the block before.  The
// launch groups the CTAs into thread-block clusters that take consecutive blocks: inside a
// cluster, the CTA of block b also offers each value that block b+1 needs first straight to the
// ring of block b+1's CTA (a store in distributed shared memory), so most hops between blocks
// skip the L2 round trip.  A ring entry is taken only by the step it was deposited for (FP64: a
// NaN pattern tagged with the awaited step, replaced by compare-and-swap; FP32: the value with its
// step beside it), so an offer that comes too early or too late is dropped or ignored and the
// fetchers deliver the value instead: the offers never wait and never decide correctness.  Entries
// keep the reference's accumulation order within each row, so results are bit-identical to the
// sequential loops of apply_ilu_array / sparse_trsv_array (sparse/hala_sparse_utils.hpp).
#include "hgb_internal.cuh"
#include "hgb_kernels.cuh"
#include "hgb_bsolve.cuh"

#include <algorithm>
#include <climits>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace hgb {

// Solver threads per CTA (NT, one row per thread per step).  The kernel is written for any
// multiple of 32; 128 is the one built.  256 threads over 32768-row FP32 blocks (two planes of a
// 128^3 wavefront per block, half as many hops) measured slower on GB300: 0.45 against 0.40 ms
// per ILU(0) application at 128^3 and 0.40 against 0.27 ms at 96^3, the longer steps of the wider
// CTA costing more than the hops saved.
constexpr int kBsThreads = 128;
// Fetcher warps (the remote dependencies of the coming steps): four for FP32 solutions, three for
// FP64 (measured at 128^3: FP32 mixed solve 71.0 ms with four, 75.7 with three, 90.2 with two,
// slower again with eight; FP64 solve 122.6 ms with three against 125.3 with four).
template <typename X> __host__ __device__ constexpr int bs_fetch_warps() { return sizeof(X) == 8 ? 3 : 4; }
template <typename X, int NT> __host__ __device__ constexpr int bs_cta() { return NT + 32 * bs_fetch_warps<X>(); }
constexpr int kBsF = 32;          // steps in the remote-value ring
using RingE = unsigned long long; // remote-ring entry (see Ring)
// Cycles a solver thread waits on its ring entry before reading the value from L2 itself.  The
// fetchers deliver every value anyway; a direct read only competes with them.  128^3 (mixed /
// FP64 solve, ms): 1500 cycles 81.5 / 133.6, 3000 70.9 / 122.5, 6000 68.6 / 115.1-116.1,
// 12000 68.1 / 114.7, 30000 67.8 / 114.7.
constexpr long long kBsDirectAfter = 30000;
constexpr int kBsStepCap = 1024;  // steps per block: the block's descriptors sit in shared memory
constexpr int kBsInline = 3;      // dependencies carried in a row packet; more go to the overflow arrays

// value pieces per packet (NV) and packet-ring depth in steps (bs_depth, a power of two; the FP64
// slice leaves room for 4)
template <typename V> struct BsCfg;
template <> struct BsCfg<double> { static constexpr int NV = 3; };
template <> struct BsCfg<float> { static constexpr int NV = 2; };
template <> struct BsCfg<uint16_t> { static constexpr int NV = 1; };
template <typename V, int NT> __host__ __device__ constexpr int bs_depth() {
    return (sizeof(V) == 8 || NT > kBsThreads) ? 4 : 8;
}

// the packet word (piece 0 .w): bits 0-14 the row's slot in the block, bits 15-30 its number of
// dependencies (kBsIdle: no row for this thread in this step), bit 31 set on the last step of a
// level (a barrier follows)
constexpr int kBsIdle = 0xFFFF;
__host__ __device__ constexpr int bs_word(int slot, int nd, int bar) {
    return (int)((unsigned)slot | ((unsigned)nd << 15) | ((unsigned)bar << 31));
}

inline int bs_nv(int vsize) { return vsize == 8 ? 3 : (vsize == 4 ? 2 : 1); }
constexpr int kBsMaxCluster = 16;  // largest thread-block cluster (above 8: non-portable sizes)

// shared memory: [packet ring D x (1 + NV) x NT pieces | step descriptors |
//                 remote-value ring kBsF x NT entries | solution slice + zero slot]
template <typename V, typename X, int NT>
constexpr size_t bs_smem_bytes(int R) {
    return (size_t)bs_depth<V, NT>() * (1 + BsCfg<V>::NV) * NT * 16 + (size_t)kBsStepCap * 16 +
           (size_t)kBsF * NT * sizeof(RingE) + ((size_t)R + 16 / sizeof(X) + 1) * sizeof(X);
}

// One row's values, unpacked from its value pieces (pieces are NT int4 apart in the ring):
//   FP64 {v0, v1} {v2, RN(1/d)} {d, push, 0};  FP32 {v0, v1, v2, dv} {push, 0, 0, 0};
//   BF16 {v0 | v1 << 16, v2, dv, push}
// dv is the FP32 diagonal (divided by) or the FP32 reciprocal of an FP64 pivot (multiplied by).
// push: where the row's value goes in the next block's remote ring (consumer step << 8 | thread),
// or -1.
template <typename V> struct BsRow;
template <> struct BsRow<double> {
    double v[3], d, dinv;
    int push;
    template <int NT> __device__ __forceinline__ void load(const int4 *p) {
        const double2 a = *(const double2 *)p, b = *(const double2 *)(p + NT);
        const int4 c = p[2 * NT];
        v[0] = a.x;
        v[1] = a.y;
        v[2] = b.x;
        dinv = b.y;
        d = __hiloint2double(c.y, c.x);
        push = c.z;
    }
};
template <> struct BsRow<float> {
    float v[3], d;
    int push;
    template <int NT> __device__ __forceinline__ void load(const int4 *p) {
        const float4 a = *(const float4 *)p;
        v[0] = a.x;
        v[1] = a.y;
        v[2] = a.z;
        d = a.w;
        push = p[NT].x;
    }
};
template <> struct BsRow<uint16_t> {
    float v[3], d;
    int push;
    template <int NT> __device__ __forceinline__ void load(const int4 *p) {
        const int4 a = *p;
        v[0] = __uint_as_float((unsigned)a.x << 16);
        v[1] = __uint_as_float((unsigned)a.x & 0xFFFF0000u);
        v[2] = __uint_as_float((unsigned)a.y << 16);
        d = __int_as_float(a.z);
        push = a.w;
    }
};

// a / d correctly rounded, from the stored y = RN(1/d): q0 = RN(a y), r = a - d q0 (exact with
// FMA), q = RN(q0 + r y) equals RN(a / d) (Markstein, IBM J. Res. Dev. 34(1), 1990) when no step
// overflows or underflows.  Operands with |exponent| >= 500, zeros, infinities and NaNs take the
// division instead; for such a d the packet stores y = 0.  The guards are integer tests (the FP64
// pipe of sm_103 is slow).
__host__ __device__ constexpr bool bs_markstein_range(unsigned biased_exp) { return biased_exp - 523u < 1000u; }
template <bool RECIP>
__device__ __forceinline__ double bs_divide(double a, const BsRow<double> &r) {
    const unsigned ea = ((unsigned)__double2hiint(a) >> 20) & 0x7FFu;
    if (bs_markstein_range(ea) && __double_as_longlong(r.dinv) != 0) {
        const double q0 = __dmul_rn(a, r.dinv);
        const double rem = __fma_rn(-r.d, q0, a);
        return __fma_rn(rem, r.dinv, q0);
    }
    return __ddiv_rn(a, r.d);
}
template <bool RECIP, typename V>
__device__ __forceinline__ float bs_divide(float a, const BsRow<V> &r) {
    return RECIP ? __fmul_rn(a, r.d) : __fdiv_rn(a, r.d);
}

struct BsArgs {
    int nblk;
    const int4 *blk;      // {first step, end step, row_lo, rows}
    const int4 *desc;     // {first packet, rows, first overflow entry, overflow width | barrier << 16}
    const int4 *pk0;      // {code0, code1, code2, slot | ndeps << 16}; code >= 0: slot, < 0: -(row + 1)
    const int4 *pkv;      // value pieces, piece p of packet i at pkv[p * npk + i]
    const int *rj;        // per packet: global row of its first dependency on an earlier block, or -1
    long npk;
    const int *ovf_codes;   // dependency k >= 3 of row t of a step: [first + (k - 3) * rows + t]
    const void *ovf_vals;
    int R;                  // rows per block; slot R of the solution slice holds 0 (padding code)
    int cl;                 // CTAs per cluster the packets' push targets were planned for
    int *ticket;
    int *err;
    const int *skip;
};

// Asynchronous-copy issue without a compiler memory clobber: the ring slots it writes are read
// only after cp_async_wait, which keeps its clobber, so the compiler may schedule the step's
// arithmetic around it.
__device__ __forceinline__ void bs_copy16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src));
}
__device__ __forceinline__ void bs_commit() { asm volatile("cp.async.commit_group;"); }
// Step numbers published between the roles: acquire / release at CTA scope on shared memory.
__device__ __forceinline__ int bs_ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.cta.shared::cta.b32 %0, [%1];" : "=r"(v) : "r"(smem_addr(p)) : "memory");
    return v;
}
__device__ __forceinline__ void bs_st_release(int *p, int v) {
    asm volatile("st.release.cta.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(p)), "r"(v) : "memory");
}
// thread-block cluster: rank, size, barrier over all its threads, peer shared-memory access
__device__ __forceinline__ unsigned bs_cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned bs_cluster_size() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void bs_cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t bs_peer(const void *local, unsigned rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_addr(local)), "r"(rank));
    return r;
}
__device__ __forceinline__ void bs_peer_store(uint32_t a, int v) {
    asm volatile("st.shared::cluster.b32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
// a timed-out wait anywhere in the launch ends this one too (checked every 256 polls)
__device__ __forceinline__ bool bs_give_up(int spins, int *err) {
    return spins > kSpinLimit || ((spins & 255) == 0 && (*(volatile int *)err & DEV_ERR_TIMEOUT));
}
constexpr int kBsSpinLimitSleeping = 1 << 22;   // polls with a 128 ns sleep: about half a second

__device__ __forceinline__ unsigned long long bs_peer_cas(uint32_t a, unsigned long long expect, unsigned long long v) {
    unsigned long long old;
    asm volatile("atom.shared::cluster.cas.b64 %0, [%1], %2, %3;" : "=l"(old) : "r"(a), "l"(expect), "l"(v) : "memory");
    return old;
}
// a strong (relaxed, cluster-scope) 64-bit store into a peer's shared memory: the peer polls the
// entry with volatile loads
__device__ __forceinline__ void bs_peer_store64(uint32_t a, unsigned long long v) {
    asm volatile("st.relaxed.cluster.shared::cluster.b64 [%0], %1;" ::"r"(a), "l"(v) : "memory");
}

// Remote-ring entries (64 bits), one per (step mod kBsF, solver thread).  A deposit (a fetched
// value or an offer from the cluster peer) may only be taken by the step it was made for.
//  - FP64: a signalling-NaN pattern tagged with the step the entry awaits (arithmetic never
//    produces signalling NaNs, and solver outputs are canonicalised); a deposit replaces exactly
//    that pattern (compare-and-swap), and the consumer puts the tag of the entry's next use back
//    after reading it.
//  - FP32: the value in the low half and the step it belongs to in the high half, written with one
//    64-bit store; the consumer takes it only when the step matches, so nothing is reset after a
//    read and a deposit needs no compare-and-swap.  A deposit that overwrites an unread older step
//    (an offer more than kBsF steps early) only sends that older step's consumer to read the value
//    from L2 itself.
template <typename X> struct Ring;
template <> struct Ring<double> {
    __device__ static RingE tag(int s) { return 0x7FF4BEEF00000000ull | (unsigned)s; }
    __device__ static RingE init(int q) { return tag(q); }
    __device__ static bool awaits(RingE e, int s) { return e == tag(s); }
    __device__ static bool ready(RingE e, int) { return (e >> 32) != 0x7FF4BEEFull; }
    __device__ static double value(RingE e) { return __longlong_as_double((long long)e); }
    __device__ static void deposit(RingE *slot, int s, double v) {
        atomicCAS(slot, tag(s), (RingE)__double_as_longlong(v));
    }
    __device__ static void consumed(volatile RingE *e, int s) { *e = tag(s + kBsF); }
    __device__ static void offer(uint32_t peer, int ps, double v) {
        bs_peer_cas(peer, tag(ps), (RingE)__double_as_longlong(v));
    }
};
template <> struct Ring<float> {
    __device__ static RingE stamp(int s, float v) { return ((RingE)(unsigned)s << 32) | __float_as_uint(v); }
    __device__ static RingE init(int) { return ~0ull; }
    __device__ static bool awaits(RingE e, int s) { return (unsigned)(e >> 32) != (unsigned)s; }
    __device__ static bool ready(RingE e, int s) { return (unsigned)(e >> 32) == (unsigned)s; }
    __device__ static float value(RingE e) { return __uint_as_float((unsigned)e); }
    __device__ static void deposit(RingE *slot, int s, float v) { *(volatile RingE *)slot = stamp(s, v); }
    __device__ static void consumed(volatile RingE *, int) {}
    __device__ static void offer(uint32_t peer, int ps, float v) { bs_peer_store64(peer, stamp(ps, v)); }
};

// MODE 0: x_i = (b_i - sum_k v_k x_k) [/ d_i]  (apply_ilu_array's order);
// MODE 1: x_i = (alpha b_i - (sum_k v_k x_k)) [/ d_i]  (sparse_trsv_array's order).
// UNIT: no division; RECIP: multiply by the stored FP32 reciprocal instead of dividing.
template <typename V, typename X, int MODE, bool UNIT, bool RECIP, int NT>
__global__ void __launch_bounds__(bs_cta<X, NT>(), 1)
bsolve_kernel(BsArgs A, X alpha, const X *in, X *out, X *pend) {
    constexpr int NV = BsCfg<V>::NV, D = bs_depth<V, NT>(), NP = 1 + NV;
    constexpr int CTA = bs_cta<X, NT>(), RPL = NT / 32;   // fetcher rows per lane
    constexpr int FW = bs_fetch_warps<X>();
    static_assert(NT % 32 == 0 && NT <= 256, "solver threads");
    static_assert((D & (D - 1)) == 0 && D >= 2, "ring shape");
    static_assert((kBsF & (kBsF - 1)) == 0 && kBsF >= 2 * FW, "remote ring shape");
    if (A.skip && *A.skip) return;
    extern __shared__ __align__(128) unsigned char smem[];
    int4 *ring = (int4 *)smem;                          // [D][NP][NT]
    int4 *sdesc = ring + D * NP * NT;                   // [kBsStepCap]
    RingE *rbuf = (RingE *)(sdesc + kBsStepCap);        // [kBsF][NT] remote values
    X *xsbuf = (X *)(rbuf + kBsF * NT);                 // [R + 16 / sizeof(X) + 1]
    __shared__ int blk_sh, done_step;                   // done_step: solver threads finished steps <= it
    const int t = threadIdx.x;
    const unsigned rank = bs_cluster_rank(), ncl = bs_cluster_size();
    if ((int)ncl != A.cl) {   // the push targets assume clusters of A.cl CTAs
        if (t == 0) atomicOr(A.err, DEV_ERR_CSR);
        return;
    }
    const bool solver = t < NT;
    int4 *myring = ring + t;                            // solver thread's piece 0 of ring slot 0
    volatile RingE *vrbuf = rbuf;
    for (;;) {
        // clusters take tickets; rank r of the cluster with ticket q solves block q * ncl + r.  The
        // cluster barriers: every CTA of the cluster is done with the previous round (including its
        // writes into its peers' rings), then the new ticket and the reset rings are visible
        bs_cluster_sync();
        if (t == 0 && rank == 0) {
            const int q = atomicAdd(A.ticket, 1);
            for (unsigned r = 0; r < ncl; r++) bs_peer_store(bs_peer(&blk_sh, r), q);
        }
        if (t == 0) done_step = -1;
        for (int i = t; i < kBsF * NT; i += CTA) rbuf[i] = Ring<X>::init(i / NT);
        bs_cluster_sync();
        const int q = blk_sh;
        if (q * (int)ncl >= A.nblk) break;   // the same for the whole cluster
        const int b = q * (int)ncl + (int)rank;
        if (b >= A.nblk) continue;            // the last cluster may have spare ranks
        const int4 bi = __ldg(A.blk + b);
        const int ns = bi.y - bi.x, row_lo = bi.z, cnt = bi.w;

        // the block's step descriptors and its right-hand side slice, in one commit group
        for (int i = t; i < ns; i += CTA) bs_copy16(sdesc + i, A.desc + bi.x + i);
        constexpr int E = 16 / (int)sizeof(X);
        const X *src = in + row_lo;
        const int mis = (int)(((size_t)src & 15) / sizeof(X));
        X *xs = xsbuf + mis;   // xs[i] and src[i] sit at the same offset modulo 16 bytes
        const int head = min(cnt, (E - mis) % E);
        const int body = (cnt - head) / E;
        for (int i = t; i < body; i += CTA) bs_copy16(xs + head + i * E, src + head + i * E);
        for (int i = head + body * E + t; i < cnt; i += CTA) xs[i] = src[i];
        if (t < head) xs[t] = src[t];
        if (t == 0) xs[A.R] = X(0);
        bs_commit();
        cp_async_wait<0>();
        __syncthreads();

        if (!solver) {
            // ---- fetcher warps: warp w takes steps w, w+FW, w+2FW, ... one at a time, polling the
            // step's remote values (RPL rows per lane) until all are deposited; the remote rows of
            // its next step are loaded meanwhile
            const int w = (t - NT) >> 5, l = t & 31;
            int jq[RPL], jn[RPL];
            auto load_rj = [&](int s, int (&jr)[RPL]) {
                const int4 d = (s < ns) ? sdesc[s] : make_int4(0, 0, 0, 0);
#pragma unroll
                for (int q = 0; q < RPL; q++) {
                    const int r = l + 32 * q;
                    jr[q] = (r < d.y) ? __ldg(A.rj + d.x + r) : -1;
                }
            };
            load_rj(w, jq);
            // The buffer passed as pend (the next launch's output, or this launch's input once its
            // slice is in shared memory; nothing in this launch reads it) goes back to the pending
            // pattern in the fetcher warps, off the solver threads' steps (a store per row in each
            // step cost the FP32 sweeps 8 %).  FP64 spreads it over the fetchers' steps, FP32 writes
            // it after them: each measured faster for its type (the FP64 slice in one burst beside the
            // solver threads' last steps cost 2 %).
            constexpr bool kPendSpread = sizeof(X) == 8;
            const int pchunk = ns > 0 ? (cnt + ns - 1) / ns : 0;   // rows per step (kPendSpread)
            for (int s = w; s < ns; s += FW) {
                load_rj(s + FW, jn);
                // the ring slot of step s was last used by step s - kBsF (the solver threads reset
                // each entry to the pending pattern after reading it)
                int spins = 0;
                while (bs_ld_acquire(&done_step) < s - kBsF) {   // sleeping: the solver threads share the LSU
                    if (bs_give_up(++spins, A.err) || spins > kBsSpinLimitSleeping) {
                        atomicOr(A.err, DEV_ERR_TIMEOUT);
                        break;
                    }
                    __nanosleep(128);
                }
                RingE *slot = rbuf + (s & (kBsF - 1)) * NT + l;
                volatile RingE *vslot = slot;
                unsigned todo = 0;
#pragma unroll
                for (int q = 0; q < RPL; q++)   // rows whose value the block before has not offered yet
                    if (jq[q] >= 0 && Ring<X>::awaits(vslot[32 * q], s)) todo |= 1u << q;
                spins = 0;
                // one lane polls a single value of the step until it is produced, then the warp
                // loads them all: one L2 load per round instead of one per row keeps the memory
                // pipeline, which the solver threads' shared-memory accesses go through, free
                const unsigned lanes = __ballot_sync(0xFFFFFFFFu, todo != 0);
                if (lanes && l == __ffs(lanes) - 1) {
                    const int q0 = __ffs(todo) - 1;
                    int jrep = jq[0];
#pragma unroll
                    for (int q = 1; q < RPL; q++)
                        if (q == q0) jrep = jq[q];
                    while (Pending<X>::is(ld_relaxed(out + jrep))) {
                        if (bs_give_up(++spins, A.err) || spins > kBsSpinLimitSleeping) break;
                        __nanosleep(32);
                    }
                }
                __syncwarp();
                while (todo) {
                    X v[RPL];
#pragma unroll
                    for (int q = 0; q < RPL; q++)
                        if (todo & (1u << q)) v[q] = ld_relaxed(out + jq[q]);
                    const unsigned before = todo;
#pragma unroll
                    for (int q = 0; q < RPL; q++)
                        if ((todo & (1u << q)) && !Pending<X>::is(v[q])) {
                            Ring<X>::deposit(slot + 32 * q, s, v[q]);
                            todo &= ~(1u << q);
                        }
                    if (!todo) break;
                    if (todo == before) __nanosleep(32);
                    if (bs_give_up(++spins, A.err) || spins > kBsSpinLimitSleeping) {
                        // give up: deposit NaN so that the solver threads terminate too
                        atomicOr(A.err, DEV_ERR_TIMEOUT);
#pragma unroll
                        for (int q = 0; q < RPL; q++)
                            if (todo & (1u << q))
                                Ring<X>::deposit(slot + 32 * q, s, Pending<X>::canon(Pending<X>::value()));
                        todo = 0;
                    }
                }
#pragma unroll
                for (int q = 0; q < RPL; q++) jq[q] = jn[q];
                // FP64: the other buffer's share of this step back to the pending pattern (below)
                if (kPendSpread && pend) {
                    const int r0 = s * pchunk, r1 = min(cnt, r0 + pchunk);
                    for (int i = r0 + l; i < r1; i += 32) pend[row_lo + i] = Pending<X>::value();
                }
            }
            // FP32: the other buffer's whole slice back to the pending pattern at the end of the
            // fetchers' steps, in 16-byte stores
            if (!kPendSpread && pend) {
                X *pb = pend + row_lo;
                const int ft = t - NT, FT = 32 * FW;
                const int pmis = (int)(((size_t)pb & 15) / sizeof(X));
                const int phead = min(cnt, (E - pmis) % E), pbody = (cnt - phead) / E;
                const X pv = Pending<X>::value();
                for (int i = ft; i < phead; i += FT) pb[i] = pv;
                for (int i = ft; i < pbody; i += FT) {
                    X *q = pb + phead + i * E;   // 16-byte aligned
                    if constexpr (sizeof(X) == 4)
                        *(float4 *)q = make_float4(pv, pv, pv, pv);
                    else
                        *(double2 *)q = make_double2(pv, pv);
                }
                for (int i = phead + pbody * E + ft; i < cnt; i += FT) pb[i] = pv;
            }
            continue;   // to the block-end barrier
        }

        // ---- solver threads
        X *outb = out + row_lo;
        // thread t's packets of steps s0 .. s0 + D/2 - 1 into their ring slots s % D, one commit
        // group per half ring (its descriptors read together); without a row in a step the thread
        // writes an idle packet (zero-slot codes, the barrier flag)
        constexpr int HB = D / 2;
        auto issue = [&](int s0) {
            int4 dd[HB];
#pragma unroll
            for (int h = 0; h < HB; h++) dd[h] = (s0 + h < ns) ? sdesc[s0 + h] : make_int4(0, 0, 0, 0);
#pragma unroll
            for (int h = 0; h < HB; h++) {
                const int s = s0 + h;
                if (s < ns) {
                    const int4 d = dd[h];
                    int4 *slot = myring + (s & (D - 1)) * (NP * NT);
                    if (t < d.y) {
                        bs_copy16(slot, A.pk0 + d.x + t);
#pragma unroll
                        for (int p = 0; p < NV; p++)
                            bs_copy16(slot + (1 + p) * NT, A.pkv + (long)p * A.npk + d.x + t);
                    } else {
                        *slot = make_int4(A.R, A.R, A.R, bs_word(0, kBsIdle, (d.w >> 16) & 1));
                    }
                }
            }
            bs_commit();
        };
        // the first remote dependency of this thread's row of step s, once the fetchers' ring
        // entry e showed the pending pattern: wait for the deposit (bounded, then read directly)
        // (an offer that was dropped, or a slow fetcher, costs at most kBsDirectAfter cycles: then
        // the thread reads the value from L2 itself)
        auto remote_wait = [&](volatile RingE *e, int s, int cd) -> X {
            const long long t0 = clock64();
            RingE v = *e;
            while (!Ring<X>::ready(v, s)) {
                if (clock64() - t0 > kBsDirectAfter) return wait_value(out + (-cd - 1), A.err);
                v = *e;
            }
            return Ring<X>::value(v);
        };
        int last_pub = -1;   // thread 0: the last step published to the fetchers
        // the next block's CTA (the next rank of this cluster): its remote ring
        const bool has_next = rank + 1 < ncl && b + 1 < A.nblk;
        const uint32_t next_rbuf = has_next ? bs_peer(rbuf, rank + 1) : 0u;
        issue(0);
        issue(HB);
        for (int s = 0; s < ns; s++) {
            if (s % HB == 0) {   // the half ring of steps s .. s + HB - 1 has landed; refill the other half
                if (s > 0) issue(s + HB);
                cp_async_wait<1>();
            }
            const int4 *slot = myring + (s & (D - 1)) * (NP * NT);
            const int4 p0 = slot[0];
            const int w = p0.w, nd = (w >> 15) & 0xFFFF, sl = w & 0x7FFF;
            BsRow<V> rw;
            rw.template load<NT>(slot + NT);
            const int code[kBsInline] = {p0.x, p0.y, p0.z};
            const X xin = xs[sl];
            // padding entries read the zero slot and the zero value: 0 * 0 leaves the sum unchanged
            X xv[kBsInline];
#pragma unroll
            for (int k = 0; k < kBsInline; k++) xv[k] = xs[max(code[k], 0)];
            // dependencies on earlier blocks: the first one comes from the fetchers' ring (an FP64
            // entry goes back to the pending pattern for its next use, kBsF steps later); any
            // further one is polled directly
            {
                const int k0 = code[0] < 0 ? 0 : (code[1] < 0 ? 1 : (code[2] < 0 ? 2 : -1));
                volatile RingE *e = vrbuf + (s & (kBsF - 1)) * NT + t;
                const RingE ev = *e;
                X rv = Ring<X>::value(ev);
                if (k0 >= 0) {
                    const int c0 = (k0 == 0) ? code[0] : (k0 == 1 ? code[1] : code[2]);
                    if (!Ring<X>::ready(ev, s)) rv = remote_wait(e, s, c0);
                }
                Ring<X>::consumed(e, s);   // FP64: the entry's next use
#pragma unroll
                for (int k = 0; k < kBsInline; k++)
                    if (k == k0) xv[k] = rv;
                if ((code[0] < 0) + (code[1] < 0) + (code[2] < 0) > 1) {
#pragma unroll
                    for (int k = 0; k < kBsInline; k++)
                        if (k > k0 && code[k] < 0) xv[k] = wait_value(out + (-code[k] - 1), A.err);
                }
            }
            X acc = (MODE == 0) ? xin : X(0);
#pragma unroll
            for (int k = 0; k < kBsInline; k++)
                acc = (MODE == 0) ? sub_rn(acc, mul_rn((X)rw.v[k], xv[k])) : add_rn(acc, mul_rn((X)rw.v[k], xv[k]));
            if (nd > kBsInline && nd != kBsIdle) {
                const int4 d = sdesc[s];
                for (int k = kBsInline; k < nd; k++) {
                    const long e = (long)d.z + (long)(k - kBsInline) * d.y + t;
                    const int cd = __ldg(A.ovf_codes + e);
                    const X vk = Val<V>::get(__ldg((const V *)A.ovf_vals + e));
                    const X xk = (cd >= 0) ? xs[cd] : wait_value(out + (-cd - 1), A.err);
                    acc = (MODE == 0) ? sub_rn(acc, mul_rn(vk, xk)) : add_rn(acc, mul_rn(vk, xk));
                }
            }
            if (MODE == 1) acc = sub_rn(mul_rn(alpha, xin), acc);
            if (!UNIT) acc = bs_divide<RECIP>(acc, rw);
            acc = Pending<X>::canon(acc);
            if (nd != kBsIdle) {
                xs[sl] = acc;
                st_relaxed(outb + sl, acc);
                if (rw.push >= 0 && has_next) {
                    // the next block reads this value first: offer it to that CTA's ring (taken only
                    // if the entry awaits exactly that step; the result is not read, which measured
                    // faster than reading it a step later)
                    const int ps = rw.push >> 8, pt = rw.push & 255;
                    Ring<X>::offer(next_rbuf + (uint32_t)(((ps & (kBsF - 1)) * NT + pt) * sizeof(RingE)), ps, acc);
                }
            }
            if (w < 0) {   // end of a level (or of 16 steps of one): publish it to the solver threads, and
                           // to the fetchers when 8 steps have passed (they lag by < 24 < kBsF steps)
                named_bar_sync(1, NT);
                if (t == 0 && s - last_pub >= 8) {
                    bs_st_release(&done_step, s);
                    last_pub = s;
                }
            }
        }
        cp_async_wait<0>();
    }
    // the last CTA to leave resets the ticket for the next launch
    if (t == 0) {
        __threadfence();
        if (atomicAdd(A.ticket + 1, 1) == (int)gridDim.x - 1) {
            A.ticket[0] = 0;
            A.ticket[1] = 0;
        }
    }
}

// value pieces of the packets (layout in BsRow)
template <typename V>
__global__ void bs_pack_kernel(long npk, const int *__restrict__ map3, const int *__restrict__ dv_map,
                               const int *__restrict__ dv_row, const int *__restrict__ push,
                               const V *__restrict__ src, const double *__restrict__ piv, int4 *__restrict__ pkv);

template <>
__global__ void bs_pack_kernel<double>(long npk, const int *__restrict__ map3, const int *__restrict__ dv_map,
                                       const int *__restrict__ dv_row, const int *__restrict__ push,
                                       const double *__restrict__ src, const double *__restrict__ piv,
                                       int4 *__restrict__ pkv) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < npk; i += (long)gridDim.x * blockDim.x) {
        double v[3];
        for (int k = 0; k < 3; k++) {
            const int m = map3[3 * i + k];
            v[k] = m >= 0 ? src[m] : 0.0;
        }
        const int dm = dv_map[i], r = dv_row[i];
        const double d = piv ? piv[r] : (dm >= 0 ? src[dm] : 1.0);
        ((double2 *)pkv)[i] = make_double2(v[0], v[1]);
        const bool fast = bs_markstein_range(((unsigned)__double2hiint(d) >> 20) & 0x7FFu);
        ((double2 *)(pkv + npk))[i] = make_double2(v[2], fast ? 1.0 / d : 0.0);   // correctly rounded reciprocal
        pkv[2 * npk + i] = make_int4(__double2loint(d), __double2hiint(d), push[i], 0);
    }
}

template <>
__global__ void bs_pack_kernel<float>(long npk, const int *__restrict__ map3, const int *__restrict__ dv_map,
                                      const int *__restrict__ dv_row, const int *__restrict__ push,
                                      const float *__restrict__ src, const double *__restrict__ piv,
                                      int4 *__restrict__ pkv) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < npk; i += (long)gridDim.x * blockDim.x) {
        float v[3];
        for (int k = 0; k < 3; k++) {
            const int m = map3[3 * i + k];
            v[k] = m >= 0 ? src[m] : 0.0f;
        }
        const int dm = dv_map[i], r = dv_row[i];
        const float dv = piv ? (float)(1.0 / piv[r]) : (dm >= 0 ? src[dm] : 1.0f);
        ((float4 *)pkv)[i] = make_float4(v[0], v[1], v[2], dv);
        pkv[npk + i] = make_int4(push[i], 0, 0, 0);
    }
}

template <>
__global__ void bs_pack_kernel<uint16_t>(long npk, const int *__restrict__ map3, const int *__restrict__ dv_map,
                                         const int *__restrict__ dv_row, const int *__restrict__ push,
                                         const uint16_t *__restrict__ src, const double *__restrict__ piv,
                                         int4 *__restrict__ pkv) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < npk; i += (long)gridDim.x * blockDim.x) {
        unsigned v[3];
        for (int k = 0; k < 3; k++) {
            const int m = map3[3 * i + k];
            v[k] = m >= 0 ? src[m] : 0u;
        }
        const int dm = dv_map[i], r = dv_row[i];
        const float dv = piv ? (float)(1.0 / piv[r]) : (dm >= 0 ? __uint_as_float((unsigned)src[dm] << 16) : 1.0f);
        pkv[i] = make_int4((int)(v[0] | (v[1] << 16)), (int)v[2], __float_as_int(dv), push[i]);
    }
}

template <typename V>
__global__ void bs_gather_kernel(long n, const int *__restrict__ map, const V *__restrict__ src, V *__restrict__ dst) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int m = map[i];
        dst[i] = (m >= 0) ? src[m] : V(0);
    }
}

void BlockSolve::release() {
    cudaFree(blk);
    cudaFree(desc);
    cudaFree(pk0);
    cudaFree(rj);
    cudaFree(push);
    cudaFree(pkv);
    cudaFree(ovf_codes);
    cudaFree(ovf_vals);
    cudaFree(map3);
    cudaFree(dv_map);
    cudaFree(dv_row);
    cudaFree(ovf_map);
    cudaFree(ticket);
    *this = BlockSolve();
}

// Co-resident thread-block clusters of cl block-solve CTAs (queried once per device and cluster
// size, with the largest shared memory of a block: the FP64 store's).  On GB300 one CTA per SM
// fits, and 15 clusters of 8, 36 of 4 or 76 of 2 are co-resident.
static int bs_clusters_fit(hgb_ctx *c, int cl) {
    static int cache[64][kBsMaxCluster + 1];
    static bool init[64][kBsMaxCluster + 1];
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    if (c->device < 0 || c->device >= 64 || cl < 1 || cl > kBsMaxCluster) return 0;
    if (init[c->device][cl]) return cache[c->device][cl];
    auto fits = [&](auto kernel, size_t smem) {
        if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
            (cl > 8 && cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)) {
            cudaGetLastError();
            return 0;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cl * 16);
        cfg.blockDim = dim3(bs_cta<double, kBsThreads>());
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cl;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, kernel, &cfg) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        return n;
    };
    DeviceGuard g(c->device);
    const int n = fits(bsolve_kernel<double, double, 0, true, false, kBsThreads>,
                       bs_smem_bytes<double, double, kBsThreads>(16384));
    cache[c->device][cl] = n;
    init[c->device][cl] = true;
    return n;
}

// Cluster size.  Every hop between clusters goes through L2 and the fetcher warps, a hop inside a
// cluster through distributed shared memory; and a block whose cluster is not co-resident starts
// only when another cluster has finished all its blocks.  So: the largest size (up to 16, sizes
// above 8 being non-portable) at which the clusters of all nblk blocks are co-resident; failing
// that, the largest of 8, 4, 2 that fits.  On GB300 (one CTA per SM) 15 clusters of 8 are
// co-resident, so for 128 blocks a size between 9 and 16 that still fits 128 CTAs at once removes
// the wait for a free cluster.
static int bs_cluster_plan(hgb_ctx *c, int nblk) {
    if (nblk < 2) return 1;
    for (int cl = std::min(kBsMaxCluster, nblk); cl > 1; cl--)
        if ((long)bs_clusters_fit(c, cl) * cl >= nblk) return cl;
    for (int cl = 8; cl > 1; cl /= 2)
        if (bs_clusters_fit(c, cl) >= 1) return cl;
    return 1;
}

// Rows per block: 16384 (the FP64 slice fills 128 KB).  For natural-ordered grids whose planes
// hold 16384 rows this puts one plane in a block; blocks that cut planes make a block's first
// local levels wait for the previous block's last ones, which serialises the wavefront.
int bsolve_rows(hgb_ctx *c, int xsize, int n) {
    (void)c;
    (void)xsize;
    (void)n;
    return 16384;
}

template <typename T>
static int upload(T **dst, const std::vector<T> &src) {
    HGB_CUDA(cudaMalloc(dst, sizeof(T) * std::max<size_t>(src.size(), 1)));
    if (!src.empty()) HGB_CUDA(cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice));
    return HGB_OK;
}

// The schedule on the host (structure only; the values are gathered on the device through map3 /
// dv_map / dv_row / ovf_map), before its upload.
struct BsPlan {
    int n = 0, R = 0, cl = 1;
    std::vector<int4> blk, desc, pk0;
    std::vector<int> map3, dv_map, dv_row, ovf_codes, ovf_map, rj, push;
};

// Host-side analysis from host arrays: blocks, local levels, steps and the packets.  Pure host
// work apart from the (cached) occupancy query of the cluster plan, so the lower and upper
// schedules can be planned in parallel threads.
static int bsolve_plan(hgb_ctx *c, int n, int nnz, const int *pntr, const int *indx, const int *diag, int lower,
                       int rev, int R, int xsize, BsPlan &P) {
    (void)nnz;
    std::vector<int4> &blk = P.blk, &desc = P.desc, &pk0 = P.pk0;
    std::vector<int> &map3 = P.map3, &dv_map = P.dv_map, &dv_row = P.dv_row, &ovf_codes = P.ovf_codes,
                     &ovf_map = P.ovf_map, &rj = P.rj;
    std::vector<int> lev, cnt, start, cur, order;
    auto row_of = [&](int pos) { return lower ? pos : n - 1 - pos; };
    auto pos_of = [&](int row) { return lower ? row : n - 1 - row; };
    auto deps = [&](int row, int &a, int &e) {
        a = lower ? pntr[row] : diag[row] + 1;
        e = lower ? diag[row] : pntr[row + 1];
    };
    // Blocks hold a whole multiple of the bandwidth (in solve order), so that every dependency
    // reaches at most one block back and block b+1 trails block b by a few steps.  Other sizes
    // break the wavefront: on the 96^3 7-point pattern (bandwidth 9216), 16384-row blocks put the
    // rows that block b+1 needs first at the end of block b's schedule, and the critical path
    // grows from ~380 steps to ~4300.
    int bw = 0;
    for (int row = 0; row < n; row++) {
        int a, e;
        deps(row, a, e);
        if (e > a) bw = std::max(bw, lower ? row - indx[a] : indx[e - 1] - row);
    }
    (void)xsize;
    constexpr int NT = kBsThreads;
    if (bw >= 1 && bw <= R) R = R / bw * bw;
    const int Rmax = R;
    lev.assign(R, 0);
    for (int p0 = 0; p0 < n;) {
        // grow the block in solve order while it fits R rows and kBsStepCap steps
        cnt.clear();
        int steps = 0, p1 = p0;
        while (p1 < n && p1 - p0 < R) {
            int a, e;
            deps(row_of(p1), a, e);
            if (e - a >= kBsIdle) return fail(HGB_ERR_UNSUPPORTED, "row %d has %d dependencies", row_of(p1), e - a);
            int lv = 0;
            for (int q = a; q < e; q++) {
                const int pj = pos_of(indx[q]);
                if (pj >= p0) lv = std::max(lv, lev[pj - p0] + 1);
            }
            if ((int)cnt.size() <= lv) cnt.resize(lv + 1, 0);
            const int add = (cnt[lv] % NT == 0) ? 1 : 0;
            if (steps + add > kBsStepCap) break;
            steps += add;
            cnt[lv]++;
            lev[p1 - p0] = lv;
            p1++;
        }
        const int rows = p1 - p0, row_lo = lower ? p0 : n - p1, nl = (int)cnt.size();
        start.assign(nl + 1, 0);
        for (int l = 0; l < nl; l++) start[l + 1] = start[l] + cnt[l];
        cur.assign(start.begin(), start.end() - 1);
        order.assign(rows, 0);
        for (int pos = p0; pos < p1; pos++) order[cur[lev[pos - p0]]++] = pos;
        const int s_first = (int)desc.size();
        for (int l = 0; l < nl; l++) {
            for (int k = start[l]; k < start[l + 1]; k += NT) {
                const int nr = std::min(NT, start[l + 1] - k);
                int kx = 0;
                for (int i = 0; i < nr; i++) {
                    int a, e;
                    deps(row_of(order[k + i]), a, e);
                    kx = std::max(kx, e - a - kBsInline);
                }
                const size_t ob = ovf_codes.size();
                if (ob + (size_t)kx * nr > (size_t)INT_MAX || pk0.size() + nr > (size_t)INT_MAX)
                    return fail(HGB_ERR_UNSUPPORTED, "block solve: packed arrays exceed 2^31 entries");
                // a barrier ends every level, and every 16th step inside a long level, so that the
                // solver threads' progress reaches the fetchers at least every 16 steps
                const int bar = (k + nr == start[l + 1] || ((k - start[l]) / NT) % 16 == 15) ? 1 : 0;
                desc.push_back(make_int4((int)pk0.size(), nr, (int)ob, kx | (bar << 16)));
                ovf_codes.resize(ob + (size_t)kx * nr, 0);
                ovf_map.resize(ob + (size_t)kx * nr, -1);
                for (int i = 0; i < nr; i++) {
                    const int row = row_of(order[k + i]);
                    int a, e;
                    deps(row, a, e);
                    const int nd = e - a;
                    int cd[kBsInline] = {Rmax, Rmax, Rmax}, mp[kBsInline] = {-1, -1, -1};   // padding: the zero slot
                    for (int q = 0; q < nd; q++) {
                        const int p = rev ? e - 1 - q : a + q;
                        const int col = indx[p];
                        const int code = pos_of(col) >= p0 ? col - row_lo : -(col + 1);
                        if (q < kBsInline) {
                            cd[q] = code;
                            mp[q] = p;
                        } else {
                            ovf_codes[ob + (size_t)(q - kBsInline) * nr + i] = code;
                            ovf_map[ob + (size_t)(q - kBsInline) * nr + i] = p;
                        }
                    }
                    pk0.push_back(make_int4(cd[0], cd[1], cd[2], bs_word(row - row_lo, nd, bar)));
                    int first_remote = -1;
                    for (int q = kBsInline - 1; q >= 0; q--)
                        if (cd[q] < 0) first_remote = -cd[q] - 1;
                    rj.push_back(first_remote);
                    for (int q = 0; q < kBsInline; q++) map3.push_back(mp[q]);
                    dv_map.push_back(diag[row]);
                    dv_row.push_back(row);
                }
            }
        }
        blk.push_back(make_int4(s_first, (int)desc.size(), row_lo, rows));
        p0 = p1;
    }
    // Push targets.  Blocks are grouped in runs of cl (one thread-block cluster each); inside a
    // run, the value that a row of block b+1 needs first from block b is offered by block b's CTA
    // straight to block b+1's ring (consumer step << 8 | consumer thread).  A producer row offers
    // to at most one consumer row.  Offered rows leave the fetchers' lists; an offer that is dropped
    // (the consumer more than a ring's length behind) is read from L2 by the consumer itself.
    const int cl = bs_cluster_plan(c, (int)blk.size());
    std::vector<int> &push = P.push;
    push.assign(pk0.size(), -1);
    if (cl > 1) {
        std::vector<int> pk_of_row(n, -1), blk_of_row(n, -1);
        for (int bb = 0; bb < (int)blk.size(); bb++)
            for (int st = blk[bb].x; st < blk[bb].y; st++)
                for (int t = 0; t < desc[st].y; t++) {
                    const int pkt = desc[st].x + t;
                    const int row = blk[bb].z + (pk0[pkt].w & 0x7FFF);
                    pk_of_row[row] = pkt;
                    blk_of_row[row] = bb;
                }
        for (int bb = 1; bb < (int)blk.size(); bb++) {
            if (bb / cl != (bb - 1) / cl) continue;
            for (int st = blk[bb].x; st < blk[bb].y; st++)
                for (int t = 0; t < desc[st].y; t++) {
                    const int cp = desc[st].x + t, j = rj[cp];
                    if (j < 0 || blk_of_row[j] != bb - 1) continue;
                    const int pp = pk_of_row[j];
                    if (push[pp] < 0) {
                        push[pp] = ((st - blk[bb].x) << 8) | t;
                        rj[cp] = -1;
                    }
                }
        }
    }
    P.n = n;
    P.R = Rmax;
    P.cl = cl;
    return HGB_OK;
}

static int bsolve_upload(const BsPlan &P, BlockSolve &S) {
    S.release();
    S.n = P.n;
    S.nblk = (int)P.blk.size();
    S.nsteps = (int)P.desc.size();
    S.R = P.R;
    S.cl = P.cl;
    S.npk = (long)P.pk0.size();
    S.novf = (long)P.ovf_codes.size();
    HGB_TRY(upload(&S.blk, P.blk));
    HGB_TRY(upload(&S.desc, P.desc));
    HGB_TRY(upload(&S.pk0, P.pk0));
    HGB_TRY(upload(&S.rj, P.rj));
    HGB_TRY(upload(&S.push, P.push));
    HGB_TRY(upload(&S.map3, P.map3));
    HGB_TRY(upload(&S.dv_map, P.dv_map));
    HGB_TRY(upload(&S.dv_row, P.dv_row));
    HGB_TRY(upload(&S.ovf_codes, P.ovf_codes));
    HGB_TRY(upload(&S.ovf_map, P.ovf_map));
    HGB_CUDA(cudaMalloc(&S.ticket, sizeof(int) * 2));
    HGB_CUDA(cudaMemset(S.ticket, 0, sizeof(int) * 2));
    return HGB_OK;
}

int bsolve_analyse(hgb_ctx *c, int n, int nnz, const int *pntr_d, const int *indx_d, const int *diag_d, int lower,
                   int rev, int R, int xsize, BlockSolve &S) {
    std::vector<int> pntr(n + 1), indx(std::max(nnz, 1)), diag(std::max(n, 1));
    HGB_CUDA(cudaMemcpyAsync(pntr.data(), pntr_d, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, c->stream));
    if (nnz > 0)
        HGB_CUDA(cudaMemcpyAsync(indx.data(), indx_d, sizeof(int) * nnz, cudaMemcpyDeviceToHost, c->stream));
    if (n > 0) HGB_CUDA(cudaMemcpyAsync(diag.data(), diag_d, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
    HGB_CUDA(cudaStreamSynchronize(c->stream));
    BsPlan P;
    HGB_TRY(bsolve_plan(c, n, nnz, pntr.data(), indx.data(), diag.data(), lower, rev, R, xsize, P));
    return bsolve_upload(P, S);
}

// The forward (lower, unit) and backward (upper) schedules of one factor from host arrays, planned
// in two host threads; uploaded separately, so the planning can overlap other work.
struct BsPlanPair {
    BsPlan L, U;
};

int bsolve_plan_pair(hgb_ctx *c, int n, int nnz, const int *pntr, const int *indx, const int *diag, int R, int xsize,
                     BsPlanPair **out) {
    *out = nullptr;
    BsPlanPair *P = new BsPlanPair();
    int stU = HGB_OK;
    std::string msgU;
    std::thread tu([&] {
        DeviceGuard g(c->device);
        stU = bsolve_plan(c, n, nnz, pntr, indx, diag, 0, 0, R, xsize, P->U);
        if (stU) msgU = hgb_last_error();   // the message is thread-local
    });
    const int stL = bsolve_plan(c, n, nnz, pntr, indx, diag, 1, 0, R, xsize, P->L);
    tu.join();
    if (stL || stU) {
        delete P;
        return stL ? stL : fail(stU, "%s", msgU.c_str());
    }
    *out = P;
    return HGB_OK;
}

int bsolve_upload_pair(BsPlanPair *P, BlockSolve &SL, BlockSolve &SU) {
    HGB_TRY(bsolve_upload(P->L, SL));
    return bsolve_upload(P->U, SU);
}

void bsolve_plan_pair_free(BsPlanPair *P) { delete P; }

// Gather the values (store precision vsize) and the diagonal terms into the packets.  With piv
// (FP64 pivots of a lower-precision store) the packets carry the pivots' reciprocals.
int bsolve_load_values(hgb_ctx *c, BlockSolve &S, const void *svals, int vsize, const double *piv) {
    cudaFree(S.pkv);
    cudaFree(S.ovf_vals);
    S.pkv = nullptr;
    S.ovf_vals = nullptr;
    S.vsize = vsize;
    S.dv_recip = (piv != nullptr && vsize != 8) ? 1 : 0;
    HGB_CUDA(cudaMalloc(&S.pkv, sizeof(int4) * (size_t)bs_nv(vsize) * std::max<long>(S.npk, 1)));
    HGB_CUDA(cudaMalloc(&S.ovf_vals, (size_t)vsize * std::max<long>(S.novf, 1)));
    const int g = (int)std::max<long>(1, std::min<long>((S.npk + 255) / 256, c->num_sms * 8));
    const int go = (int)std::max<long>(1, std::min<long>((S.novf + 255) / 256, c->num_sms * 8));
    if (vsize == 8) {
        bs_pack_kernel<double><<<g, 256, 0, c->stream>>>(S.npk, S.map3, S.dv_map, S.dv_row, S.push, (const double *)svals, piv, S.pkv);
        if (S.novf) bs_gather_kernel<double><<<go, 256, 0, c->stream>>>(S.novf, S.ovf_map, (const double *)svals, (double *)S.ovf_vals);
    } else if (vsize == 4) {
        bs_pack_kernel<float><<<g, 256, 0, c->stream>>>(S.npk, S.map3, S.dv_map, S.dv_row, S.push, (const float *)svals, piv, S.pkv);
        if (S.novf) bs_gather_kernel<float><<<go, 256, 0, c->stream>>>(S.novf, S.ovf_map, (const float *)svals, (float *)S.ovf_vals);
    } else {
        bs_pack_kernel<uint16_t><<<g, 256, 0, c->stream>>>(S.npk, S.map3, S.dv_map, S.dv_row, S.push, (const uint16_t *)svals, piv, S.pkv);
        if (S.novf)
            bs_gather_kernel<uint16_t><<<go, 256, 0, c->stream>>>(S.novf, S.ovf_map, (const uint16_t *)svals, (uint16_t *)S.ovf_vals);
    }
    return launch_check("bsolve_load_values");
}

template <typename V, typename X, int MODE, bool UNIT, bool RECIP, int NT>
static int bs_launch_nt(hgb_ctx *c, const BlockSolve &S, const BsArgs &A, X alpha, const X *in, X *out, X *pend) {
    constexpr int CTA = bs_cta<X, NT>();
    const size_t smem = bs_smem_bytes<V, X, NT>(S.R);
    // the attribute allows the largest block (16384 rows), so solves with smaller blocks launch too
    const size_t smem_max = bs_smem_bytes<V, X, NT>(16384);
    static int attr_dev = -1;   // device on which the kernel's shared-memory attribute was set
    if (attr_dev != c->device) {
        int mx = 0;
        HGB_CUDA(cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
        if (smem_max > (size_t)mx)
            return fail(HGB_ERR_UNSUPPORTED, "bsolve: %zu bytes of shared memory (max %d)", smem_max, mx);
        HGB_CUDA(cudaFuncSetAttribute(bsolve_kernel<V, X, MODE, UNIT, RECIP, NT>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
        // clusters above 8 CTAs are planned only where the occupancy query accepted them with this
        // attribute set; a refusal here leaves the portable sizes working
        if (cudaFuncSetAttribute(bsolve_kernel<V, X, MODE, UNIT, RECIP, NT>,
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
            cudaGetLastError();
        attr_dev = c->device;
    }
    if (smem > smem_max) return fail(HGB_ERR_UNSUPPORTED, "bsolve: %d rows per block", S.R);
    if (S.cl <= 1) {
        const int grid = std::max(1, std::min(S.nblk, c->num_sms));
        bsolve_kernel<V, X, MODE, UNIT, RECIP, NT><<<grid, CTA, smem, c->stream>>>(A, alpha, in, out, pend);
        return launch_check("bsolve_kernel");
    }
    // thread-block clusters of S.cl CTAs (the push targets were planned for that size); as many
    // clusters as are co-resident with this launch's shared memory, at most one per run of S.cl
    // blocks.  The occupancy query is cached per (device, cluster size, shared memory).
    struct FitKey { int dev, cl; size_t smem; int n; };
    static std::vector<FitKey> fit_cache;
    static std::mutex fit_mu;
    std::lock_guard<std::mutex> lock(fit_mu);
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = S.cl;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(CTA);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = c->stream;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int clusters_max = 0;
    for (const FitKey &k : fit_cache)
        if (k.dev == c->device && k.cl == S.cl && k.smem == smem) clusters_max = k.n;
    if (clusters_max == 0) {
        cfg.gridDim = dim3(S.cl * 16);
        HGB_CUDA(cudaOccupancyMaxActiveClusters(&clusters_max, bsolve_kernel<V, X, MODE, UNIT, RECIP, NT>, &cfg));
        if (clusters_max < 1) return fail(HGB_ERR_UNSUPPORTED, "bsolve: no cluster of %d CTAs fits", S.cl);
        fit_cache.push_back(FitKey{c->device, S.cl, smem, clusters_max});
    }
    const int runs = (S.nblk + S.cl - 1) / S.cl;
    cfg.gridDim = dim3(S.cl * std::max(1, std::min(runs, clusters_max)));
    HGB_CUDA(cudaLaunchKernelEx(&cfg, bsolve_kernel<V, X, MODE, UNIT, RECIP, NT>, A, alpha, in, out, pend));
    return launch_check("bsolve_kernel");
}

template <typename V, typename X, int MODE, bool UNIT, bool RECIP>
static int bs_launch_one(hgb_ctx *c, const BlockSolve &S, const BsArgs &A, X alpha, const X *in, X *out, X *pend) {
    return bs_launch_nt<V, X, MODE, UNIT, RECIP, kBsThreads>(c, S, A, alpha, in, out, pend);
}

template <typename V, typename X>
int bsolve_launch(hgb_ctx *c, const BlockSolve &S, int mode, int unit, X alpha, const X *in, X *out, X *pend,
                  const int *skip) {
    if (S.n == 0) return HGB_OK;
    if (S.R > 16384) return fail(HGB_ERR_ARG, "bsolve: %d rows per block exceed the shared-memory slice", S.R);
    if (S.vsize != (int)sizeof(V) || !S.pkv) return fail(HGB_ERR_ARG, "bsolve: values not loaded for this store");
    BsArgs A;
    A.nblk = S.nblk;
    A.blk = S.blk;
    A.desc = S.desc;
    A.pk0 = S.pk0;
    A.pkv = S.pkv;
    A.rj = S.rj;
    A.npk = S.npk;
    A.ovf_codes = S.ovf_codes;
    A.ovf_vals = S.ovf_vals;
    A.R = S.R;
    A.cl = S.cl;
    A.ticket = S.ticket;
    A.err = c->err;
    A.skip = skip;
    const bool recip = S.dv_recip && sizeof(V) != 8;
    if (mode == 0) {
        if (unit) return bs_launch_one<V, X, 0, true, false>(c, S, A, alpha, in, out, pend);
        return recip ? bs_launch_one<V, X, 0, false, (sizeof(V) != 8)>(c, S, A, alpha, in, out, pend)
                     : bs_launch_one<V, X, 0, false, false>(c, S, A, alpha, in, out, pend);
    }
    if (unit) return bs_launch_one<V, X, 1, true, false>(c, S, A, alpha, in, out, pend);
    return recip ? bs_launch_one<V, X, 1, false, (sizeof(V) != 8)>(c, S, A, alpha, in, out, pend)
                 : bs_launch_one<V, X, 1, false, false>(c, S, A, alpha, in, out, pend);
}

template int bsolve_launch<double, double>(hgb_ctx *, const BlockSolve &, int, int, double, const double *, double *,
                                           double *, const int *);
template int bsolve_launch<float, float>(hgb_ctx *, const BlockSolve &, int, int, float, const float *, float *, float *,
                                         const int *);
template int bsolve_launch<uint16_t, float>(hgb_ctx *, const BlockSolve &, int, int, float, const float *, float *,
                                            float *, const int *);

}  // namespace hgb
