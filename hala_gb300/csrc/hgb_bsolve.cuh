// Block-local level-scheduled triangular solve (hgb_bsolve.cu): analysis data and entry points.
#pragma once

#include "hgb_internal.cuh"

namespace hgb {

struct BlockSolve {
    int n = 0, lower = 1, nblk = 0, nchunks = 0, nrec = 0, nent = 0, R = 0;
    int vsize = 0, dv_double = 0;
    int *blk_chunk = nullptr;   // [nblk+1]
    int4 *chunks = nullptr;     // [nchunks] {rec_off, nrows, ent_off, nent}
    int4 *recs = nullptr;       // [nrec] {row, entry offset in chunk, ndeps, smem slot}
    int *codes = nullptr;       // [nent]
    void *vals = nullptr;       // [nent] store precision
    void *dvals = nullptr;      // [nrec] store precision or FP64 pivots
    int *ent_map = nullptr, *dv_map = nullptr, *dv_row = nullptr;   // value gather maps
    int *ticket = nullptr;
    void release();
};

// rows per block: the block's solution slice (128 KB) lives in shared memory
inline int bsolve_rows(int xsize) { return xsize == 8 ? 16384 : 32768; }

int bsolve_analyse(hgb_ctx *c, int n, int nnz, const int *pntr_d, const int *indx_d, const int *diag_d, int lower,
                   int rev, int R, BlockSolve &S);
int bsolve_load_values(hgb_ctx *c, BlockSolve &S, const void *svals, int vsize, const double *piv);
template <typename V, typename X>
int bsolve_launch(hgb_ctx *c, const BlockSolve &S, int mode, int unit, X alpha, const X *in, X *out, X *pend_a,
                  X *pend_b, const int *skip);

}  // namespace hgb
