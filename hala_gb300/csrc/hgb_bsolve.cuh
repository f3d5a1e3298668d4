// Block-local level-scheduled triangular solve (hgb_bsolve.cu): analysis data and entry points.
#pragma once

#include "hgb_internal.cuh"

namespace hgb {

struct BlockSolve {
    int n = 0, nblk = 0, nsteps = 0, R = 0;
    long npk = 0, novf = 0;
    int vsize = 0, dv_recip = 0;
    int4 *blk = nullptr;        // [nblk] {first step, end step, row_lo, rows}
    int4 *desc = nullptr;       // [nsteps] {first packet, rows, first overflow entry, overflow width | barrier << 16}
    int4 *pk0 = nullptr;        // [npk] {code0, code1, code2, slot | ndeps << 16}
    int4 *pkv = nullptr;        // [NV * npk] value pieces (store precision, diagonal terms)
    int *rj = nullptr;          // [npk] first dependency of the row on an earlier block (fetched), or -1
    int *push = nullptr;        // [npk] where the row's value goes in the next block's ring, or -1
    int cl = 1;                 // CTAs per thread-block cluster the push targets assume
    int *ovf_codes = nullptr;   // [novf] dependencies beyond the third, column-major per step
    void *ovf_vals = nullptr;
    int *map3 = nullptr, *dv_map = nullptr, *dv_row = nullptr, *ovf_map = nullptr;   // value gather maps
    int *ticket = nullptr;
    void release();
};

// Rows per block for a solve over n rows with an xsize-byte solution (the block's slice lives in
// shared memory: at most 16384 rows).
int bsolve_rows(hgb_ctx *c, int xsize, int n);

int bsolve_analyse(hgb_ctx *c, int n, int nnz, const int *pntr_d, const int *indx_d, const int *diag_d, int lower,
                   int rev, int R, int xsize, BlockSolve &S);
// the lower (unit) and upper schedules of an ILU factor planned from HOST copies of the pattern and
// the diagonal index (two host threads), then uploaded
struct BsPlanPair;
int bsolve_plan_pair(hgb_ctx *c, int n, int nnz, const int *pntr, const int *indx, const int *diag, int R, int xsize,
                     BsPlanPair **out);
int bsolve_upload_pair(BsPlanPair *P, BlockSolve &SL, BlockSolve &SU);
void bsolve_plan_pair_free(BsPlanPair *P);
int bsolve_load_values(hgb_ctx *c, BlockSolve &S, const void *svals, int vsize, const double *piv);
template <typename V, typename X>
int bsolve_launch(hgb_ctx *c, const BlockSolve &S, int mode, int unit, X alpha, const X *in, X *out, X *pend,
                  const int *skip);

}  // namespace hgb
