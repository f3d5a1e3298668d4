// Lower / upper split of a CSR matrix on the device: the patterns (split_pattern,
// sparse/hala_sparse_core.hpp:72-94, and its two passes split_pattern_array,
// sparse/hala_sparse_utils.hpp:176-193) and the values (split_values, core:97-120, and
// split_values_array, utils:201-221).  Row i of the lower triangle holds the entries [pntr_i, diag_i]
// and row i of the upper triangle the entries [diag_i, pntr_{i+1}): the diagonal is in both, and
// split_values sets it to 0 (diag 'N') or 1 (diag 'U') in the triangle that uplo does not select.
// Integer and copy work only: the results are bit-identical to the reference's loops.
#include "hgb_internal.cuh"
#include "hgb_kernels.cuh"

#include <algorithm>

namespace hgb {

// counts of row i in the lower / upper pattern; entry n is 0, so an exclusive scan of the n + 1
// counts gives the row pointers
__global__ void split_counts_kernel(int n, const int *__restrict__ pntr, const int *__restrict__ diag, int *lc, int *uc,
                                    int *err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x) {
        if (i == n) {
            lc[n] = 0;
            uc[n] = 0;
            continue;
        }
        const int a = pntr[i], b = pntr[i + 1], d = diag[i];
        if (d < a || d >= b) {   // the diagonal index must point into its row
            atomicOr(err, DEV_ERR_CSR);
            lc[i] = uc[i] = 0;
            continue;
        }
        lc[i] = d - a + 1;
        uc[i] = b - d;
    }
}

// One warp per row: the row's lower run [pntr_i, d_i] and upper run [d_i, pntr_{i+1}) copied with
// coalesced loads.  d_i comes from diag (patterns) or from the lower row length (values).
template <typename T>
__global__ void split_copy_kernel(int n, const int *__restrict__ pntr, const int *__restrict__ diag,
                                  const T *__restrict__ src, const int *__restrict__ up, const int *__restrict__ lp,
                                  T *ud, T *ld) {
    const int lane = threadIdx.x & 31;
    const long warp = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5, nw = ((long)gridDim.x * blockDim.x) >> 5;
    for (long i = warp; i < n; i += nw) {
        const int a = pntr[i], b = pntr[i + 1];
        const int l0 = lp[i], u0 = up[i];
        const int d = diag ? diag[i] : a + (lp[i + 1] - l0) - 1;
        for (int k = lane; k <= d - a; k += 32) ld[l0 + k] = src[a + k];
        for (int k = lane; k < b - d; k += 32) ud[u0 + k] = src[d + k];
    }
}

// the diagonal of the triangle uplo does not select becomes alpha (0 for diag 'N', 1 for 'U')
template <typename T>
__global__ void split_diag_kernel(int n, int lower_owns, T alpha, const int *__restrict__ up,
                                  const int *__restrict__ lp, T *uv, T *lv) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (lower_owns) uv[up[i]] = alpha;
        else lv[lp[i + 1] - 1] = alpha;
    }
}

static int split_grid(hgb_ctx *c, long work) {
    return (int)std::max<long>(1, std::min<long>((work + 255) / 256, (long)c->num_sms * 8));
}

template <typename T>
static int split_values_impl(hgb_ctx *c, char uplo, char diagc, int n, const int *pntr, const T *vals,
                             const int *upper_pntr, const int *lower_pntr, T *upper_vals, T *lower_vals) {
    if (!c || n < 0) return fail(HGB_ERR_ARG, "split_values: bad arguments");
    const bool lo = (uplo == 'L' || uplo == 'l'), up = (uplo == 'U' || uplo == 'u');
    const bool unit = (diagc == 'U' || diagc == 'u'), nonunit = (diagc == 'N' || diagc == 'n');
    if (!(lo || up) || !(unit || nonunit)) return fail(HGB_ERR_ARG, "split_values: uplo '%c' diag '%c'", uplo, diagc);
    if (n == 0) return HGB_OK;
    if (!pntr || !vals || !upper_pntr || !lower_pntr || !upper_vals || !lower_vals)
        return fail(HGB_ERR_ARG, "split_values: null array");
    DeviceGuard g(c->device);
    split_copy_kernel<T><<<split_grid(c, 32L * n), 256, 0, c->stream>>>(n, pntr, nullptr, vals, upper_pntr, lower_pntr,
                                                                        upper_vals, lower_vals);
    split_diag_kernel<T><<<split_grid(c, n), 256, 0, c->stream>>>(n, lo ? 1 : 0, unit ? T(1) : T(0), upper_pntr,
                                                                  lower_pntr, upper_vals, lower_vals);
    return launch_check("split_values");
}

}  // namespace hgb

using namespace hgb;

extern "C" {

int hgb_split_pattern_pntr(hgb_ctx *c, int n, const int *pntr, const int *diag, int *upper_pntr, int *lower_pntr,
                           int *upper_nnz, int *lower_nnz) {
    if (!c || n < 0 || !upper_pntr || !lower_pntr || !upper_nnz || !lower_nnz || (n > 0 && (!pntr || !diag)))
        return fail(HGB_ERR_ARG, "split_pattern_pntr: bad arguments");
    DeviceGuard g(c->device);
    int *cnt = nullptr;
    const size_t nb = (size_t)(n + 1 + 1023) / 1024 + 2;
    HGB_CUDA(ws_alloc(c, &cnt, 2 * (size_t)(n + 1) + 2 * nb));
    int *lc = cnt, *uc = cnt + (n + 1), *scratch = cnt + 2 * (n + 1);
    int st = HGB_OK;
    do {
        split_counts_kernel<<<split_grid(c, n + 1), 256, 0, c->stream>>>(n, pntr, diag, lc, uc, c->err);
        if ((st = launch_check("split_counts_kernel"))) break;
        if ((st = exclusive_scan(c, lc, lower_pntr, n + 1, scratch + nb, scratch))) break;
        if ((st = exclusive_scan(c, uc, upper_pntr, n + 1, scratch + nb, scratch))) break;
        if ((st = collect_dev_error(c))) break;   // synchronises
        if (cudaMemcpy(lower_nnz, lower_pntr + n, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(upper_nnz, upper_pntr + n, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
            st = cuda_fail(cudaGetLastError(), "split_pattern_pntr");
    } while (0);
    ws_free(c, cnt);
    if (st == HGB_ERR_CSR) return fail(HGB_ERR_CSR, "split_pattern: a diagonal index lies outside its row");
    return st;
}

int hgb_split_pattern_indx(hgb_ctx *c, int n, const int *pntr, const int *indx, const int *diag,
                           const int *upper_pntr, const int *lower_pntr, int *upper_indx, int *lower_indx) {
    if (!c || n < 0) return fail(HGB_ERR_ARG, "split_pattern_indx: bad arguments");
    if (n == 0) return HGB_OK;
    if (!pntr || !indx || !diag || !upper_pntr || !lower_pntr || !upper_indx || !lower_indx)
        return fail(HGB_ERR_ARG, "split_pattern_indx: null array");
    DeviceGuard g(c->device);
    split_copy_kernel<int><<<split_grid(c, 32L * n), 256, 0, c->stream>>>(n, pntr, diag, indx, upper_pntr, lower_pntr,
                                                                          upper_indx, lower_indx);
    return launch_check("split_pattern_indx");
}

int hgb_split_values_f64(hgb_ctx *c, char uplo, char diag, int n, const int *pntr, const double *vals,
                         const int *upper_pntr, const int *lower_pntr, double *upper_vals, double *lower_vals) {
    return split_values_impl<double>(c, uplo, diag, n, pntr, vals, upper_pntr, lower_pntr, upper_vals, lower_vals);
}
int hgb_split_values_f32(hgb_ctx *c, char uplo, char diag, int n, const int *pntr, const float *vals,
                         const int *upper_pntr, const int *lower_pntr, float *upper_vals, float *lower_vals) {
    return split_values_impl<float>(c, uplo, diag, n, pntr, vals, upper_pntr, lower_pntr, upper_vals, lower_vals);
}

}  // extern "C"
