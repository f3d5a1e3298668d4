"""Python mirror of the reference's GPU-engine interface for the sparse Krylov path.

Names and argument meaning follow HALA's overloads (gpu_engine, make_sparse_matrix, sparse_gemv,
make_ilu / ilu_apply, make_triangular_matrix / sparse_trsv, dot / norm2 / axpy / scal / vcopy,
stop_criteria, solve_cg / solve_cg_ilu / solve_gmres_ilu), acting on torch CUDA tensors.  Every
call goes through libhgb.so; errors raise HgbError (a RuntimeError), as the reference throws
std::runtime_error from check_cuda() (gpu/hala_cuda_common.hpp:78-152).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import hgb as _h
from .hgb import SolveInfo, check, ch_

INT_MAX = 2**31 - 1
_DT = {torch.float64: _h.HGB_F64, torch.float32: _h.HGB_F32, torch.bfloat16: _h.HGB_BF16,
       torch.complex128: _h.HGB_C128, torch.complex64: _h.HGB_C64}
_CPLX = {torch.complex128: ("c128", C.c_double), torch.complex64: ("c64", C.c_float)}


def _pair(v, ct):
    """a complex scalar as the {re, im} array the complex entry points take"""
    v = complex(v)
    return (ct * 2)(v.real, v.imag)


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _need(t, dtype=None, name="tensor"):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    return t


class stop_criteria:
    """hex/solvers/hala_solvers_core.hpp:52-70: an int sets only the iteration limit (tol 0),
    a float sets only the tolerance (limit INT_MAX), both set both."""

    def __init__(self, a=None, max_iter=None):
        if isinstance(a, int) and max_iter is None:
            self.max_iter, self.tol = a, 0.0
        else:
            self.tol = float(a)
            self.max_iter = INT_MAX if max_iter is None else int(max_iter)


class gpu_engine:
    """gpu/hala_gpu_engine.hpp:47: owns the device context (and the stream it runs on)."""

    def __init__(self, device=0):
        self.device = int(device)
        h = C.c_void_p()
        check(_h.lib().hgb_ctx_create(self.device, C.byref(h)), "gpu_engine")
        self.h = h
        self.set_stream(torch.cuda.current_stream(self.device))

    def set_stream(self, stream):
        self.stream = stream
        check(_h.lib().hgb_ctx_set_stream(self.h, C.c_void_p(stream.cuda_stream)), "set_stream")

    def synchronize(self):
        check(_h.lib().hgb_ctx_synchronize(self.h))

    def set_spmv_mode(self, mode):
        """'exact' (separately rounded multiply and add: bit-identical to the reference's CPU
        product) or 'fused' (one fused multiply-add per entry, the default)."""
        m = {"fused": _h.HGB_SPMV_FUSED, "exact": _h.HGB_SPMV_EXACT}[mode]
        check(_h.lib().hgb_ctx_set_spmv_mode(self.h, m), "set_spmv_mode")

    def spmv_mode(self):
        m = C.c_int()
        check(_h.lib().hgb_ctx_get_spmv_mode(self.h, C.byref(m)), "spmv_mode")
        return "exact" if m.value == _h.HGB_SPMV_EXACT else "fused"

    def __del__(self):
        try:
            if getattr(self, "h", None):
                _h.lib().hgb_ctx_destroy(self.h)
                self.h = None
        except Exception:
            pass


# --------------------------------------------------------------------------- BLAS-1 ----
def _sfx(t):
    if t.dtype == torch.float64:
        return "f64"
    if t.dtype == torch.float32:
        return "f32"
    raise TypeError(f"unsupported vector dtype {t.dtype}")


def dot(engine, x, y):
    """gpu/hala_gpu_blas1.hpp:179 (host-returned scalar; complex: conjugated, cublasZdotc)."""
    _need(x, name="x"); _need(y, x.dtype, "y")
    if x.dtype in _CPLX:
        sx, ct = _CPLX[x.dtype]
        r = (ct * 2)()
        check(getattr(_h.lib(), "hgb_dotc_" + sx)(engine.h, x.numel(), _p(x), _p(y), r, 0), "dot")
        return complex(r[0], r[1])
    r = (C.c_double if x.dtype == torch.float64 else C.c_float)()
    check(getattr(_h.lib(), "hgb_dot_" + _sfx(x))(engine.h, x.numel(), _p(x), _p(y), C.byref(r), 0), "dot")
    return r.value


def dotu(engine, x, y):
    """the unconjugated complex product sum x_i y_i (gpu/hala_gpu_blas1.hpp:179, dotu)."""
    _need(x, name="x"); _need(y, x.dtype, "y")
    sx, ct = _CPLX[x.dtype]
    r = (ct * 2)()
    check(getattr(_h.lib(), "hgb_dotu_" + sx)(engine.h, x.numel(), _p(x), _p(y), r, 0), "dotu")
    return complex(r[0], r[1])


def norm2(engine, x):
    """gpu/hala_gpu_blas1.hpp:102."""
    _need(x, name="x")
    if x.dtype in _CPLX:
        sx, ct = _CPLX[x.dtype]
        r = ct()
        check(getattr(_h.lib(), "hgb_nrm2_" + sx)(engine.h, x.numel(), _p(x), C.byref(r), 0), "norm2")
        return r.value
    r = (C.c_double if x.dtype == torch.float64 else C.c_float)()
    check(getattr(_h.lib(), "hgb_nrm2_" + _sfx(x))(engine.h, x.numel(), _p(x), C.byref(r), 0), "norm2")
    return r.value


def axpy(engine, alpha, x, y):
    """y += alpha x, gpu/hala_gpu_blas1.hpp:205."""
    _need(x, name="x"); _need(y, x.dtype, "y")
    if x.dtype in _CPLX:
        sx, ct = _CPLX[x.dtype]
        check(getattr(_h.lib(), "hgb_axpy_" + sx)(engine.h, x.numel(), _pair(alpha, ct), _p(x), _p(y)), "axpy")
        return
    check(getattr(_h.lib(), "hgb_axpy_" + _sfx(x))(engine.h, x.numel(), alpha, _p(x), _p(y)), "axpy")


def scal(engine, alpha, x):
    """x *= alpha, gpu/hala_gpu_blas1.hpp:229."""
    _need(x, name="x")
    if x.dtype in _CPLX:
        sx, ct = _CPLX[x.dtype]
        check(getattr(_h.lib(), "hgb_scal_" + sx)(engine.h, x.numel(), _pair(alpha, ct), _p(x)), "scal")
        return
    check(getattr(_h.lib(), "hgb_scal_" + _sfx(x))(engine.h, x.numel(), alpha, _p(x)), "scal")


def vcopy(engine, x, y):
    """y = x, gpu/hala_gpu_blas1.hpp:49."""
    _need(x, name="x"); _need(y, x.dtype, "y")
    if x.dtype in _CPLX:   # interleaved pairs: a copy of 2n reals
        x, y = torch.view_as_real(x).reshape(-1), torch.view_as_real(y).reshape(-1)
    check(getattr(_h.lib(), "hgb_copy_" + _sfx(x))(engine.h, x.numel(), _p(x), _p(y)), "vcopy")


def set_zero(engine, x):
    _need(x, name="x")
    check(_h.lib().hgb_set_zero(engine.h, x.numel() * x.element_size(), _p(x)), "set_zero")


def gemv(engine, trans, m, k, alpha, W, x, beta, y):
    """Tall-skinny dense gemv (column-major W, m x k), gpu/hala_gpu_blas2.hpp:40."""
    check(_h.lib().hgb_gemv_f64(engine.h, ch_(trans), m, k, alpha, _p(W), _p(x), beta, _p(y)), "gemv")


def get_diagonal_index(engine, pntr, indx):
    """sparse/hala_sparse_core.hpp:45-60 on the device."""
    n = pntr.numel() - 1
    diag = torch.empty(n, dtype=torch.int32, device=pntr.device)
    check(_h.lib().hgb_diag_index(engine.h, n, indx.numel(), _p(pntr), _p(indx), _p(diag)), "get_diagonal_index")
    return diag


def split_pattern(engine, pntr, indx, diag):
    """split_pattern (sparse/hala_sparse_core.hpp:72-94) on the device: the upper and lower CSR
    patterns, the diagonal in both.  Returns (upper_pntr, upper_indx, lower_pntr, lower_indx)."""
    _need(pntr, torch.int32, "pntr"); _need(indx, torch.int32, "indx"); _need(diag, torch.int32, "diag")
    n = pntr.numel() - 1
    up = torch.empty(n + 1, dtype=torch.int32, device=pntr.device)
    lp = torch.empty(n + 1, dtype=torch.int32, device=pntr.device)
    nu, nl = C.c_int(), C.c_int()
    check(_h.lib().hgb_split_pattern_pntr(engine.h, n, _p(pntr), _p(diag), _p(up), _p(lp), C.byref(nu), C.byref(nl)),
          "split_pattern")
    ui = torch.empty(max(nu.value, 1), dtype=torch.int32, device=pntr.device)[:nu.value]
    li = torch.empty(max(nl.value, 1), dtype=torch.int32, device=pntr.device)[:nl.value]
    check(_h.lib().hgb_split_pattern_indx(engine.h, n, _p(pntr), _p(indx), _p(diag), _p(up), _p(lp), _p(ui), _p(li)),
          "split_pattern")
    return up, ui, lp, li


def split_values(engine, uplo, diag, pntr, vals, upper_pntr, lower_pntr):
    """split_values (sparse/hala_sparse_core.hpp:97-120) on the device.  Returns (upper_vals,
    lower_vals); the diagonal of the triangle uplo does not select is 0 (diag 'N') or 1 ('U')."""
    _need(pntr, torch.int32, "pntr"); _need(vals, name="vals")
    n = pntr.numel() - 1
    nu, nl = int(upper_pntr[-1]), int(lower_pntr[-1])
    uv = torch.empty(max(nu, 1), dtype=vals.dtype, device=vals.device)[:nu]
    lv = torch.empty(max(nl, 1), dtype=vals.dtype, device=vals.device)[:nl]
    check(getattr(_h.lib(), f"hgb_split_values_{_sfx(vals)}")(engine.h, ch_(uplo), ch_(diag), n, _p(pntr), _p(vals),
                                                               _p(upper_pntr), _p(lower_pntr), _p(uv), _p(lv)),
          "split_values")
    return uv, lv


# ------------------------------------------------------------------------- sparse ------
def sparse_gemv(engine, trans, M, N, alpha, pntr, indx, vals, x, beta, y):
    """sparse_gemv(gpu_engine, trans, M, N, alpha, pntr, indx, vals, x, beta, y),
    gpu/hala_cuda_sparse_general.hpp:408-419.  y is updated in place."""
    _need(pntr, torch.int32, "pntr"); _need(indx, torch.int32, "indx"); _need(vals, name="vals")
    nnz = indx.numel()
    L = _h.lib()
    t = ch_(trans)
    if vals.dtype == torch.float64:
        st = L.hgb_spmv_f64(engine.h, t, M, N, nnz, _p(pntr), _p(indx), _p(vals), alpha, _p(x), beta, _p(y))
    elif vals.dtype == torch.float32:
        st = L.hgb_spmv_f32(engine.h, t, M, N, nnz, _p(pntr), _p(indx), _p(vals), alpha, _p(x), beta, _p(y))
    elif vals.dtype == torch.bfloat16:
        st = L.hgb_spmv_bf16f32(engine.h, t, M, N, nnz, _p(pntr), _p(indx), _p(vals), alpha, _p(x), beta, _p(y))
    elif vals.dtype in _CPLX:
        sx, ct = _CPLX[vals.dtype]
        st = getattr(L, "hgb_spmv_" + sx)(engine.h, t, M, N, nnz, _p(pntr), _p(indx), _p(vals), _pair(alpha, ct),
                                          _p(x), _pair(beta, ct), _p(y))
    else:
        raise TypeError(f"unsupported value dtype {vals.dtype}")
    check(st, "sparse_gemv")
    return y


class gpu_sparse_matrix:
    """gpu/hala_cuda_sparse_general.hpp:192-375: non-owning view + cached analysis."""

    def __init__(self, engine, num_rows, pntr, indx, vals, num_cols=None):
        _need(pntr, torch.int32, "pntr"); _need(indx, torch.int32, "indx"); _need(vals, name="vals")
        self.engine = engine
        self.rows = int(num_rows)
        self.cols = int(num_rows if num_cols is None else num_cols)
        self._keep = (pntr, indx, vals)
        self.dtype = vals.dtype
        h = C.c_void_p()
        check(_h.lib().hgb_csr_create(engine.h, self.rows, self.cols, indx.numel(), _p(pntr), _p(indx), _p(vals),
                                      _DT[vals.dtype], C.byref(h)), "make_sparse_matrix")
        self.h = h

    def gemv(self, trans, alpha, x, beta, y):
        if self.dtype in _CPLX:
            check(_h.lib().hgb_csr_gemv_z(self.h, ch_(trans), _pair(alpha, C.c_double), _p(x),
                                          _pair(beta, C.c_double), _p(y)), "gemv")
            return y
        check(_h.lib().hgb_csr_gemv(self.h, ch_(trans), float(alpha), _p(x), float(beta), _p(y)), "gemv")
        return y

    def gemm(self, nrhs, alpha, x, beta, y):
        """Y = alpha A X + beta Y for n x nrhs column-major blocks (sparse_gemm 'N','N')."""
        check(_h.lib().hgb_csr_gemm(self.h, int(nrhs), float(alpha), _p(x), self.cols, float(beta), _p(y),
                                    self.rows), "gemm")
        return y

    def gemv_dot(self, x, y, dot_out):
        """y = A x and dot_out[0] = <x, y> (device scalar, float64 tensor)."""
        check(_h.lib().hgb_csr_gemv_dot(self.h, _p(x), _p(y), _p(dot_out)), "gemv_dot")
        return y

    def __del__(self):
        try:
            if getattr(self, "h", None):
                _h.lib().hgb_csr_destroy(self.h)
                self.h = None
        except Exception:
            pass


def make_sparse_matrix(engine, num_rows, pntr, indx, vals, num_cols=None):
    return gpu_sparse_matrix(engine, num_rows, pntr, indx, vals, num_cols)


class gpu_ilu:
    """gpu/hala_gpu_ilu.hpp:45-185.  store: torch dtype of the factor the solves read
    (float64 default; float32 or bfloat16 keep FP64 pivots)."""

    def __init__(self, engine, pntr, indx, vals, policy="N", store=None):
        _need(pntr, torch.int32, "pntr"); _need(indx, torch.int32, "indx"); _need(vals, name="vals")
        store = vals.dtype if store is None else store
        self.engine = engine
        self.n = pntr.numel() - 1
        self.nnz = indx.numel()
        self.store = store
        self.fdtype = vals.dtype
        self._keep = (pntr, indx)
        h = C.c_void_p()
        st = _h.lib().hgb_ilu0_create(engine.h, self.n, self.nnz, _p(pntr), _p(indx), _p(vals), _DT[vals.dtype],
                                      _DT[store], ch_(policy), C.byref(h))
        self.h = h if h.value else None
        self.zero_pivot = (st == _h.HGB_ERR_ZERO_PIVOT)
        if st not in (_h.HGB_OK, _h.HGB_ERR_ZERO_PIVOT):
            check(st, "make_ilu")

    @property
    def vector_dtype(self):
        if self.store in _CPLX or self.store == torch.float64:
            return self.store
        return torch.float32

    def apply(self, x, r=None, trans="N"):
        r = torch.empty_like(x) if r is None else r
        check(_h.lib().hgb_ilu0_apply(self.h, ch_(trans), _p(x), _p(r)), "ilu apply")
        return r

    def apply_nrhs(self, x, nrhs, r=None, trans="N"):
        """apply(x, r, num_rhs): nrhs column-major right-hand sides."""
        r = torch.empty_like(x) if r is None else r
        check(_h.lib().hgb_ilu0_apply_nrhs(self.h, ch_(trans), int(nrhs), _p(x), _p(r)), "ilu apply nrhs")
        return r

    def factor(self):
        f = torch.empty(self.nnz, dtype=self.fdtype, device="cuda")
        d = torch.empty(self.n, dtype=torch.int32, device="cuda")
        check(_h.lib().hgb_ilu0_export(self.h, _p(f), _p(d)), "ilu export")
        return f, d

    def levels(self, uplo):
        lev = torch.empty(self.n, dtype=torch.int32, device="cuda")
        nl = C.c_int()
        check(_h.lib().hgb_ilu0_levels(self.h, ch_(uplo), _p(lev), C.byref(nl)), "ilu levels")
        return lev, nl.value

    def __del__(self):
        try:
            if getattr(self, "h", None):
                _h.lib().hgb_ilu0_destroy(self.h)
                self.h = None
        except Exception:
            pass


def make_ilu(engine, pntr, indx, vals, policy="N", store=None):
    return gpu_ilu(engine, pntr, indx, vals, policy, store)


class mixed_ilu(gpu_ilu):
    """make_ilu(mixed_engine, pntr, indx, vals, policy), wax/hala_lib_extensions.hpp:311-366: HOST
    (numpy) pattern and values; the handle owns their device copies, which travel while the host
    plans the triangular schedules (hgb_ilu0_create_host)."""

    def __init__(self, engine, pntr_h, indx_h, vals_h, policy="N", store=None):
        import numpy as np
        pntr_h = np.ascontiguousarray(pntr_h, dtype=np.int32)
        indx_h = np.ascontiguousarray(indx_h, dtype=np.int32)
        vdt = {np.dtype(np.float64): torch.float64, np.dtype(np.float32): torch.float32,
               np.dtype(np.complex128): torch.complex128, np.dtype(np.complex64): torch.complex64}[vals_h.dtype]
        vals_h = np.ascontiguousarray(vals_h)
        store = vdt if store is None else store
        self.engine = engine
        self.n = len(pntr_h) - 1
        self.nnz = len(indx_h)
        self.store = store
        self.fdtype = vdt
        self._keep = ()
        h = C.c_void_p()
        st = _h.lib().hgb_ilu0_create_host(engine.h, self.n, self.nnz, pntr_h.ctypes.data_as(C.c_void_p),
                                           indx_h.ctypes.data_as(C.c_void_p), vals_h.ctypes.data_as(C.c_void_p),
                                           _DT[vdt], _DT[store], ch_(policy), C.byref(h))
        self.h = h if h.value else None
        self.zero_pivot = (st == _h.HGB_ERR_ZERO_PIVOT)
        if st not in (_h.HGB_OK, _h.HGB_ERR_ZERO_PIVOT):
            check(st, "make_ilu(mixed_engine)")


def make_ilu_host(engine, pntr_h, indx_h, vals_h, policy="N", store=None):
    return mixed_ilu(engine, pntr_h, indx_h, vals_h, policy, store)


def ilu_apply(ilu, x, r, num_rhs=1):
    """wax/hala_sparse_extensions.hpp:51."""
    if num_rhs != 1:
        raise NotImplementedError("multiple right-hand sides")
    return ilu.apply(x, r)


class gpu_triangular_matrix:
    """gpu/hala_cuda_sparse_triangular.hpp:38."""

    def __init__(self, engine, uplo, diag, pntr, indx, vals):
        _need(pntr, torch.int32, "pntr"); _need(indx, torch.int32, "indx"); _need(vals, name="vals")
        self._keep = (pntr, indx, vals)
        self.n = pntr.numel() - 1
        h = C.c_void_p()
        check(_h.lib().hgb_tri_create(engine.h, ch_(uplo), ch_(diag), self.n, indx.numel(), _p(pntr), _p(indx),
                                      _p(vals), _DT[vals.dtype], C.byref(h)), "make_triangular_matrix")
        self.h = h

    def trsv(self, trans, alpha, b, x):
        check(_h.lib().hgb_tri_solve(self.h, ch_(trans), float(alpha), _p(b), _p(x)), "trsv")
        return x

    def __del__(self):
        try:
            if getattr(self, "h", None):
                _h.lib().hgb_tri_destroy(self.h)
                self.h = None
        except Exception:
            pass


def make_triangular_matrix(engine, uplo, diag, pntr, indx, vals):
    return gpu_triangular_matrix(engine, uplo, diag, pntr, indx, vals)


def sparse_trsv(trans, tri, alpha, b, x):
    return tri.trsv(trans, alpha, b, x)


# ------------------------------------------------------------------------ solvers ------
def _stop(stop):
    return stop if isinstance(stop, stop_criteria) else stop_criteria(stop)


def solve_cg(engine, stop, pntr, indx, vals, b, x, ilu=None, matrix=None):
    """solve_cg / solve_cg_ilu(gpu_engine, ...), hex/solvers/hala_solvers_cg.hpp:181-326.
    Returns the reference's iteration count; x is updated in place."""
    s = _stop(stop)
    A = matrix or gpu_sparse_matrix(engine, pntr.numel() - 1, pntr, indx, vals)
    info = SolveInfo()
    check(_h.lib().hgb_cg_solve(engine.h, A.h, ilu.h if ilu else None, _p(b), _p(x), s.tol, s.max_iter,
                                C.byref(info)), "solve_cg")
    return info.iterations


def solve_cg_ilu(engine, stop, pntr, indx, vals, b, x, ilu=None, policy="N"):
    """solve_cg_ilu: factorises on the fly when no ILU is given (hala_solvers_cg.hpp:359-369)."""
    ilu = ilu or make_ilu(engine, pntr, indx, vals, policy)
    return solve_cg(engine, stop, pntr, indx, vals, b, x, ilu=ilu)


def sparse_gemm(A, nrhs, alpha, x, beta, y):
    return A.gemm(nrhs, alpha, x, beta, y)


def solve_batch_cg(engine, stop, pntr, indx, vals, B, X, ilu=None, matrix=None):
    """solve_batch_cg / solve_batch_cg_ilu(gpu_engine, ...), hex/solvers/hala_solvers_cg_batch.hpp:
    B, X hold nrhs = B.numel() / n column-major right-hand sides; all columns iterate together until
    the largest column residual is below stop.tol.  Returns the iteration count; X in place."""
    s = _stop(stop)
    n = pntr.numel() - 1
    nrhs = B.numel() // n
    A = matrix or gpu_sparse_matrix(engine, n, pntr, indx, vals)
    info = SolveInfo()
    check(_h.lib().hgb_cg_solve_nrhs(engine.h, A.h, ilu.h if ilu else None, nrhs, _p(B), _p(X), s.tol, s.max_iter,
                                     C.byref(info)), "solve_batch_cg")
    return info.iterations


def solve_batch_cg_ilu(engine, stop, pntr, indx, vals, B, X, ilu=None, policy="N"):
    ilu = ilu or make_ilu(engine, pntr, indx, vals, policy)
    return solve_batch_cg(engine, stop, pntr, indx, vals, B, X, ilu=ilu)


def solve_cg_info(engine, A, ilu, b, x, tol, max_iter=INT_MAX):
    info = SolveInfo()
    check(_h.lib().hgb_cg_solve(engine.h, A.h, ilu.h if ilu else None, _p(b), _p(x), float(tol), int(max_iter),
                                C.byref(info)), "solve_cg")
    return info


def solve_cg_op(engine, A, ilu, trans, b, x, tol, max_iter=INT_MAX):
    """CG on op(A) = A or A^T with the matching preconditioner (LU)^-1 or (LU)^-T; the adjoint
    solve of the differentiable path.  Returns SolveInfo."""
    info = SolveInfo()
    check(_h.lib().hgb_cg_solve_op(engine.h, A.h, ilu.h if ilu else None, ch_(trans), _p(b), _p(x), float(tol),
                                   int(max_iter), C.byref(info)), "solve_cg_op")
    return info


def solve_ir_pcg_op(engine, A64, A_inner, ilu_inner, trans, b, x, tol, inner_rtol=1e-4, max_inner=5000,
                    max_outer=50):
    info = SolveInfo()
    check(_h.lib().hgb_ir_pcg_solve_op(engine.h, A64.h, A_inner.h, ilu_inner.h if ilu_inner else None, ch_(trans),
                                       _p(b), _p(x), float(tol), float(inner_rtol), int(max_inner), int(max_outer),
                                       C.byref(info)), "solve_ir_pcg_op")
    return info


def pattern_grad(A, alpha, lam, u, grad):
    """grad[p] = alpha * lam[row(p)] * u[col(p)] over A's pattern (dL/dA with alpha = -1)."""
    check(_h.lib().hgb_csr_pattern_grad(A.h, float(alpha), _p(lam), _p(u), _p(grad)), "pattern_grad")
    return grad


def solve_gmres(engine, stop, restart, pntr, indx, vals, b, x, ilu=None, matrix=None):
    """solve_gmres / solve_gmres_ilu(gpu_engine, ...), hex/solvers/hala_solvers_gmres.hpp:127-267.
    Returns the number of operator applications (the reference's return value)."""
    s = _stop(stop)
    A = matrix or gpu_sparse_matrix(engine, pntr.numel() - 1, pntr, indx, vals)
    info = SolveInfo()
    check(_h.lib().hgb_gmres_solve(engine.h, A.h, ilu.h if ilu else None, int(restart), _p(b), _p(x), s.tol,
                                   s.max_iter, C.byref(info)), "solve_gmres")
    return info.iterations


def solve_gmres_ilu(engine, stop, restart, pntr, indx, vals, b, x, ilu=None, policy="N"):
    ilu = ilu or make_ilu(engine, pntr, indx, vals, policy)
    return solve_gmres(engine, stop, restart, pntr, indx, vals, b, x, ilu=ilu)


def solve_ir_pcg(engine, A64, A_inner, ilu_inner, b, x, tol, inner_rtol=1e-4, max_inner=5000, max_outer=50):
    """Mixed-precision ILU(0)-PCG: FP32/BF16 inner solves, FP64 refinement (no reference
    counterpart).  Returns SolveInfo."""
    info = SolveInfo()
    st = _h.lib().hgb_ir_pcg_solve(engine.h, A64.h, A_inner.h, ilu_inner.h if ilu_inner else None, _p(b), _p(x),
                                   float(tol), float(inner_rtol), int(max_inner), int(max_outer), C.byref(info))
    check(st, "solve_ir_pcg")
    return info


def solve_ru_pcg(engine, A64, A_inner, ilu_inner, b, x, tol, delta=0.01, max_iter=100000):
    """Mixed-precision ILU(0)-PCG with FP64 reliable updates: one FP32/BF16 PCG whose residual is
    replaced by the FP64 b - A x whenever it has dropped by delta (no reference counterpart).
    Returns SolveInfo (iterations; outer = reliable updates)."""
    info = SolveInfo()
    st = _h.lib().hgb_ru_pcg_solve(engine.h, A64.h, A_inner.h, ilu_inner.h if ilu_inner else None, _p(b), _p(x),
                                   float(tol), float(delta), int(max_iter), C.byref(info))
    check(st, "solve_ru_pcg")
    return info


def solve_ru_pcg_op(engine, A64, A_inner, ilu_inner, trans, b, x, tol, delta=0.01, max_iter=100000):
    """solve_ru_pcg on op(A) ('N' or 'T'): the adjoint solve of the mixed forward solve."""
    info = SolveInfo()
    st = _h.lib().hgb_ru_pcg_solve_op(engine.h, A64.h, A_inner.h, ilu_inner.h if ilu_inner else None, ch_(trans),
                                      _p(b), _p(x), float(tol), float(delta), int(max_iter), C.byref(info))
    check(st, "solve_ru_pcg")
    return info


def solve_ir_gmres(engine, A64, A_inner, ilu_inner, restart, b, x, tol, inner_rtol=1e-4, max_inner=3000,
                   max_outer=50):
    """Mixed-precision ILU(0)-GMRES(restart): FP32/BF16 inner solves, FP64 refinement to
    ||b - A x|| < tol (no reference counterpart; the inner solver is solve_gmres).  Returns SolveInfo."""
    info = SolveInfo()
    st = _h.lib().hgb_ir_gmres_solve(engine.h, A64.h, A_inner.h, ilu_inner.h if ilu_inner else None, int(restart),
                                     _p(b), _p(x), float(tol), float(inner_rtol), int(max_inner), int(max_outer),
                                     C.byref(info))
    check(st, "solve_ir_gmres")
    return info


def solve_cg_mixed(engine, stop, pntr_h, indx_h, vals_h, ilu, b_h, x_h):
    """solve_cg_ilu(mixed_engine, ...) (hala_solvers_cg.hpp:330-340): numpy host arrays in,
    device solve, x written back to the host array.  Returns SolveInfo."""
    import numpy as np
    s = _stop(stop)
    for a, dt in ((pntr_h, np.int32), (indx_h, np.int32), (vals_h, np.float64), (b_h, np.float64), (x_h, np.float64)):
        if a.dtype != dt or not a.flags.c_contiguous:
            raise TypeError("mixed solve: contiguous int32 pattern and float64 values/vectors required")
    info = SolveInfo()
    n = pntr_h.size - 1
    check(_h.lib().hgb_mixed_cg_solve(engine.h, n, indx_h.size, pntr_h.ctypes.data_as(C.c_void_p),
                                      indx_h.ctypes.data_as(C.c_void_p), vals_h.ctypes.data_as(C.c_void_p),
                                      ilu.h if ilu else None, b_h.ctypes.data_as(C.c_void_p),
                                      x_h.ctypes.data_as(C.c_void_p), s.tol, s.max_iter, C.byref(info)),
          "solve_cg (mixed)")
    return info


def solve_ir_pcg_mixed(engine, tol, pntr_h, indx_h, vals_h, ilu_inner, b_h, x_h, inner_rtol=1e-4,
                       max_inner=5000, max_outer=50):
    """Host-buffer mixed-precision refinement (hgb_mixed_ir_pcg_solve).  Returns SolveInfo."""
    info = SolveInfo()
    n = pntr_h.size - 1
    check(_h.lib().hgb_mixed_ir_pcg_solve(engine.h, n, indx_h.size, pntr_h.ctypes.data_as(C.c_void_p),
                                          indx_h.ctypes.data_as(C.c_void_p), vals_h.ctypes.data_as(C.c_void_p),
                                          ilu_inner.h, b_h.ctypes.data_as(C.c_void_p),
                                          x_h.ctypes.data_as(C.c_void_p), float(tol), float(inner_rtol),
                                          int(max_inner), int(max_outer), C.byref(info)), "solve_ir_pcg (mixed)")
    return info


def solve_ru_pcg_mixed(engine, tol, pntr_h, indx_h, vals_h, ilu_inner, b_h, x_h, delta=0.01, max_iter=100000):
    """Host-buffer mixed-precision PCG with reliable updates (hgb_mixed_ru_pcg_solve).  Returns SolveInfo."""
    info = SolveInfo()
    n = pntr_h.size - 1
    check(_h.lib().hgb_mixed_ru_pcg_solve(engine.h, n, indx_h.size, pntr_h.ctypes.data_as(C.c_void_p),
                                          indx_h.ctypes.data_as(C.c_void_p), vals_h.ctypes.data_as(C.c_void_p),
                                          ilu_inner.h, b_h.ctypes.data_as(C.c_void_p),
                                          x_h.ctypes.data_as(C.c_void_p), float(tol), float(delta), int(max_iter),
                                          C.byref(info)), "solve_ru_pcg (mixed)")
    return info


class gpu_batch:
    """Many independent SPD systems (block-diagonal CSR, FP32 values) solved in one persistent
    launch with FP64 refinement (hgb_batch_*; no reference counterpart)."""

    def __init__(self, engine, sys_ptr, pntr, indx, vals):
        _need(sys_ptr, torch.int32, "sys_ptr"); _need(pntr, torch.int32, "pntr"); _need(indx, torch.int32, "indx")
        _need(vals, torch.float32, "vals")
        self.engine = engine
        self.S = sys_ptr.numel() - 1
        self.n = pntr.numel() - 1
        self._keep = (sys_ptr, pntr, indx, vals)
        h = C.c_void_p()
        check(_h.lib().hgb_batch_create(engine.h, self.S, _p(sys_ptr), self.n, indx.numel(), _p(pntr), _p(indx),
                                        _p(vals), C.byref(h)), "batch_create")
        self.h = h

    @property
    def config(self):
        c = _h.BatchConfig()
        check(_h.lib().hgb_batch_get_config(self.h, C.byref(c)), "batch config")
        return (c.block_threads, c.warp_max_n)

    def set_config(self, block_threads, warp_max_n):
        c = _h.BatchConfig(block_threads, warp_max_n)
        check(_h.lib().hgb_batch_set_config(self.h, C.byref(c)), "batch config")

    def autotune(self, b, x, rtol, cache_path=None):
        c = _h.BatchConfig()
        check(_h.lib().hgb_batch_autotune(self.h, _p(b), _p(x), float(rtol),
                                          cache_path.encode() if cache_path else None, C.byref(c)), "batch autotune")
        return (c.block_threads, c.warp_max_n)

    def solve(self, b, x, rtol=1e-8, inner_rtol=1e-4, max_inner=1000, max_outer=20, iters=None, relres=None):
        _need(b, torch.float64, "b"); _need(x, torch.float64, "x")
        check(_h.lib().hgb_batch_cg_solve(self.h, _p(b), _p(x), float(rtol), float(inner_rtol), int(max_inner),
                                          int(max_outer), _p(iters), _p(relres)), "batch_cg_solve")
        return x

    def __del__(self):
        try:
            if getattr(self, "h", None):
                _h.lib().hgb_batch_destroy(self.h)
                self.h = None
        except Exception:
            pass
