"""ctypes binding of libhgb.so (include/hgb.h).

Loads the in-tree library built by hala_gb300/build.py.  There is no fallback: if the library
is missing or no CUDA device is visible, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

HGB_OK, HGB_ERR_ARG, HGB_ERR_CSR, HGB_ERR_ZERO_PIVOT, HGB_ERR_TIMEOUT = 0, 1, 2, 3, 4
HGB_ERR_NOT_CONVERGED, HGB_ERR_CUDA, HGB_ERR_ALLOC, HGB_ERR_UNSUPPORTED = 5, 6, 7, 8
HGB_F64, HGB_F32, HGB_BF16, HGB_C128, HGB_C64 = 0, 1, 2, 3, 4
HGB_SPMV_FUSED, HGB_SPMV_EXACT = 0, 1


class HgbError(RuntimeError):
    """A non-zero hgb_status, raised like the reference's check_cuda() runtime_error."""

    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("outer", C.c_int), ("residual", C.c_double),
                ("true_residual", C.c_double), ("kernel_launches", C.c_longlong)]


class BatchConfig(C.Structure):
    _fields_ = [("block_threads", C.c_int), ("warp_max_n", C.c_int)]


_lib = None
vp, i32, f64, f32, ch = C.c_void_p, C.c_int, C.c_double, C.c_float, C.c_char

_SIGS = {
    "hgb_status_string": ([i32], C.c_char_p),
    "hgb_last_error": ([], C.c_char_p),
    "hgb_version": ([], i32),
    "hgb_ctx_create": ([i32, C.POINTER(vp)], i32),
    "hgb_ctx_destroy": ([vp], i32),
    "hgb_ctx_set_stream": ([vp, vp], i32),
    "hgb_ctx_synchronize": ([vp], i32),
    "hgb_ctx_set_spmv_mode": ([vp, i32], i32),
    "hgb_ctx_get_spmv_mode": ([vp, C.POINTER(i32)], i32),
    "hgb_dot_f64": ([vp, i32, vp, vp, vp, i32], i32),
    "hgb_dot_f32": ([vp, i32, vp, vp, vp, i32], i32),
    "hgb_nrm2_f64": ([vp, i32, vp, vp, i32], i32),
    "hgb_nrm2_f32": ([vp, i32, vp, vp, i32], i32),
    "hgb_axpy_f64": ([vp, i32, f64, vp, vp], i32),
    "hgb_axpy_f32": ([vp, i32, f32, vp, vp], i32),
    "hgb_scal_f64": ([vp, i32, f64, vp], i32),
    "hgb_scal_f32": ([vp, i32, f32, vp], i32),
    "hgb_copy_f64": ([vp, i32, vp, vp], i32),
    "hgb_copy_f32": ([vp, i32, vp, vp], i32),
    "hgb_set_zero": ([vp, C.c_size_t, vp], i32),
    "hgb_split_pattern_pntr": ([vp, i32, vp, vp, vp, vp, C.POINTER(i32), C.POINTER(i32)], i32),
    "hgb_split_pattern_indx": ([vp, i32, vp, vp, vp, vp, vp, vp, vp], i32),
    "hgb_split_values_f64": ([vp, ch, ch, i32, vp, vp, vp, vp, vp, vp], i32),
    "hgb_split_values_f32": ([vp, ch, ch, i32, vp, vp, vp, vp, vp, vp], i32),
    "hgb_ilu0_create_host": ([vp, i32, i32, vp, vp, vp, i32, i32, ch, C.POINTER(vp)], i32),
    "hgb_gemv_f64": ([vp, ch, i32, i32, f64, vp, vp, f64, vp], i32),
    "hgb_gemv_f32": ([vp, ch, i32, i32, f32, vp, vp, f32, vp], i32),
    "hgb_dgmm_f64": ([vp, ch, i32, i32, vp, vp, vp], i32),
    "hgb_dgmm_f32": ([vp, ch, i32, i32, vp, vp, vp], i32),
    "hgb_spmv_f64": ([vp, ch, i32, i32, i32, vp, vp, vp, f64, vp, f64, vp], i32),
    "hgb_spmv_f32": ([vp, ch, i32, i32, i32, vp, vp, vp, f32, vp, f32, vp], i32),
    "hgb_spmv_bf16f32": ([vp, ch, i32, i32, i32, vp, vp, vp, f32, vp, f32, vp], i32),
    "hgb_spmv_c128": ([vp, ch, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp], i32),
    "hgb_spmv_c64": ([vp, ch, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp], i32),
    "hgb_dotc_c128": ([vp, i32, vp, vp, vp, i32], i32),
    "hgb_dotc_c64": ([vp, i32, vp, vp, vp, i32], i32),
    "hgb_dotu_c128": ([vp, i32, vp, vp, vp, i32], i32),
    "hgb_dotu_c64": ([vp, i32, vp, vp, vp, i32], i32),
    "hgb_nrm2_c128": ([vp, i32, vp, vp, i32], i32),
    "hgb_nrm2_c64": ([vp, i32, vp, vp, i32], i32),
    "hgb_axpy_c128": ([vp, i32, vp, vp, vp], i32),
    "hgb_axpy_c64": ([vp, i32, vp, vp, vp], i32),
    "hgb_scal_c128": ([vp, i32, vp, vp], i32),
    "hgb_scal_c64": ([vp, i32, vp, vp], i32),
    "hgb_csr_gemv_z": ([vp, ch, vp, vp, vp, vp], i32),
    "hgb_csr_create": ([vp, i32, i32, i32, vp, vp, vp, i32, C.POINTER(vp)], i32),
    "hgb_csr_gemv": ([vp, ch, f64, vp, f64, vp], i32),
    "hgb_csr_gemv_dot": ([vp, vp, vp, vp], i32),
    "hgb_csr_destroy": ([vp], i32),
    "hgb_diag_index": ([vp, i32, i32, vp, vp, vp], i32),
    "hgb_ilu0_create": ([vp, i32, i32, vp, vp, vp, i32, i32, ch, C.POINTER(vp)], i32),
    "hgb_ilu0_apply": ([vp, ch, vp, vp], i32),
    "hgb_ilu0_export": ([vp, vp, vp], i32),
    "hgb_ilu0_levels": ([vp, ch, vp, C.POINTER(i32)], i32),
    "hgb_ilu0_destroy": ([vp], i32),
    "hgb_tri_create": ([vp, ch, ch, i32, i32, vp, vp, vp, i32, C.POINTER(vp)], i32),
    "hgb_tri_solve": ([vp, ch, f64, vp, vp], i32),
    "hgb_tri_destroy": ([vp], i32),
    "hgb_cg_solve": ([vp, vp, vp, vp, vp, f64, i32, C.POINTER(SolveInfo)], i32),
    "hgb_ir_pcg_solve": ([vp, vp, vp, vp, vp, vp, f64, f64, i32, i32, C.POINTER(SolveInfo)], i32),
    "hgb_cg_solve_op": ([vp, vp, vp, ch, vp, vp, f64, i32, C.POINTER(SolveInfo)], i32),
    "hgb_csr_gemm": ([vp, i32, f64, vp, i32, f64, vp, i32], i32),
    "hgb_ilu0_apply_nrhs": ([vp, ch, i32, vp, vp], i32),
    "hgb_cg_solve_nrhs": ([vp, vp, vp, i32, vp, vp, f64, i32, C.POINTER(SolveInfo)], i32),
    "hgb_ir_pcg_solve_op": ([vp, vp, vp, vp, ch, vp, vp, f64, f64, i32, i32, C.POINTER(SolveInfo)], i32),
    "hgb_csr_pattern_grad": ([vp, f64, vp, vp, vp], i32),
    "hgb_gmres_solve": ([vp, vp, vp, i32, vp, vp, f64, i32, C.POINTER(SolveInfo)], i32),
    "hgb_ru_pcg_solve": ([vp, vp, vp, vp, vp, vp, f64, f64, i32, C.POINTER(SolveInfo)], i32),
    "hgb_ru_pcg_solve_op": ([vp, vp, vp, vp, ch, vp, vp, f64, f64, i32, C.POINTER(SolveInfo)], i32),
    "hgb_ir_gmres_solve": ([vp, vp, vp, vp, i32, vp, vp, f64, f64, i32, i32, C.POINTER(SolveInfo)], i32),
    "hgb_mixed_cg_solve": ([vp, i32, i32, vp, vp, vp, vp, vp, vp, f64, i32, C.POINTER(SolveInfo)], i32),
    "hgb_mixed_ir_pcg_solve": ([vp, i32, i32, vp, vp, vp, vp, vp, vp, f64, f64, i32, i32, C.POINTER(SolveInfo)], i32),
    "hgb_mixed_ru_pcg_solve": ([vp, i32, i32, vp, vp, vp, vp, vp, vp, f64, f64, i32, C.POINTER(SolveInfo)], i32),
    "hgb_batch_create": ([vp, i32, vp, i32, i32, vp, vp, vp, C.POINTER(vp)], i32),
    "hgb_batch_set_config": ([vp, vp], i32),
    "hgb_batch_get_config": ([vp, vp], i32),
    "hgb_batch_cg_solve": ([vp, vp, vp, f64, f64, i32, i32, vp, vp], i32),
    "hgb_batch_autotune": ([vp, vp, vp, f64, C.c_char_p, vp], i32),
    "hgb_batch_destroy": ([vp], i32),
    "hgb_dot_f64_noalloc": ([i32, vp, vp, vp, vp], i32),
    "hgb_selftest_wait_timeout": ([vp, i32], i32),
}


def lib_path():
    return _build.LIB


def lib():
    """The loaded libhgb.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError(f"libhgb.so not built ({path}); run __graft_entry__.build() or "
                               "python -m hala_gb300.build")
        L = C.CDLL(path)
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(status, what=""):
    if status != HGB_OK:
        msg = lib().hgb_last_error().decode(errors="replace")
        raise HgbError(status, f"{what}: {msg}" if what else msg)
    return status


def ch_(c):
    return c.encode() if isinstance(c, str) else c
