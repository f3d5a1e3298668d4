"""The C ABI library builds, loads and exports every entry point include/hgb.h declares.
No compute call is made (this runs without a GPU)."""
import ctypes as C
import os
import re

from hala_gb300 import build, hgb

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "hgb.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hgb_\w+)\s*\(", src)))


def test_header_declares_the_path():
    names = declared_symbols()
    for must in ("hgb_spmv_f64", "hgb_ilu0_create", "hgb_ilu0_apply", "hgb_tri_solve", "hgb_cg_solve",
                 "hgb_gmres_solve", "hgb_ir_pcg_solve", "hgb_ir_gmres_solve", "hgb_ru_pcg_solve", "hgb_dot_f64", "hgb_nrm2_f64", "hgb_axpy_f64"):
        assert must in names


def test_library_exports_every_declared_symbol():
    build.build()
    lib = C.CDLL(build.LIB)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(declared_symbols()) <= set(hgb._SIGS)


def test_host_only_entry_points():
    L = hgb.lib()
    assert L.hgb_status_string(hgb.HGB_ERR_CSR) == b"HGB_ERR_CSR"
    assert L.hgb_version() == 10100
    # argument checks run before any device work
    assert L.hgb_ctx_create(0, None) == hgb.HGB_ERR_ARG
    assert b"null output" in L.hgb_last_error()


def test_solver_argument_checks_need_no_device():
    # null handles and out-of-range limits are rejected before any CUDA call, with a message
    L = hgb.lib()
    info = hgb.SolveInfo()
    cases = [
        (lambda: L.hgb_cg_solve(None, None, None, None, None, 1e-10, 10, C.byref(info)), b"cg_solve"),
        (lambda: L.hgb_gmres_solve(None, None, None, 30, None, None, 1e-10, 10, C.byref(info)), b"gmres"),
        (lambda: L.hgb_gmres_solve(None, None, None, 513, None, None, 1e-10, 10, C.byref(info)), b"restart"),
        (lambda: L.hgb_ru_pcg_solve(None, None, None, None, None, None, 1e-10, 0.01, 10, C.byref(info)),
         b"ru_pcg"),
        (lambda: L.hgb_ru_pcg_solve_op(None, None, None, None, b"T", None, None, 1e-10, 0.01, 10, C.byref(info)),
         b"ru_pcg"),
        (lambda: L.hgb_ir_pcg_solve(None, None, None, None, None, None, 1e-10, 1e-4, 10, 5, C.byref(info)),
         b"ir_pcg"),
        (lambda: L.hgb_ir_gmres_solve(None, None, None, None, 30, None, None, 1e-10, 1e-4, 10, 5, C.byref(info)),
         b"ir_gmres"),
        (lambda: L.hgb_cg_solve_nrhs(None, None, None, 2, None, None, 1e-10, 10, C.byref(info)), b"cg_solve_nrhs"),
    ]
    for call, what in cases:
        assert call() == hgb.HGB_ERR_ARG
        assert what in L.hgb_last_error(), what
