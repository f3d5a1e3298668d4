"""numpy front-end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads ``oracle/_build/liboracle.so`` (the C restatement in hala_oracle.c) and, when it was built
in a container that holds the reference sources, ``oracle/_ref/libhalaref.so`` (the reference's
own CPU templates, see oracle/ref/).  Only tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline leg import this module; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libhalaref.so")

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_u16p = np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS")


def build():
    """Compile the C restatement (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def _load():
    if not os.path.exists(LIB_PATH):
        build()
    lib = C.CDLL(LIB_PATH)
    i, c, vp = C.c_int, C.c_char, C.c_void_p
    lib.or_diag_index.argtypes = [i, _i32p, _i32p, _i32p]
    lib.or_diag_index.restype = i
    lib.or_split_pattern.argtypes = [i, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p]
    lib.or_levels.argtypes = [i, _i32p, _i32p, _i32p, c, _i32p]
    lib.or_levels.restype = i
    lib.or_ilu_factor_pivot_d.argtypes = [i, _i32p, _i32p, _i32p, _f64p]
    lib.or_ilu_apply_mixed.argtypes = [i, _i32p, _i32p, _i32p, _f32p, _f64p, _f32p]
    lib.or_spmv_bf16f32.argtypes = [c, i, i, C.c_float, _i32p, _i32p, _u16p, _f32p, C.c_float, _f32p]
    for s, fp, ft in (("d", _f64p, C.c_double), ("f", _f32p, C.c_float)):
        getattr(lib, f"or_spmv_{s}").argtypes = [c, i, i, ft, _i32p, _i32p, fp, fp, ft, fp]
        getattr(lib, f"or_split_values_{s}").argtypes = [c, c, i, _i32p, fp, _i32p, _i32p, fp, fp]
        getattr(lib, f"or_ilu_factor_{s}").argtypes = [i, _i32p, _i32p, _i32p, fp]
        getattr(lib, f"or_ilu_factor_{s}").restype = i
        getattr(lib, f"or_ilu_apply_{s}").argtypes = [i, _i32p, _i32p, _i32p, fp, fp]
        getattr(lib, f"or_ilu_apply_t_{s}").argtypes = [i, _i32p, _i32p, _i32p, fp, fp]
        getattr(lib, f"or_trsv_{s}").argtypes = [c, c, c, i, ft, _i32p, _i32p, fp, fp, fp]
        getattr(lib, f"or_dot_{s}").argtypes = [i, fp, fp]
        getattr(lib, f"or_dot_{s}").restype = ft
        getattr(lib, f"or_nrm2_{s}").argtypes = [i, fp]
        getattr(lib, f"or_nrm2_{s}").restype = ft
        getattr(lib, f"or_cg_{s}").argtypes = [i, _i32p, _i32p, fp, vp, vp, fp, fp, ft, i, C.POINTER(ft)]
        getattr(lib, f"or_cg_{s}").restype = i
        getattr(lib, f"or_batch_cg_{s}").argtypes = [i, _i32p, _i32p, fp, vp, vp, i, fp, fp, ft, i, C.POINTER(ft)]
        getattr(lib, f"or_batch_cg_{s}").restype = i
        getattr(lib, f"or_gmres_{s}").argtypes = [i, _i32p, _i32p, fp, vp, vp, i, fp, fp, ft, i]
        getattr(lib, f"or_gmres_{s}").restype = i
    lib.or_ir_pcg.argtypes = [i, _i32p, _i32p, _f64p, _f32p, _i32p, _f32p, _f64p, _f64p, _f64p,
                              C.c_double, C.c_double, i, i, C.POINTER(i)]
    lib.or_ir_pcg.restype = i
    lib.or_ir_gmres.argtypes = [i, _i32p, _i32p, _f64p, _f32p, _i32p, _f32p, _f64p, i, _f64p, _f64p,
                                C.c_double, C.c_double, i, i, C.POINTER(i)]
    lib.or_ir_gmres.restype = i
    lib.or_ru_pcg.argtypes = [i, _i32p, _i32p, _f64p, _f32p, _i32p, _f32p, _f64p, _f64p, _f64p,
                              C.c_double, C.c_double, i, C.POINTER(i)]
    lib.or_ru_pcg.restype = i
    return lib


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = _load()
    return _lib


def _sfx(dtype):
    return "d" if np.dtype(dtype) == np.float64 else "f"


def _b(ch):
    return ch.encode() if isinstance(ch, str) else ch


def diag_index(pntr, indx):
    n = len(pntr) - 1
    d = np.zeros(n, np.int32)
    st = lib().or_diag_index(n, pntr, indx, d)
    if st != 0:
        raise ValueError(f"row {-st - 1} has no diagonal entry")
    return d


def split_pattern(pntr, indx, diag):
    n = len(pntr) - 1
    nnz = int(pntr[-1])
    up = np.zeros(n + 1, np.int32); lp = np.zeros(n + 1, np.int32)
    ui = np.zeros(nnz + n, np.int32); li = np.zeros(nnz + n, np.int32)
    lib().or_split_pattern(n, pntr, indx, diag, up, ui, lp, li)
    return up, ui[: up[-1]].copy(), lp, li[: lp[-1]].copy()


def split_values(uplo, diagc, pntr, vals, up, lp):
    n = len(pntr) - 1
    uv = np.zeros(int(up[-1]), vals.dtype); lv = np.zeros(int(lp[-1]), vals.dtype)
    getattr(lib(), f"or_split_values_{_sfx(vals.dtype)}")(_b(uplo), _b(diagc), n, pntr, vals, up, lp, uv, lv)
    return uv, lv


def levels(pntr, indx, diag, uplo):
    n = len(pntr) - 1
    lev = np.zeros(n, np.int32)
    nl = lib().or_levels(n, pntr, indx, diag, _b(uplo), lev)
    return lev, nl


def spmv(trans, m, ncols, alpha, pntr, indx, vals, x, beta, y=None):
    out_len = m if trans in ("N", "n") else ncols
    y = np.zeros(out_len, vals.dtype) if y is None else np.array(y, vals.dtype)
    getattr(lib(), f"or_spmv_{_sfx(vals.dtype)}")(_b(trans), m, ncols, alpha, pntr, indx, vals,
                                                  np.ascontiguousarray(x, vals.dtype), beta, y)
    return y


def spmv_bf16f32(trans, m, ncols, alpha, pntr, indx, vals_bf16, x, beta, y=None):
    out_len = m if trans in ("N", "n") else ncols
    y = np.zeros(out_len, np.float32) if y is None else np.array(y, np.float32)
    lib().or_spmv_bf16f32(_b(trans), m, ncols, alpha, pntr, indx, vals_bf16,
                          np.ascontiguousarray(x, np.float32), beta, y)
    return y


def f32_to_bf16(a):
    """Round-to-nearest-even float32 -> bfloat16 bit pattern (uint16), vectorised."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    nan = (u & 0x7FFFFFFF) > 0x7F800000
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    r[nan] = ((u[nan] >> 16) | 0x40).astype(np.uint16)
    return r


def bf16_to_f32(b):
    return (np.asarray(b, np.uint16).astype(np.uint32) << 16).view(np.float32)


def ilu_factor(pntr, indx, vals, diag=None):
    """Row-wise restatement of factorize_ilu (bit-identical to the reference loop)."""
    diag = diag_index(pntr, indx) if diag is None else diag
    n = len(pntr) - 1
    f = np.array(vals, copy=True)
    st = getattr(lib(), f"or_ilu_factor_{_sfx(vals.dtype)}")(n, pntr, indx, diag, f)
    return f, diag, st


def ilu_factor_pivot(pntr, indx, vals, diag):
    """The reference's own O(n^2) loop, restated (small n only)."""
    f = np.array(vals, np.float64, copy=True)
    lib().or_ilu_factor_pivot_d(len(pntr) - 1, pntr, indx, diag, f)
    return f


def ilu_apply(pntr, indx, diag, ilu, x, trans="N"):
    n = len(pntr) - 1
    y = np.array(x, ilu.dtype, copy=True)
    fn = "or_ilu_apply_" if trans in ("N", "n") else "or_ilu_apply_t_"
    getattr(lib(), fn + _sfx(ilu.dtype))(n, pntr, indx, diag, ilu, y)
    return y


def ilu_apply_mixed(pntr, indx, diag, ilu32, piv, x):
    """FP32 factor with FP64 pivots (the inner preconditioner of ir_pcg)."""
    y = np.array(x, np.float32, copy=True)
    lib().or_ilu_apply_mixed(len(pntr) - 1, pntr, indx, diag, np.ascontiguousarray(ilu32, np.float32),
                             np.ascontiguousarray(piv, np.float64), y)
    return y


def trsv(uplo, diagc, trans, alpha, pntr, indx, vals, b):
    n = len(pntr) - 1
    x = np.zeros(n, vals.dtype)
    getattr(lib(), f"or_trsv_{_sfx(vals.dtype)}")(_b(uplo), _b(diagc), _b(trans), n, alpha, pntr,
                                                  indx, vals, np.ascontiguousarray(b, vals.dtype), x)
    return x


def dot(x, y):
    return getattr(lib(), f"or_dot_{_sfx(x.dtype)}")(len(x), x, np.ascontiguousarray(y, x.dtype))


def nrm2(x):
    return getattr(lib(), f"or_nrm2_{_sfx(x.dtype)}")(len(x), x)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def cg(pntr, indx, vals, b, x0=None, tol=0.0, max_iter=2**31 - 1, diag=None, ilu=None):
    """solve_cg / solve_cg_ilu restated.  Returns (x, iterations, final ||r||)."""
    n = len(pntr) - 1
    x = np.zeros(n, vals.dtype) if x0 is None else np.array(x0, vals.dtype, copy=True)
    ft = C.c_double if vals.dtype == np.float64 else C.c_float
    res = ft(0)
    it = getattr(lib(), f"or_cg_{_sfx(vals.dtype)}")(n, pntr, indx, vals, _ptr(diag), _ptr(ilu),
                                                     np.ascontiguousarray(b, vals.dtype), x, tol,
                                                     max_iter, C.byref(res))
    return x, it, res.value


def batch_cg(pntr, indx, vals, B, nrhs, X0=None, tol=0.0, max_iter=2**31 - 1, diag=None, ilu=None):
    """solve_batch_cg / solve_batch_cg_ilu restated (B, X: n x nrhs column-major, flattened).
    Returns (X, iterations, final batch_max_norm2(r))."""
    n = len(pntr) - 1
    X = np.zeros(n * nrhs, vals.dtype) if X0 is None else np.array(X0, vals.dtype, copy=True).reshape(-1)
    ft = C.c_double if vals.dtype == np.float64 else C.c_float
    res = ft(0)
    it = getattr(lib(), f"or_batch_cg_{_sfx(vals.dtype)}")(n, pntr, indx, vals, _ptr(diag), _ptr(ilu), nrhs,
                                                           np.ascontiguousarray(B, vals.dtype).reshape(-1), X,
                                                           tol, max_iter, C.byref(res))
    return X, it, res.value


def gmres(pntr, indx, vals, b, restart, x0=None, tol=0.0, max_iter=2**31 - 1, diag=None, ilu=None):
    """solve_gmres / solve_gmres_ilu restated.  Returns (x, total applications)."""
    n = len(pntr) - 1
    x = np.zeros(n, vals.dtype) if x0 is None else np.array(x0, vals.dtype, copy=True)
    it = getattr(lib(), f"or_gmres_{_sfx(vals.dtype)}")(n, pntr, indx, vals, _ptr(diag), _ptr(ilu),
                                                        restart, np.ascontiguousarray(b, vals.dtype),
                                                        x, tol, max_iter)
    return x, it


def ir_pcg(pntr, indx, vals, vals32, diag, ilu32, piv, b, tol, inner_rtol=1e-4, max_inner=100000,
           max_outer=50, x0=None):
    n = len(pntr) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64, copy=True)
    outer = C.c_int(0)
    tot = lib().or_ir_pcg(n, pntr, indx, vals, vals32, diag, ilu32, piv, b, x, tol, inner_rtol,
                          max_inner, max_outer, C.byref(outer))
    return x, tot, outer.value


def ru_pcg(pntr, indx, vals, vals32, diag, ilu32, piv, b, tol, delta=0.1, max_iter=100000, x0=None):
    """Mixed FP32 ILU(0)-PCG with FP64 reliable updates (no reference counterpart).
    Returns (x, iterations, reliable updates)."""
    n = len(pntr) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64, copy=True)
    upd = C.c_int(0)
    it = lib().or_ru_pcg(n, pntr, indx, vals, vals32, diag, ilu32, piv, b, x, tol, delta, max_iter,
                         C.byref(upd))
    return x, it, upd.value


def ir_gmres(pntr, indx, vals, vals32, diag, ilu32, piv, restart, b, tol, inner_rtol=1e-4, max_inner=3000,
             max_outer=50, x0=None):
    """Mixed FP32-inner / FP64-refined GMRES(restart) (no reference counterpart).
    Returns (x, total inner applications, sweeps)."""
    n = len(pntr) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64, copy=True)
    outer = C.c_int(0)
    tot = lib().or_ir_gmres(n, pntr, indx, vals, vals32, diag, ilu32, piv, restart, b, x, tol, inner_rtol,
                            max_inner, max_outer, C.byref(outer))
    return x, tot, outer.value


# ---------------------------------------------------------------- reference (oracle/_ref) ---

_ref = None


def ref_available():
    return os.path.exists(REF_PATH)


def ref():
    """The reference's own CPU templates (oracle/_ref/libhalaref.so), or None when not built."""
    global _ref
    if _ref is None and ref_available():
        r = C.CDLL(REF_PATH)
        i, c, vp = C.c_int, C.c_char, C.c_void_p
        r.ref_sparse_gemv_d.argtypes = [c, i, i, C.c_double, _i32p, _i32p, _f64p, _f64p, C.c_double, _f64p]
        r.ref_sparse_gemv_f.argtypes = [c, i, i, C.c_float, _i32p, _i32p, _f32p, _f32p, C.c_float, _f32p]
        r.ref_get_diagonal_index.argtypes = [i, _i32p, _i32p, _i32p]
        r.ref_split_pattern.argtypes = [i, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p,
                                        C.POINTER(i), C.POINTER(i)]
        r.ref_split_values_d.argtypes = [c, c, i, _i32p, _f64p, _i32p, _i32p, _f64p, _f64p]
        r.ref_factorize_ilu_d.argtypes = [i, _i32p, _i32p, _f64p, _f64p]
        r.ref_factorize_ilu_f.argtypes = [i, _i32p, _i32p, _f32p, _f32p]
        r.ref_apply_ilu_d.argtypes = [i, _i32p, _i32p, _i32p, _f64p, _f64p]
        r.ref_apply_ilu_f.argtypes = [i, _i32p, _i32p, _i32p, _f32p, _f32p]
        r.ref_trsv_d.argtypes = [c, c, c, i, C.c_double, _i32p, _i32p, _f64p, _f64p, _f64p]
        r.ref_solve_cg_d.argtypes = [i, _i32p, _i32p, _f64p, vp, vp, _f64p, _f64p, C.c_double, i]
        r.ref_solve_cg_d.restype = i
        r.ref_solve_cg_f.argtypes = [i, _i32p, _i32p, _f32p, vp, vp, _f32p, _f32p, C.c_float, i]
        r.ref_solve_cg_f.restype = i
        r.ref_solve_gmres_d.argtypes = [i, _i32p, _i32p, _f64p, vp, vp, i, _f64p, _f64p, C.c_double, i]
        r.ref_solve_gmres_d.restype = i
        r.ref_solve_gmres_f.argtypes = [i, _i32p, _i32p, _f32p, vp, vp, i, _f32p, _f32p, C.c_float, i]
        r.ref_solve_gmres_f.restype = i
        r.ref_solve_batch_cg_ilu_d.argtypes = [i, _i32p, _i32p, _f64p, i, _f64p, _f64p, C.c_double, i]
        r.ref_solve_batch_cg_ilu_d.restype = i
        _ref = r
    return _ref


# ------------------------------------------------------------------------------ complex -----
# C128 (numpy complex128) and C64 (complex64) through hala_oracle_cplx.c (suffix z / c) and, when
# built, the reference's templates on std::complex (ref_*_z / ref_*_c in oracle/ref/ref_shim.cpp).

def _zs(dtype):
    dt = np.dtype(dtype)
    if dt == np.complex128:
        return "z", C.c_double, np.float64
    if dt == np.complex64:
        return "c", C.c_float, np.float32
    raise TypeError(f"complex oracle: {dt}")


def _vp(a):
    return a.ctypes.data_as(C.c_void_p)


def _pair(v, rt):
    v = complex(v)
    return np.array([v.real, v.imag], rt)


def _zbind(lib_, prefix, s, rt):
    """argtypes of the complex entry points named prefix + name + '_' + s."""
    i, c, vp = C.c_int, C.c_char, C.c_void_p
    sigs = {
        "spmv": ([c, i, i, vp, vp, vp, vp, vp, vp, vp], None),
        "ilu_factor": ([i, vp, vp, vp, vp], i),
        "ilu_apply": ([i, vp, vp, vp, vp, vp], None),
        "ilu_apply_t": ([c, i, vp, vp, vp, vp, vp], None),
        "trsv": ([c, c, c, i, rt, vp, vp, vp, vp, vp], None),
        "dotc": ([i, vp, vp, vp], None),
        "nrm2": ([i, vp], rt),
        "cg": ([i, vp, vp, vp, vp, vp, vp, vp, rt, i, C.POINTER(rt)], i),
        "gmres": ([i, vp, vp, vp, vp, vp, i, vp, vp, rt, i], i),
    }
    for name, (args, res) in sigs.items():
        f = getattr(lib_, f"{prefix}{name}_{s}")
        f.argtypes, f.restype = args, res


_zbound = set()


def _zlib(dtype):
    s, rt, rnp = _zs(dtype)
    L = lib()
    if s not in _zbound:
        _zbind(L, "or_", s, rt)
        _zbound.add(s)
    return L, s, rt, rnp


def _i32(a):
    return np.ascontiguousarray(a, np.int32)


def zspmv(trans, m, ncols, alpha, pntr, indx, vals, x, beta, y=None):
    L, s, rt, rnp = _zlib(vals.dtype)
    out_len = m if trans in ("N", "n") else ncols
    y = np.zeros(out_len, vals.dtype) if y is None else np.array(y, vals.dtype)
    p, ix, v, xx = _i32(pntr), _i32(indx), np.ascontiguousarray(vals), np.ascontiguousarray(x, vals.dtype)
    a, b = _pair(alpha, rnp), _pair(beta, rnp)
    getattr(L, f"or_spmv_{s}")(_b(trans), m, ncols, _vp(a), _vp(p), _vp(ix), _vp(v), _vp(xx), _vp(b), _vp(y))
    return y


def zilu_factor(pntr, indx, vals, diag=None):
    """factorize_ilu_array on complex values.  Returns (factor, diag, first zero pivot row + 1 or 0)."""
    L, s, rt, rnp = _zlib(vals.dtype)
    diag = diag_index(_i32(pntr), _i32(indx)) if diag is None else _i32(diag)
    p, ix = _i32(pntr), _i32(indx)
    f = np.array(vals, copy=True)
    st = getattr(L, f"or_ilu_factor_{s}")(len(p) - 1, _vp(p), _vp(ix), _vp(diag), _vp(f))
    return f, diag, st


def zilu_apply(pntr, indx, diag, ilu, x, trans="N"):
    L, s, rt, rnp = _zlib(ilu.dtype)
    p, ix, d = _i32(pntr), _i32(indx), _i32(diag)
    f = np.ascontiguousarray(ilu)
    y = np.array(x, ilu.dtype, copy=True)
    if trans in ("N", "n"):
        getattr(L, f"or_ilu_apply_{s}")(len(p) - 1, _vp(p), _vp(ix), _vp(d), _vp(f), _vp(y))
    else:
        getattr(L, f"or_ilu_apply_t_{s}")(_b(trans), len(p) - 1, _vp(p), _vp(ix), _vp(d), _vp(f), _vp(y))
    return y


def ztrsv(uplo, diagc, trans, alpha, pntr, indx, vals, b):
    L, s, rt, rnp = _zlib(vals.dtype)
    p, ix, v = _i32(pntr), _i32(indx), np.ascontiguousarray(vals)
    bb = np.ascontiguousarray(b, vals.dtype)
    x = np.zeros(len(p) - 1, vals.dtype)
    getattr(L, f"or_trsv_{s}")(_b(uplo), _b(diagc), _b(trans), len(p) - 1, float(alpha), _vp(p), _vp(ix), _vp(v),
                               _vp(bb), _vp(x))
    return x


def zdotc(x, y):
    L, s, rt, rnp = _zlib(x.dtype)
    xx, yy = np.ascontiguousarray(x), np.ascontiguousarray(y, x.dtype)
    out = np.zeros(2, rnp)
    getattr(L, f"or_dotc_{s}")(len(xx), _vp(xx), _vp(yy), _vp(out))
    return complex(out[0], out[1])


def znrm2(x):
    L, s, rt, rnp = _zlib(x.dtype)
    xx = np.ascontiguousarray(x)
    return getattr(L, f"or_nrm2_{s}")(len(xx), _vp(xx))


def _opt(a):
    return None if a is None else _vp(a)


def zcg(pntr, indx, vals, b, x0=None, tol=0.0, max_iter=2**31 - 1, diag=None, ilu=None):
    """solve_cg / solve_cg_ilu on complex data.  Returns (x, iterations, final ||r||)."""
    L, s, rt, rnp = _zlib(vals.dtype)
    p, ix, v = _i32(pntr), _i32(indx), np.ascontiguousarray(vals)
    n = len(p) - 1
    x = np.zeros(n, vals.dtype) if x0 is None else np.array(x0, vals.dtype, copy=True)
    bb = np.ascontiguousarray(b, vals.dtype)
    d = None if diag is None else _i32(diag)
    f = None if ilu is None else np.ascontiguousarray(ilu, vals.dtype)
    res = rt(0)
    it = getattr(L, f"or_cg_{s}")(n, _vp(p), _vp(ix), _vp(v), _opt(d), _opt(f), _vp(bb), _vp(x), tol, max_iter,
                                  C.byref(res))
    return x, it, res.value


def zgmres(pntr, indx, vals, b, restart, x0=None, tol=0.0, max_iter=2**31 - 1, diag=None, ilu=None):
    """solve_gmres / solve_gmres_ilu on complex data.  Returns (x, total applications)."""
    L, s, rt, rnp = _zlib(vals.dtype)
    p, ix, v = _i32(pntr), _i32(indx), np.ascontiguousarray(vals)
    n = len(p) - 1
    x = np.zeros(n, vals.dtype) if x0 is None else np.array(x0, vals.dtype, copy=True)
    bb = np.ascontiguousarray(b, vals.dtype)
    d = None if diag is None else _i32(diag)
    f = None if ilu is None else np.ascontiguousarray(ilu, vals.dtype)
    it = getattr(L, f"or_gmres_{s}")(n, _vp(p), _vp(ix), _vp(v), _opt(d), _opt(f), restart, _vp(bb), _vp(x), tol,
                                     max_iter)
    return x, it


_zref_bound = set()


def zref(dtype):
    """(library, suffix) of the reference's complex templates, or None when not built."""
    r = ref()
    if r is None:
        return None
    s, rt, rnp = _zs(dtype)
    if s not in _zref_bound:
        i, c, vp = C.c_int, C.c_char, C.c_void_p
        getattr(r, f"ref_sparse_gemv_{s}").argtypes = [c, i, i, vp, vp, vp, vp, vp, vp, vp]
        getattr(r, f"ref_factorize_ilu_{s}").argtypes = [i, vp, vp, vp, vp]
        getattr(r, f"ref_apply_ilu_{s}").argtypes = [i, vp, vp, vp, vp, vp]
        getattr(r, f"ref_trsv_{s}").argtypes = [c, c, c, i, rt, vp, vp, vp, vp, vp]
        getattr(r, f"ref_solve_cg_{s}").argtypes = [i, vp, vp, vp, vp, vp, vp, vp, rt, i]
        getattr(r, f"ref_solve_cg_{s}").restype = i
        getattr(r, f"ref_solve_gmres_{s}").argtypes = [i, vp, vp, vp, vp, vp, i, vp, vp, rt, i]
        getattr(r, f"ref_solve_gmres_{s}").restype = i
        _zref_bound.add(s)
    return r, s
