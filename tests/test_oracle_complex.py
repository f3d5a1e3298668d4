"""The complex (complex128 / complex64) CPU oracle pinned against the reference: the complex cases
of its own solver tests (tests/solvers_tests.hpp, instantiated on std::complex), the committed
complex fixtures (made by the reference's templates on std::complex, tests/golden/make_golden.py)
and, where it was built here, the reference's CPU path itself.  Oracle and reference perform the
same sequence of separately rounded complex operations, so the comparisons are bit for bit."""
import glob
import os

import numpy as np
import pytest

from hala_gb300 import problems as P
from oracle import oracle as O
from tests import refcases as R

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "cplx_*.npz")))
CTYPES = {"z": np.complex128, "c": np.complex64}
needs_ref = pytest.mark.skipif(not O.ref_available(), reason="reference CPU path not built here")


def same(a, b):
    """bit-identical complex arrays (signed zeros compare equal)"""
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


# ------------------------------------------------------- reference test golden values ---
@pytest.mark.parametrize("ct", [np.complex128, np.complex64])
def test_cg_golden_complex(ct):
    """test_cg<std::complex<T>> (solvers_tests.hpp:12-55): the tridiagonal case is exact in two
    iterations, the cyclic one converges from a given start"""
    tol_rel = 1e-14 if ct == np.complex128 else 1e-6
    c = R.TRIDIAG5
    v = c["vals"].astype(ct)
    b = (R.dense(c) @ R.XREF5).astype(ct)
    f, d, _ = O.zilu_factor(c["pntr"], c["indx"], v)
    x, it, _ = O.zcg(c["pntr"], c["indx"], v, b, max_iter=2, diag=d, ilu=f)
    assert it == 2 and np.linalg.norm(x - R.XREF5) <= tol_rel * 10 * np.linalg.norm(R.XREF5)
    c = R.CYCLIC5
    v = c["vals"].astype(ct)
    b = (R.dense(c) @ R.XREF5).astype(ct)
    f, d, _ = O.zilu_factor(c["pntr"], c["indx"], v)
    tol = 1e-9 if ct == np.complex128 else 1e-4
    x, it, _ = O.zcg(c["pntr"], c["indx"], v, b, x0=R.CG_X0, tol=tol, diag=d, ilu=f)
    assert np.linalg.norm(x - R.XREF5) <= 10 * tol * np.linalg.norm(R.XREF5)


@pytest.mark.parametrize("ct", [np.complex128, np.complex64])
def test_gmres_golden_complex(ct):
    """test_gmres<std::complex<T>> (solvers_tests.hpp:105-137)"""
    tol_rel = 1e-12 if ct == np.complex128 else 1e-5
    c = R.TRIDIAG5
    v = c["vals"].astype(ct)
    b = (R.dense(c) @ R.XREF5).astype(ct)
    f, d, _ = O.zilu_factor(c["pntr"], c["indx"], v)
    x, _ = O.zgmres(c["pntr"], c["indx"], v, b, 2, max_iter=2, diag=d, ilu=f)
    assert np.linalg.norm(x - R.XREF5) <= tol_rel * np.linalg.norm(R.XREF5)
    c = R.NONSYM5
    v = c["vals"].astype(ct)
    b = (R.dense(c) @ R.XREF5).astype(ct)
    f, d, _ = O.zilu_factor(c["pntr"], c["indx"], v)
    tol = 1e-9 if ct == np.complex128 else 1e-4
    x, _ = O.zgmres(c["pntr"], c["indx"], v, b, 6, tol=tol, diag=d, ilu=f)
    assert np.linalg.norm(x - R.XREF5) <= 100 * tol * np.linalg.norm(R.XREF5)


def test_magnetic_laplacian_is_hermitian_positive_definite():
    p, i, v = P.magnetic2d(8)
    A = P.csr_to_dense(p, i, v)
    assert np.array_equal(A, A.conj().T) and np.linalg.eigvalsh(A).min() > 0


# ----------------------------------------------------------------- committed fixtures ---
@pytest.mark.parametrize("s", ["z", "c"])
@pytest.mark.parametrize("path", FIXTURES)
def test_complex_oracle_matches_fixture(path, s):
    g = np.load(path)
    ct = CTYPES[s]
    p, i = g["pntr"], g["indx"]
    v, x, y0 = g["vals"].astype(ct), g["x"].astype(ct), g["y0"].astype(ct)
    n = len(p) - 1
    alpha, beta = complex(g["alpha"]), complex(g["beta"])
    f, d, st = O.zilu_factor(p, i, v)
    assert st == 0 and np.array_equal(d, g["diag"])
    assert same(f, g[f"ilu_{s}"])
    assert same(O.zilu_apply(p, i, d, f, x), g[f"apply_{s}"])
    for t in "NTC":
        assert same(O.zspmv(t, n, n, alpha, p, i, v, x, beta, y0), g[f"spmv_{t.lower()}_{s}"]), t
    b = g[f"b_{s}"]
    if bool(g["hpd"]):
        xo, it, _ = O.zcg(p, i, v, b, tol=float(g[f"cg_tol_{s}"]), max_iter=2000, diag=d, ilu=f)
        assert it == int(g[f"cg_iters_{s}"]) and same(xo, g[f"cg_x_{s}"])
    xo, it = O.zgmres(p, i, v, b, 30, tol=float(g[f"gmres_tol_{s}"]), max_iter=200, diag=d, ilu=f)
    assert it == int(g[f"gmres_iters_{s}"]) and same(xo, g[f"gmres_x_{s}"])


# ------------------------------------------------------------ the reference build -------
def _random_complex(rng, n, ct):
    p, i, v = P.random_csr(n, 0.05, rng)
    vz = v + 1j * rng.uniform(-1, 1, len(v))
    return p, i, vz.astype(ct)


@needs_ref
@pytest.mark.parametrize("ct", [np.complex128, np.complex64])
def test_complex_trsv_matches_reference_build(rng, ct):
    r, s = O.zref(ct)
    p, i, v = _random_complex(rng, 60, ct)
    n = len(p) - 1
    d = O.diag_index(p, i)
    up, ui, lp, li = O.split_pattern(p, i, d)
    L = np.concatenate([v[p[k]:d[k] + 1] for k in range(n)])
    U = np.concatenate([v[d[k]:p[k + 1]] for k in range(n)])
    b = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(ct)
    for (tp, ti, tv, uplo) in ((lp, li, L, "L"), (up, ui, U, "U")):
        tv = np.ascontiguousarray(tv)
        for diagc in "NU":
            for t in "NTC":
                xo = O.ztrsv(uplo, diagc, t, 0.5, tp, ti, tv, b)
                xr = np.zeros(n, ct)
                getattr(r, f"ref_trsv_{s}")(uplo.encode(), diagc.encode(), t.encode(), n, 0.5, tp.ctypes.data,
                                            ti.ctypes.data, tv.ctypes.data, b.ctypes.data, xr.ctypes.data)
                assert same(xo, xr), (uplo, diagc, t)


@needs_ref
@pytest.mark.parametrize("ct", [np.complex128, np.complex64])
def test_complex_solvers_match_reference_build(rng, ct):
    r, s = O.zref(ct)
    p, i, v = P.magnetic2d(9, flux=0.7, shift=0.3)
    v = v.astype(ct)
    n = len(p) - 1
    f, d, _ = O.zilu_factor(p, i, v)
    b = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(ct)
    tol = (1e-10 if ct == np.complex128 else 1e-4) * float(np.linalg.norm(b))
    xo, ito, _ = O.zcg(p, i, v, b, tol=tol, max_iter=500, diag=d, ilu=f)
    xr = np.zeros(n, ct)
    itr = getattr(r, f"ref_solve_cg_{s}")(n, p.ctypes.data, i.ctypes.data, v.ctypes.data, d.ctypes.data,
                                          f.ctypes.data, b.ctypes.data, xr.ctypes.data, tol, 500)
    assert ito == itr and same(xo, xr)
    for restart, max_iter in ((5, 3), (20, 4)):
        xo, ito = O.zgmres(p, i, v, b, restart, tol=tol, max_iter=max_iter, diag=d, ilu=f)
        xr = np.zeros(n, ct)
        itr = getattr(r, f"ref_solve_gmres_{s}")(n, p.ctypes.data, i.ctypes.data, v.ctypes.data, d.ctypes.data,
                                                 f.ctypes.data, restart, b.ctypes.data, xr.ctypes.data, tol, max_iter)
        assert ito == itr and same(xo, xr), restart


@needs_ref
def test_complex_ilu_apply_t_is_the_transposed_inverse(rng):
    """(LU)^-T and (LU)^-H of the oracle against dense inverses of the reference's factor"""
    p, i, v = _random_complex(rng, 50, np.complex128)
    n = len(p) - 1
    r, s = O.zref(np.complex128)
    f = np.zeros_like(v)
    r.ref_factorize_ilu_z(n, p.ctypes.data, i.ctypes.data, v.ctypes.data, f.ctypes.data)
    d = O.diag_index(p, i)
    F = P.csr_to_dense(p, i, f)
    Lm = np.tril(F, -1) + np.eye(n)
    Um = np.triu(F)
    M = Lm @ Um
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for t, Mt in (("T", M.T), ("C", M.conj().T)):
        y = O.zilu_apply(p, i, d, f, x, trans=t)
        assert np.linalg.norm(Mt @ y - x) <= 1e-12 * np.linalg.norm(x)
