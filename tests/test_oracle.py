"""The CPU oracle pinned against the reference: its tests' golden values, its compiled CPU path
(oracle/_ref, when built in this container) and the committed fixtures in tests/golden/."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O
from hala_gb300 import problems as P
from tests import refcases as R

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


# ------------------------------------------------------- reference test golden values ---
def test_ilu_golden():
    c = R.ILU3
    d = O.diag_index(c["pntr"], c["indx"])
    assert np.array_equal(d, c["diag"])
    f, _, st = O.ilu_factor(c["pntr"], c["indx"], c["vals"], d)
    assert st == 0 and R.testvec(f, c["ilu"])
    assert R.testvec(O.ilu_apply(c["pntr"], c["indx"], d, f, c["x"]), c["apply"])
    # the O(n^2) pivot loop of the reference gives the same bits
    assert np.array_equal(O.ilu_factor_pivot(c["pntr"], c["indx"], c["vals"], d), f)


def test_split_golden():
    c = R.SPLIT6
    d = O.diag_index(c["pntr"], c["indx"])
    assert np.array_equal(d, c["diag"])
    up, ui, lp, li = O.split_pattern(c["pntr"], c["indx"], d)
    for got, ref in ((up, "up"), (ui, "ui"), (lp, "lp"), (li, "li")):
        assert np.array_equal(got, c[ref]), ref
    uv, lv = O.split_values("U", "N", c["pntr"], c["vals"], up, lp)
    assert R.testvec(uv, c["uv"]) and R.testvec(lv, c["lv"])


def test_trsv_golden():
    X = R.TRSV_X
    L = R.TRSV_L
    B = 2.0 * R.TRSV_A @ X
    assert R.testvec(O.trsv("L", "N", "N", 0.5, L["pntr"], L["indx"], L["vals"], B), X)
    B = 2.0 * R.TRSV_A.T @ X
    assert R.testvec(O.trsv("L", "N", "T", 0.5, L["pntr"], L["indx"], L["vals"], B), X)
    B = 2.0 * R.TRSV_AU @ X
    assert R.testvec(O.trsv("L", "U", "N", 0.5, L["pntr"], L["indx"], R.TRSV_LU_VALS, B), X)
    U = R.TRSV_U
    B = 2.0 * R.TRSV_A.T @ X
    assert R.testvec(O.trsv("U", "N", "N", 0.5, U["pntr"], U["indx"], U["vals"], B), X)
    B = 2.0 * R.TRSV_A @ X
    assert R.testvec(O.trsv("U", "N", "T", 0.5, U["pntr"], U["indx"], U["vals"], B), X)


def test_spmv_golden():
    c = R.TRIDIAG5
    A = R.dense(c)
    x = R.make_vector(-1, 5)
    for t, M in (("N", A), ("T", A.T), ("C", A.T)):
        assert R.testvec(O.spmv(t, 5, 5, 2.0, c["pntr"], c["indx"], c["vals"], x, 0.0), 2.0 * M @ x)
    # cuda_sparse_tests.hpp sparse_matvec: x = {1..5}
    x = R.D(1, 2, 3, 4, 5)
    assert R.testvec(O.spmv("N", 5, 5, 2.0, c["pntr"], c["indx"], c["vals"], x, 0.0), 2.0 * A @ x)


def test_cg_golden():
    c = R.TRIDIAG5
    b = R.dense(c) @ R.XREF5
    f, d, _ = O.ilu_factor(c["pntr"], c["indx"], c["vals"])
    # stop_criteria(2): ILU is exact on a tridiagonal matrix, two iterations reach the solution
    x, it, _ = O.cg(c["pntr"], c["indx"], c["vals"], b, max_iter=2, diag=d, ilu=f)
    assert it == 2 and R.testvec(x, R.XREF5)
    c = R.CYCLIC5
    b = R.dense(c) @ R.XREF5
    f, d, _ = O.ilu_factor(c["pntr"], c["indx"], c["vals"])
    x, it, _ = O.cg(c["pntr"], c["indx"], c["vals"], b, x0=R.CG_X0, tol=1e-9, diag=d, ilu=f)
    assert R.testvec(x, R.XREF5, np.linalg.norm(R.XREF5))


def test_gmres_golden():
    c = R.TRIDIAG5
    b = R.dense(c) @ R.XREF5
    f, d, _ = O.ilu_factor(c["pntr"], c["indx"], c["vals"])
    x, it = O.gmres(c["pntr"], c["indx"], c["vals"], b, 2, max_iter=2, diag=d, ilu=f)
    assert R.testvec(x, R.XREF5)
    c = R.NONSYM5
    b = R.dense(c) @ R.XREF5
    f, d, _ = O.ilu_factor(c["pntr"], c["indx"], c["vals"])
    x, it = O.gmres(c["pntr"], c["indx"], c["vals"], b, 6, tol=1e-9, diag=d, ilu=f)
    assert R.testvec(x, R.XREF5)


# ---------------------------------------------------------- restatement invariants ------
def test_row_wise_ilu_equals_pivot_loop(rng):
    for _ in range(5):
        p, i, v = P.random_csr(60, 0.08, rng)
        d = O.diag_index(p, i)
        f, _, _ = O.ilu_factor(p, i, v, d)
        assert np.array_equal(O.ilu_factor_pivot(p, i, v, d).view(np.uint64), f.view(np.uint64))


def test_levels_definition():
    p, i, v = P.aniso3d(6, 5, 4)
    d = O.diag_index(p, i)
    lev, nl = O.levels(p, i, d, "L")
    idx = np.arange(len(p) - 1)
    ix, iy, iz = idx % 6, (idx // 6) % 5, idx // 30
    assert np.array_equal(lev, ix + iy + iz) and nl == 6 + 5 + 4 - 2
    levu, nlu = O.levels(p, i, d, "U")
    assert np.array_equal(levu, (5 - ix) + (4 - iy) + (3 - iz)) and nlu == nl


def test_transposed_apply_is_adjoint(rng):
    p, i, v = P.convdiff3d(5)
    f, d, _ = O.ilu_factor(p, i, v)
    n = len(p) - 1
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    lhs = y @ O.ilu_apply(p, i, d, f, x)
    rhs = O.ilu_apply(p, i, d, f, y, trans="T") @ x
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)


def test_ir_pcg_reaches_tolerance(rng):
    p, i, v = P.aniso3d(10)
    n = len(p) - 1
    xt = rng.standard_normal(n)
    b = P.csr_matvec(p, i, v, xt)
    f, d, _ = O.ilu_factor(p, i, v)
    x, tot, outer = O.ir_pcg(p, i, v, v.astype(np.float32), d, f.astype(np.float32), f[d], b,
                             1e-10 * np.linalg.norm(b), inner_rtol=1e-4)
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, x)) < 1e-10 * np.linalg.norm(b)
    assert outer >= 2


def test_ru_pcg_keeps_fp64_iterations(rng):
    p, i, v = P.aniso3d(12)
    n = len(p) - 1
    xt = rng.standard_normal(n)
    b = P.csr_matvec(p, i, v, xt)
    tol = 1e-10 * np.linalg.norm(b)
    f, d, _ = O.ilu_factor(p, i, v)
    _, it64, _ = O.cg(p, i, v, b, tol=tol, diag=d, ilu=f)
    x, it, upd = O.ru_pcg(p, i, v, v.astype(np.float32), d, f.astype(np.float32), f[d], b, tol, delta=0.01)
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, x)) < tol
    assert upd >= 2 and abs(it - (it64 - 1)) <= 2, (it, it64, upd)
    # at the iteration limit the correction is folded into x and the FP64 residual reported
    x5, it5, upd5 = O.ru_pcg(p, i, v, v.astype(np.float32), d, f.astype(np.float32), f[d], b, tol, max_iter=5)
    assert it5 == 5 and upd5 >= 1
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, x5)) < 0.5 * np.linalg.norm(b)


@pytest.mark.parametrize("restart", [5, 30])
def test_ir_gmres_reaches_tolerance(rng, restart):
    p, i, v = P.convdiff3d(12)
    n = len(p) - 1
    b = rng.uniform(-1, 1, n)
    f, d, _ = O.ilu_factor(p, i, v)
    tol = 1e-9 * np.linalg.norm(b)
    x, tot, outer = O.ir_gmres(p, i, v, v.astype(np.float32), d, f.astype(np.float32), f[d], restart, b, tol,
                               inner_rtol=1e-4)
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, x)) < tol
    assert outer >= 2
    # the same system in FP64 GMRES lands on the same solution
    xo, _ = O.gmres(p, i, v, b, restart, tol=1e-12 * np.linalg.norm(b), diag=d, ilu=f)
    assert np.linalg.norm(x - xo) <= 1e-7 * np.linalg.norm(xo)


# --------------------------------------------- against the reference's compiled CPU path ---
needs_ref = pytest.mark.skipif(not O.ref_available(), reason="reference CPU path not built here")


@needs_ref
def test_oracle_matches_reference_build(rng):
    ref = O.ref()
    cases = [(P.aniso3d(9, 8, 7), True), (P.convdiff3d(7), False), (P.random_csr(150, 0.03, rng), False),
             (P.poisson2d(20), True)]
    for (p, i, v), spd in cases:
        n = len(p) - 1
        x = rng.standard_normal(n)
        for t in ("N", "T"):
            y0 = rng.standard_normal(n)
            yo = O.spmv(t, n, n, 1.5, p, i, v, x, 0.25, y0)
            yr = y0.copy()
            ref.ref_sparse_gemv_d(t.encode(), n, n, 1.5, p, i, v, x, 0.25, yr)
            assert np.array_equal(yo, yr)
        d = O.diag_index(p, i)
        dr = np.zeros_like(d)
        ref.ref_get_diagonal_index(n, p, i, dr)
        assert np.array_equal(d, dr)
        f, _, _ = O.ilu_factor(p, i, v, d)
        fr = np.zeros_like(v)
        ref.ref_factorize_ilu_d(n, p, i, v, fr)
        assert np.array_equal(f.view(np.uint64), fr.view(np.uint64))
        a = O.ilu_apply(p, i, d, f, x)
        ar = x.copy()
        ref.ref_apply_ilu_d(n, p, i, d, fr, ar)
        assert np.array_equal(a, ar)
        b = O.spmv("N", n, n, 1.0, p, i, v, x, 0.0)
        tol = 1e-10 * np.linalg.norm(b)
        cap = 2000 if spd else 40     # CG on a nonsymmetric matrix: compare a capped run
        xo, ito, _ = O.cg(p, i, v, b, tol=tol, max_iter=cap, diag=d, ilu=f)
        xr = np.zeros(n)
        itr = ref.ref_solve_cg_d(n, p, i, v, d.ctypes.data, f.ctypes.data, b, xr, tol, cap)
        assert ito == itr and np.array_equal(xo, xr)
        xo, ito = O.gmres(p, i, v, b, 30, tol=1e-9 * np.linalg.norm(b), max_iter=20, diag=d, ilu=f)
        xr = np.zeros(n)
        itr = ref.ref_solve_gmres_d(n, p, i, v, d.ctypes.data, f.ctypes.data, 30, b, xr,
                                    1e-9 * np.linalg.norm(b), 20)
        assert ito == itr and np.array_equal(xo, xr)


@needs_ref
def test_trsv_matches_reference_build(rng):
    ref = O.ref()
    p, i, v = P.random_csr(80, 0.05, rng)
    d = O.diag_index(p, i)
    up, ui, lp, li = O.split_pattern(p, i, d)
    uv, lv = O.split_values("U", "N", p, v, up, lp)
    n = len(p) - 1
    b = rng.standard_normal(n)
    for (tp, ti, tv, uplo) in ((lp, li, lv, "L"), (up, ui, uv, "U")):
        tv = tv.copy()
        if uplo == "L":
            tv[lp[1:] - 1] = 1.0 + np.abs(rng.standard_normal(n))
        for diagc in ("N", "U"):
            for t in ("N", "T"):
                xo = O.trsv(uplo, diagc, t, 0.5, tp, ti, tv, b)
                xr = np.zeros(n)
                ref.ref_trsv_d(uplo.encode(), diagc.encode(), t.encode(), n, 0.5, tp, ti, tv, b, xr)
                assert np.array_equal(xo, xr), (uplo, diagc, t)


# ----------------------------------------------------------------- committed fixtures ---
@pytest.mark.parametrize("path", sorted(f for f in glob.glob(os.path.join(GOLDEN, "*.npz"))
                                        if not os.path.basename(f).startswith("cplx_")))
def test_oracle_matches_fixture(path):
    g = np.load(path)
    p, i, v = g["pntr"], g["indx"], g["vals"]
    n = len(p) - 1
    assert np.array_equal(O.diag_index(p, i), g["diag"])
    f, d, _ = O.ilu_factor(p, i, v)
    assert np.array_equal(f.view(np.uint64), g["ilu"].view(np.uint64))
    assert np.array_equal(O.ilu_apply(p, i, d, f, g["x"]), g["apply"])
    assert np.array_equal(O.spmv("N", n, n, 1.0, p, i, v, g["x"], 0.0), g["spmv_n"])
    assert np.array_equal(O.spmv("T", n, n, 1.0, p, i, v, g["x"], 0.0), g["spmv_t"])
    xo, ito, _ = O.cg(p, i, v, g["b"], tol=float(g["cg_tol"]), max_iter=int(g["cg_max_iter"]), diag=d, ilu=f)
    assert ito == int(g["cg_iters"]) and np.array_equal(xo, g["cg_x"])
    xo, ito = O.gmres(p, i, v, g["b"], int(g["gmres_restart"]), tol=float(g["gmres_tol"]),
                      max_iter=int(g["gmres_max_iter"]), diag=d, ilu=f)
    assert ito == int(g["gmres_iters"]) and np.array_equal(xo, g["gmres_x"])


def test_batch_cg_reference_cases():
    # tests/solvers_tests.hpp:56-104 (test_cg_batch): xref = make_vector(15), three columns
    xref = R.make_vector(0, 15)
    for case, tol, cap in [(R.TRIDIAG5, 0.0, 2), (R.CYCLIC5, 1e-9, 6)]:
        A = R.dense(case)
        B = np.concatenate([A @ xref[5 * c:5 * c + 5] for c in range(3)])
        f, d, _ = O.ilu_factor(case["pntr"], case["indx"], case["vals"])
        X, it, _ = O.batch_cg(case["pntr"], case["indx"], case["vals"], B, 3, tol=tol, max_iter=cap, diag=d, ilu=f)
        assert R.testvec(X, xref, np.linalg.norm(xref))


@needs_ref
def test_batch_cg_matches_reference_build(rng):
    p, i, v = P.aniso3d(9, 8, 7)
    n, k = len(p) - 1, 3
    B = rng.standard_normal(n * k)
    tol = 1e-9 * np.linalg.norm(B[:n])
    f, d, _ = O.ilu_factor(p, i, v)
    X, it, _ = O.batch_cg(p, i, v, B, k, tol=tol, max_iter=500, diag=d, ilu=f)
    Xr = np.zeros(n * k)
    itr = O.ref().ref_solve_batch_cg_ilu_d(n, p, i, v, k, B, Xr, tol, 500)
    assert it == itr and np.array_equal(X, Xr)
