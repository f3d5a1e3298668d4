"""Properties of the oracle on random inputs (CPU): linearity of the SpMV, ILU(0) exact where it
must be (tridiagonal), the ILU apply inverting the factor's own L U, triangular-solve round trips in
both orientations, level sets forming a valid schedule, and the mixed-precision restatements
converging on random SPD / nonsymmetric systems."""
import numpy as np
import pytest

from hala_gb300 import problems as P
from oracle import oracle as O


@pytest.fixture
def rng():
    return np.random.default_rng(2024)


def dense(p, i, v, n=None):
    return P.csr_to_dense(p, i, v, n)


def test_spmv_linear_and_transposed(rng):
    for _ in range(5):
        n = int(rng.integers(20, 120))
        p, i, v = P.random_csr(n, 0.08, rng)
        A = dense(p, i, v)
        x, y = rng.standard_normal(n), rng.standard_normal(n)
        a, b = rng.standard_normal(2)
        lhs = O.spmv("N", n, n, 1.0, p, i, v, a * x + b * y, 0.0)
        rhs = a * O.spmv("N", n, n, 1.0, p, i, v, x, 0.0) + b * O.spmv("N", n, n, 1.0, p, i, v, y, 0.0)
        assert np.allclose(lhs, rhs, rtol=1e-12, atol=1e-12)
        assert np.allclose(O.spmv("T", n, n, 1.0, p, i, v, x, 0.0), A.T @ x, rtol=1e-12, atol=1e-12)


def test_ilu_is_exact_on_tridiagonal(rng):
    for _ in range(5):
        n = int(rng.integers(5, 200))
        off = rng.uniform(-1, 1, (2, n))
        rows, cols, vals = [], [], []
        for r in range(n):
            for c, val in ((r - 1, off[0, r]), (r, 3.0 + rng.random()), (r + 1, off[1, r])):
                if 0 <= c < n:
                    rows.append(r), cols.append(c), vals.append(val)
        p = np.zeros(n + 1, np.int32)
        np.cumsum(np.bincount(rows, minlength=n), out=p[1:])
        i, v = np.array(cols, np.int32), np.array(vals)
        f, d, st = O.ilu_factor(p, i, v)
        assert st == 0
        x = rng.standard_normal(n)
        assert np.allclose(O.ilu_apply(p, i, d, f, P.csr_matvec(p, i, v, x)), x, rtol=1e-11, atol=1e-11)


def test_ilu_apply_inverts_its_factor(rng):
    for _ in range(5):
        n = int(rng.integers(30, 150))
        p, i, v = P.random_csr(n, 0.06, rng)
        f, d, st = O.ilu_factor(p, i, v)
        assert st == 0
        F = dense(p, i, f)
        L = np.tril(F, -1) + np.eye(n)
        U = np.triu(F)
        y = rng.standard_normal(n)
        assert np.allclose(O.ilu_apply(p, i, d, f, L @ (U @ y)), y, rtol=1e-9, atol=1e-9)
        # the transposed apply is (L U)^-T
        assert np.allclose(O.ilu_apply(p, i, d, f, U.T @ (L.T @ y), trans="T"), y, rtol=1e-9, atol=1e-9)


def _csr(M):
    rows, cols = np.nonzero(M)
    p = np.zeros(M.shape[0] + 1, np.int32)
    np.cumsum(np.bincount(rows, minlength=M.shape[0]), out=p[1:])
    return p, cols.astype(np.int32), M[rows, cols]


def test_trsv_round_trips(rng):
    # sparse_trsv takes the triangle's own CSR (as the reference's test cases do)
    for _ in range(5):
        n = int(rng.integers(10, 120))
        A = dense(*P.random_csr(n, 0.1, rng))
        x = rng.standard_normal(n)
        for uplo, T in (("L", np.tril(A)), ("U", np.triu(A))):
            p, i, v = _csr(T)
            for trans, M in (("N", T), ("T", T.T)):
                got = O.trsv(uplo, "N", trans, 2.0, p, i, v, M @ x)
                assert np.allclose(got, 2.0 * x, rtol=1e-9, atol=1e-9), (uplo, trans)
            # unit diagonal: the stored diagonal is ignored
            Tu = T - np.diag(np.diag(T)) + np.eye(n)
            got = O.trsv(uplo, "U", "N", 1.0, p, i, v, Tu @ x)
            assert np.allclose(got, x, rtol=1e-9, atol=1e-9), (uplo, "unit")


def test_levels_form_a_schedule(rng):
    for _ in range(5):
        n = int(rng.integers(20, 200))
        p, i, v = P.random_csr(n, 0.05, rng)
        d = O.diag_index(p, i)
        lev, nl = O.levels(p, i, d, "L")
        for r in range(n):
            deps = [c for c in i[p[r]:p[r + 1]] if c < r]
            want = 1 + max((lev[c] for c in deps), default=-1)
            assert lev[r] == want
        assert nl == lev.max() + 1


def test_ru_pcg_converges_on_random_spd(rng):
    for _ in range(3):
        n = int(rng.integers(100, 300))
        p, i, v = P.random_csr(n, 0.03, rng)
        A = dense(p, i, v)
        S = 0.5 * (A + A.T)
        S += np.diag(np.abs(S).sum(1))               # SPD: symmetric and diagonally dominant
        ps, is_, vs = _csr(S)
        f, d, _ = O.ilu_factor(ps, is_, vs)
        b = rng.standard_normal(n)
        tol = 1e-10 * np.linalg.norm(b)
        x, it, upd = O.ru_pcg(ps, is_, vs, vs.astype(np.float32), d, f.astype(np.float32), f[d], b, tol)
        assert np.linalg.norm(b - S @ x) < tol and upd >= 1


def test_ir_gmres_converges_on_random_nonsymmetric(rng):
    for _ in range(3):
        n = int(rng.integers(100, 300))
        p, i, v = P.random_csr(n, 0.03, rng)
        f, d, _ = O.ilu_factor(p, i, v)
        b = rng.standard_normal(n)
        tol = 1e-9 * np.linalg.norm(b)
        x, tot, outer = O.ir_gmres(p, i, v, v.astype(np.float32), d, f.astype(np.float32), f[d], 10, b, tol)
        assert np.linalg.norm(b - P.csr_matvec(p, i, v, x)) < tol
