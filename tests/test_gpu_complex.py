"""Complex (C128 / C64) path on the GPU, through the C ABI, against the complex CPU oracle.

Tolerances: SpMV 'N' and the cached 'T' / 'C' perform the oracle's sequence of separately rounded
complex operations and are compared BIT-EXACTLY; the atomic transpose (no matrix handle) within
1e-14 relative (C128) / 1e-6 (C64).  ILU(0), its apply and the triangular solves divide with
Smith's method where the reference's std::complex division scales differently: 1e-12 relative
(C128) and 1e-5 (C64).  Reductions accumulate in double: 1e-13 / 1e-6.  CG and GMRES: the same
iteration counts (CG within one) and solutions within 1e-9 (C128) / 1e-4 (C64) of the oracle's."""
import numpy as np
import pytest
import torch

from hala_gb300 import engine as E
from hala_gb300 import problems as P
from hala_gb300.hgb import HgbError
from oracle import oracle as O
from tests import refcases as R

pytestmark = pytest.mark.gpu
dev = torch.device("cuda")
CT = [np.complex128, np.complex64]
TOL_FACT = {np.complex128: 1e-12, np.complex64: 1e-5}
TOL_RED = {np.complex128: 1e-13, np.complex64: 1e-6}


def T(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def H(t):
    return t.cpu().numpy()


def rel(a, b):
    a, b = np.asarray(a, np.complex128), np.asarray(b, np.complex128)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def cvec(rng, n, ct):
    return (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(ct)


def random_complex(rng, n, ct, density=0.05):
    p, i, v = P.random_csr(n, density, rng)
    return p, i, (v + 1j * rng.uniform(-1, 1, len(v))).astype(ct)


CASES = {
    "magnetic2d_20": lambda rng, ct: (*P.magnetic2d(20)[:2], P.magnetic2d(20)[2].astype(ct)),
    "helmholtz_convdiff3d_9": lambda rng, ct: (*P.convdiff3d(9)[:2],
                                               P.helmholtz_shift(*P.convdiff3d(9))[2].astype(ct)),
    "random_300": lambda rng, ct: random_complex(rng, 300, ct),
}


@pytest.mark.parametrize("ct", CT)
@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("ab", [(1.0, 0.0), (0.5 - 0.25j, 1.0 + 0.5j)])
def test_complex_spmv_bit_exact(eng, rng, ct, name, ab):
    p, i, v = CASES[name](rng, ct)
    n = len(p) - 1
    alpha, beta = ab
    x, y0 = cvec(rng, n, ct), cvec(rng, n, ct)
    A = E.make_sparse_matrix(eng, n, T(p), T(i), T(v))
    for t in "NTC":
        y = T(y0)
        A.gemv(t, alpha, T(x), beta, y)
        ref = O.zspmv(t, n, n, alpha, p, i, v, x, beta, y0)
        assert np.array_equal(H(y), ref), t


@pytest.mark.parametrize("ct", CT)
def test_complex_spmv_raw_entry_points(eng, rng, ct):
    """hgb_spmv_c128 / _c64 without a handle: 'N' bit-exact, 'T' / 'C' scatter with atomics"""
    p, i, v = random_complex(rng, 400, ct)
    n = len(p) - 1
    x, y0 = cvec(rng, n, ct), cvec(rng, n, ct)
    for t in "NTC":
        y = T(y0)
        E.sparse_gemv(eng, t, n, n, 2.0 - 1j, T(p), T(i), T(v), T(x), 0.5j, y)
        ref = O.zspmv(t, n, n, 2.0 - 1j, p, i, v, x, 0.5j, y0)
        if t == "N":
            assert np.array_equal(H(y), ref)
        else:
            assert rel(H(y), ref) < 10 * TOL_RED[ct], t


@pytest.mark.parametrize("ct", CT)
def test_complex_blas1(eng, rng, ct):
    for n in (0, 1, 1000, 300_001):
        x, y = cvec(rng, n, ct), cvec(rng, n, ct)
        xd, yd = T(x), T(y)
        x128, y128 = x.astype(np.complex128), y.astype(np.complex128)
        scale = max(np.sum(np.abs(x128) * np.abs(y128)), 1e-300)
        assert abs(E.dot(eng, xd, yd) - np.vdot(x128, y128)) <= TOL_RED[ct] * scale
        assert abs(E.dotu(eng, xd, yd) - np.sum(x128 * y128)) <= TOL_RED[ct] * scale
        assert abs(E.norm2(eng, xd) - np.linalg.norm(x128)) <= TOL_RED[ct] * max(np.linalg.norm(x128), 1e-300)
        a = 0.75 - 1.25j
        E.axpy(eng, a, xd, yd)
        assert rel(H(yd), y + ct(a) * x) <= TOL_RED[ct]
        E.scal(eng, a, xd)
        assert rel(H(xd), ct(a) * x) <= TOL_RED[ct]
        z = torch.empty_like(xd)
        E.vcopy(eng, xd, z)
        assert torch.equal(z, xd)


@pytest.mark.parametrize("ct", CT)
@pytest.mark.parametrize("name", list(CASES))
def test_complex_ilu_factor_and_apply(eng, rng, ct, name):
    p, i, v = CASES[name](rng, ct)
    n = len(p) - 1
    M = E.make_ilu(eng, T(p), T(i), T(v))
    assert not M.zero_pivot
    f, d = M.factor()
    fo, do, st = O.zilu_factor(p, i, v)
    assert st == 0 and np.array_equal(H(d), do)
    assert rel(H(f), fo) < TOL_FACT[ct]
    x = cvec(rng, n, ct)
    for t in "NTC":
        r = M.apply(T(x), trans=t)
        ro = O.zilu_apply(p, i, do, fo, x, trans=t)
        assert rel(H(r), ro) < 10 * TOL_FACT[ct], t
    # in place (x and r alias)
    xd = T(x)
    M.apply(xd, xd)
    assert rel(H(xd), O.zilu_apply(p, i, do, fo, x)) < 10 * TOL_FACT[ct]


@pytest.mark.parametrize("ct", CT)
def test_complex_ilu_host_buffers(eng, rng, ct):
    p, i, v = random_complex(rng, 500, ct)
    M = E.make_ilu_host(eng, p, i, v)
    f, d = M.factor()
    fo, do, _ = O.zilu_factor(p, i, v)
    assert np.array_equal(H(d), do) and rel(H(f), fo) < TOL_FACT[ct]


@pytest.mark.parametrize("ct", CT)
def test_complex_triangular_solves(eng, rng, ct):
    """make_triangular_matrix on the full pattern (fill mode): L / U, unit / non-unit, N / T / C"""
    p, i, v = random_complex(rng, 200, ct)
    n = len(p) - 1
    d = O.diag_index(p, i)
    up, ui, lp, li = O.split_pattern(p, i, d)
    Lv = np.ascontiguousarray(np.concatenate([v[p[k]:d[k] + 1] for k in range(n)]))
    Uv = np.ascontiguousarray(np.concatenate([v[d[k]:p[k + 1]] for k in range(n)]))
    b = cvec(rng, n, ct)
    for uplo, tp, ti, tv in (("L", lp, li, Lv), ("U", up, ui, Uv)):
        for diagc in "NU":
            tri = E.make_triangular_matrix(eng, uplo, diagc, T(p), T(i), T(v))
            for t in "NTC":
                x = T(np.zeros(n, ct))
                tri.trsv(t, 0.5, T(b), x)
                xo = O.ztrsv(uplo, diagc, t, 0.5, tp, ti, tv, b)
                assert rel(H(x), xo) < 10 * TOL_FACT[ct], (uplo, diagc, t)
            bd = T(b)   # b aliases x
            tri.trsv("N", 0.5, bd, bd)
            assert rel(H(bd), O.ztrsv(uplo, diagc, "N", 0.5, tp, ti, tv, b)) < 10 * TOL_FACT[ct]


@pytest.mark.parametrize("ct", CT)
def test_complex_reference_solver_cases(eng, ct):
    """test_cg / test_gmres on std::complex (solvers_tests.hpp:12-137): exact ILU on the tridiagonal
    matrix (two CG iterations, GMRES(2)), the cyclic matrix with CG from a given start, GMRES(6)
    on the nonsymmetric one"""
    tol = 1e-9 if ct == np.complex128 else 1e-4
    c = R.TRIDIAG5
    v = c["vals"].astype(ct)
    b = (R.dense(c) @ R.XREF5).astype(ct)
    M = E.make_ilu(eng, T(c["pntr"]), T(c["indx"]), T(v))
    x = T(np.zeros(5, ct))
    it = E.solve_cg(eng, 2, T(c["pntr"]), T(c["indx"]), T(v), T(b), x, ilu=M)
    assert it == 2 and rel(H(x), R.XREF5) < 100 * TOL_RED[ct]
    x = T(np.zeros(5, ct))
    E.solve_gmres(eng, E.stop_criteria(0.0, 2), 2, T(c["pntr"]), T(c["indx"]), T(v), T(b), x, ilu=M)
    assert rel(H(x), R.XREF5) < 100 * TOL_RED[ct]
    c = R.CYCLIC5
    v = c["vals"].astype(ct)
    b = (R.dense(c) @ R.XREF5).astype(ct)
    M = E.make_ilu(eng, T(c["pntr"]), T(c["indx"]), T(v))
    x = T(R.CG_X0.astype(ct))
    E.solve_cg(eng, tol, T(c["pntr"]), T(c["indx"]), T(v), T(b), x, ilu=M)
    assert np.linalg.norm(H(x) - R.XREF5) <= 10 * tol * np.linalg.norm(R.XREF5)
    c = R.NONSYM5
    v = c["vals"].astype(ct)
    b = (R.dense(c) @ R.XREF5).astype(ct)
    M = E.make_ilu(eng, T(c["pntr"]), T(c["indx"]), T(v))
    x = T(np.zeros(5, ct))
    E.solve_gmres(eng, tol, 6, T(c["pntr"]), T(c["indx"]), T(v), T(b), x, ilu=M)
    assert np.linalg.norm(H(x) - R.XREF5) <= 100 * tol * np.linalg.norm(R.XREF5)


@pytest.mark.parametrize("ct", CT)
@pytest.mark.parametrize("precond", [True, False])
def test_complex_cg_vs_oracle(eng, rng, ct, precond):
    p, i, v = P.magnetic2d(40, flux=0.4, shift=0.02)
    v = v.astype(ct)
    n = len(p) - 1
    b = cvec(rng, n, ct)
    tol = (1e-10 if ct == np.complex128 else 1e-4) * float(np.linalg.norm(b))
    M = E.make_ilu(eng, T(p), T(i), T(v)) if precond else None
    x = T(np.zeros(n, ct))
    it = E.solve_cg(eng, tol, T(p), T(i), T(v), T(b), x, ilu=M)
    fo, do, _ = O.zilu_factor(p, i, v)
    xo, ito, _ = O.zcg(p, i, v, b, tol=tol, diag=do if precond else None, ilu=fo if precond else None)
    assert abs(it - ito) <= 1 + ito // 50
    A = P.csr_to_dense(p, i, v.astype(np.complex128))
    assert np.linalg.norm(A @ H(x).astype(np.complex128) - b) < (2 if ct == np.complex128 else 10) * tol
    assert rel(H(x), xo) < (1e-8 if ct == np.complex128 else 1e-3)


@pytest.mark.parametrize("ct", CT)
@pytest.mark.parametrize("restart,max_iter", [(5, 2), (25, 3)])
def test_complex_gmres_vs_oracle(eng, rng, ct, restart, max_iter):
    """a few restarts on the shifted convection-diffusion operator: applications and iterate against
    the oracle's loop (the reference's unconjugated projection)"""
    p, i, v = P.helmholtz_shift(*P.convdiff3d(10), sigma=(1.0, 2.0))
    v = v.astype(ct)
    n = len(p) - 1
    b = cvec(rng, n, ct)
    M = E.make_ilu(eng, T(p), T(i), T(v))
    fo, do, _ = O.zilu_factor(p, i, v)
    tol = 1e-30
    x = T(np.zeros(n, ct))
    # tol 1e-30 is not reached: every restart runs its full cycle, and the limit is not an error
    it = E.solve_gmres(eng, E.stop_criteria(tol, max_iter), restart, T(p), T(i), T(v), T(b), x, ilu=M)
    xo, ito = O.zgmres(p, i, v, b, restart, tol=tol, max_iter=max_iter, diag=do, ilu=fo)
    assert it == ito == max_iter * (restart + 1)
    assert rel(H(x), xo) < (1e-9 if ct == np.complex128 else 1e-3)


def test_complex_rejections(eng, rng):
    p, i, v = random_complex(rng, 50, np.complex128)
    A = E.make_sparse_matrix(eng, 50, T(p), T(i), T(v))
    with pytest.raises(HgbError):   # the complex factor is stored in its own precision
        E.make_ilu(eng, T(p), T(i), T(v), store=torch.complex64)
    M = E.make_ilu(eng, T(p), T(i), T(v))
    with pytest.raises(HgbError):   # no level sets for a complex factor
        M.levels("L")
    with pytest.raises(HgbError):   # transposed complex CG is not offered
        E.solve_cg_op(eng, A, M, "T", T(cvec(rng, 50, np.complex128)), T(np.zeros(50, np.complex128)), 1e-8)
    M32 = E.make_ilu(eng, T(p), T(i), T(v.astype(np.complex64)))
    with pytest.raises(HgbError):   # preconditioner precision must match
        E.solve_cg(eng, 1e-8, T(p), T(i), T(v), T(cvec(rng, 50, np.complex128)),
                   T(np.zeros(50, np.complex128)), ilu=M32)
