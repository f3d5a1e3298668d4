"""Several right-hand sides with one matrix (solve_batch_cg / solve_batch_cg_ilu,
hex/solvers/hala_solvers_cg_batch.hpp): the SpMM column by column bit-exact against the
single-column SpMV, the multi-column ILU apply bit-exact against the oracle, and the multi-RHS PCG
against the oracle's restatement and the reference's test_cg_batch cases
(tests/solvers_tests.hpp:56-104)."""
import numpy as np
import pytest
import torch

from hala_gb300 import engine as E
from hala_gb300 import problems as P
from oracle import oracle as O
from tests import refcases as R

pytestmark = pytest.mark.gpu
dev = torch.device("cuda")


def T(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def test_gemm_columns_bit_exact(eng, rng):
    p, i, v = P.aniso3d(20, 19, 18)
    n, k = len(p) - 1, 5
    X = rng.standard_normal(n * k)
    A = E.make_sparse_matrix(eng, n, T(p), T(i), T(v))
    Y = torch.zeros(n * k, dtype=torch.float64, device=dev)
    A.gemm(k, 1.0, T(X), 0.0, Y)
    y = Y.cpu().numpy()
    for c in range(k):
        assert np.array_equal(y[c * n:(c + 1) * n], O.spmv("N", n, n, 1.0, p, i, v, X[c * n:(c + 1) * n], 0.0))


@pytest.mark.parametrize("vdt", [torch.float64, torch.float32, torch.bfloat16])
@pytest.mark.parametrize("mode", ["exact", "fused"])
def test_gemm_one_pass_equals_columns(eng, rng, vdt, mode):
    """The SpMM reads the matrix once for all columns; every column must equal the single-column
    product bit for bit, in both arithmetic modes, for column counts around the kernel's group of
    four, beta != 0 and leading dimensions larger than n."""
    from hala_gb300 import hgb as H
    p, i, v = P.aniso3d(23, 21, 17)
    n = len(p) - 1
    xdt = torch.float64 if vdt == torch.float64 else torch.float32
    A = E.make_sparse_matrix(eng, n, T(p), T(i), T(v).to(vdt))
    eng.set_spmv_mode(mode)
    try:
        for k, ld, beta in ((1, n, 0.0), (4, n, 0.5), (7, n + 5, -1.25), (9, n + 1, 0.0)):
            X = torch.from_numpy(rng.standard_normal(ld * k)).to(dev, xdt)
            Y0 = torch.from_numpy(rng.standard_normal(ld * k)).to(dev, xdt)
            Y = Y0.clone()
            H.check(H.lib().hgb_csr_gemm(A.h, k, 0.75, E._p(X), ld, beta, E._p(Y), ld), "gemm")
            for c in range(k):
                yc = Y0[c * ld:c * ld + n].clone()
                A.gemv("N", 0.75, X[c * ld:c * ld + n].contiguous(), beta, yc)
                assert torch.equal(Y[c * ld:c * ld + n], yc), (k, c)
                # rows between n and ld are not touched
                assert torch.equal(Y[c * ld + n:(c + 1) * ld], Y0[c * ld + n:(c + 1) * ld])
    finally:
        eng.set_spmv_mode("exact")


def test_ilu_apply_nrhs_bit_exact(eng, rng):
    p, i, v = P.aniso3d(24)
    n, k = len(p) - 1, 3
    fo, do, _ = O.ilu_factor(p, i, v)
    ilu = E.make_ilu(eng, T(p), T(i), T(v))
    X = rng.standard_normal(n * k)
    r = ilu.apply_nrhs(T(X), k).cpu().numpy()
    for c in range(k):
        assert np.array_equal(r[c * n:(c + 1) * n], O.ilu_apply(p, i, do, fo, X[c * n:(c + 1) * n]))


def test_reference_batch_cg_cases(eng):
    xref = R.make_vector(0, 15)
    for case, stop in [(R.TRIDIAG5, E.stop_criteria(2)), (R.CYCLIC5, E.stop_criteria(1e-9, 6))]:
        A = R.dense(case)
        B = np.concatenate([A @ xref[5 * c:5 * c + 5] for c in range(3)])
        gp, gi, gv = T(case["pntr"]), T(case["indx"]), T(case["vals"])
        X = torch.zeros(15, dtype=torch.float64, device=dev)
        E.solve_batch_cg_ilu(eng, stop, gp, gi, gv, T(B), X)
        assert R.testvec(X.cpu().numpy(), xref, np.linalg.norm(xref))


@pytest.mark.parametrize("precond", [False, True])
def test_batch_cg_matches_oracle(eng, rng, precond):
    p, i, v = P.aniso3d(24)
    n, k = len(p) - 1, 4
    B = rng.standard_normal(n * k)
    tol = 1e-8 * np.linalg.norm(B[:n])
    fo = do = None
    if precond:
        fo, do, _ = O.ilu_factor(p, i, v)
    Xo, ito, reso = O.batch_cg(p, i, v, B, k, tol=tol, diag=do, ilu=fo)
    gp, gi, gv = T(p), T(i), T(v)
    ilu = E.make_ilu(eng, gp, gi, gv) if precond else None
    X = torch.zeros(n * k, dtype=torch.float64, device=dev)
    it = E.solve_batch_cg(eng, E.stop_criteria(tol), gp, gi, gv, T(B), X, ilu=ilu)
    # dot products are summed in another order than the oracle's sequential loop
    assert abs(it - ito) <= max(1, int(0.05 * ito)), (it, ito)
    x = X.cpu().numpy()
    for c in range(k):
        r = B[c * n:(c + 1) * n] - P.csr_matvec(p, i, v, x[c * n:(c + 1) * n])
        assert np.linalg.norm(r) < 1.5 * tol
        assert np.linalg.norm(x[c * n:(c + 1) * n] - Xo[c * n:(c + 1) * n]) <= 1e-6 * np.linalg.norm(Xo[c * n:(c + 1) * n])
