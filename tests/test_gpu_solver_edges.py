"""Edge cases of the solvers: a zero right-hand side, a start at the solution, a 1 x 1 system,
GMRES(1), GMRES from a nonzero start, iteration limits of zero; each against the oracle (the
reference's solve_cg / solve_gmres loops) or the exact answer."""
import numpy as np
import pytest
import torch

from hala_gb300 import engine as E
from hala_gb300 import problems as P
from hala_gb300.hgb import HgbError
from oracle import oracle as O

pytestmark = pytest.mark.gpu
dev = torch.device("cuda")


def T(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def mixed_ops(eng, p, i, v):
    n = len(p) - 1
    gp, gi, gv = T(p), T(i), T(v)
    return (E.make_sparse_matrix(eng, n, gp, gi, gv), E.make_sparse_matrix(eng, n, gp, gi, gv.to(torch.float32)),
            E.make_ilu(eng, gp, gi, gv, store=torch.float32))


def test_zero_rhs(eng):
    # b = 0 with the relative target 1e-10 * ||b|| = 0: x = 0 is exact, no iteration runs
    p, i, v = P.aniso3d(10)
    n = len(p) - 1
    A64, A32, M = mixed_ops(eng, p, i, v)
    b = torch.zeros(n, dtype=torch.float64, device=dev)
    for solve in (lambda x: E.solve_ru_pcg(eng, A64, A32, M, b, x, 0.0),
                  lambda x: E.solve_ir_pcg(eng, A64, A32, M, b, x, 0.0),
                  lambda x: E.solve_ir_gmres(eng, A64, A32, M, 10, b, x, 0.0)):
        x = torch.zeros(n, dtype=torch.float64, device=dev)
        info = solve(x)
        assert info.iterations == 0 and info.true_residual == 0.0
        assert torch.count_nonzero(x).item() == 0
    gp, gi, gv = T(p), T(i), T(v)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    it = E.solve_gmres(eng, E.stop_criteria(0.0), 10, gp, gi, gv, b, x, ilu=E.make_ilu(eng, gp, gi, gv))
    assert it == 1 and torch.count_nonzero(x).item() == 0      # the reference counts the initial application


def test_start_at_solution(eng, rng):
    p, i, v = P.aniso3d(10)
    n = len(p) - 1
    xt = rng.standard_normal(n)
    b = P.csr_matvec(p, i, v, xt)
    A64, A32, M = mixed_ops(eng, p, i, v)
    tol = 1e-10 * np.linalg.norm(b)
    x = T(xt)
    info = E.solve_ru_pcg(eng, A64, A32, M, T(b), x, tol)
    assert info.iterations == 0 and info.outer == 0
    assert np.array_equal(x.cpu().numpy(), xt)


def test_one_by_one(eng):
    p, i, v = np.array([0, 1], np.int32), np.array([0], np.int32), np.array([4.0])
    b = np.array([2.0])
    gp, gi, gv = T(p), T(i), T(v)
    x = torch.zeros(1, dtype=torch.float64, device=dev)
    it = E.solve_cg(eng, E.stop_criteria(1e-12), gp, gi, gv, T(b), x, ilu=E.make_ilu(eng, gp, gi, gv))
    _, ito, _ = O.cg(p, i, v, b, tol=1e-12)
    assert x.item() == 0.5 and it == ito
    x.zero_()
    E.solve_gmres(eng, E.stop_criteria(1e-12), 5, gp, gi, gv, T(b), x)
    assert abs(x.item() - 0.5) <= 1e-15
    A64, A32, M = mixed_ops(eng, p, i, v)
    x.zero_()
    E.solve_ru_pcg(eng, A64, A32, M, T(b), x, 1e-12)
    assert x.item() == 0.5


@pytest.mark.parametrize("restart", [1, 2])
def test_gmres_short_restart_and_start(eng, rng, restart):
    p, i, v = P.convdiff3d(8, peclet=1.0)
    n = len(p) - 1
    b = rng.uniform(-1, 1, n)
    x0 = rng.uniform(-1, 1, n)
    fo, do, _ = O.ilu_factor(p, i, v)
    tol = 1e-9 * np.linalg.norm(O.ilu_apply(p, i, do, fo, b))
    xo, ito = O.gmres(p, i, v, b, restart, x0=x0, tol=tol, max_iter=5000, diag=do, ilu=fo)
    gp, gi, gv = T(p), T(i), T(v)
    x = T(x0)
    it = E.solve_gmres(eng, E.stop_criteria(tol, 5000), restart, gp, gi, gv, T(b), x, ilu=E.make_ilu(eng, gp, gi, gv))
    assert abs(it - ito) <= max(2, int(round(0.05 * ito))), (it, ito)
    assert np.linalg.norm(x.cpu().numpy() - xo) <= 1e-6 * np.linalg.norm(xo)


def test_zero_iteration_limits(eng, rng):
    p, i, v = P.aniso3d(8)
    n = len(p) - 1
    b = rng.standard_normal(n)
    A64, A32, M = mixed_ops(eng, p, i, v)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    with pytest.raises(HgbError):           # no iteration allowed and b != 0: not converged, x untouched
        E.solve_ru_pcg(eng, A64, A32, M, T(b), x, 1e-10, max_iter=0)
    assert torch.count_nonzero(x).item() == 0
    with pytest.raises(HgbError):
        E.solve_ir_pcg(eng, A64, A32, M, T(b), x, 1e-10, max_outer=0)
    assert torch.count_nonzero(x).item() == 0
    gp, gi, gv = T(p), T(i), T(v)
    it = E.solve_gmres(eng, E.stop_criteria(0), 4, gp, gi, gv, T(b), x)   # zero restart cycles
    assert it == 0 and torch.count_nonzero(x).item() == 0
