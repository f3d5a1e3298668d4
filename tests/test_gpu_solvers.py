"""CG / PCG / GMRES / iterative refinement on the GPU vs the oracle (the reference's algorithms).

Solves must reach the same residual target with iteration counts within 5% of the oracle's
(reductions are parallel, so the Krylov recurrences are not bit-identical); the reference's
own solver tests are replayed with its tolerances (sum|x - xref| / correction < 1e-14)."""
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


def within5(a, b):
    return abs(a - b) <= max(1, int(round(0.05 * b)))


def test_reference_cg_goldens(eng):
    c = R.TRIDIAG5
    b = R.dense(c) @ R.XREF5
    gp, gi, gv = T(c["pntr"]), T(c["indx"]), T(c["vals"])
    ilu = E.make_ilu(eng, gp, gi, gv)
    x = torch.zeros(5, dtype=torch.float64, device=dev)
    it = E.solve_cg(eng, E.stop_criteria(2), gp, gi, gv, T(b), x, ilu=ilu)
    assert it == 2 and R.testvec(x.cpu().numpy(), R.XREF5)
    c = R.CYCLIC5
    b = R.dense(c) @ R.XREF5
    gp, gi, gv = T(c["pntr"]), T(c["indx"]), T(c["vals"])
    x = T(R.CG_X0)
    E.solve_cg_ilu(eng, 1e-9, gp, gi, gv, T(b), x)
    assert R.testvec(x.cpu().numpy(), R.XREF5, np.linalg.norm(R.XREF5))


def test_reference_gmres_goldens(eng):
    c = R.TRIDIAG5
    b = R.dense(c) @ R.XREF5
    gp, gi, gv = T(c["pntr"]), T(c["indx"]), T(c["vals"])
    x = torch.zeros(5, dtype=torch.float64, device=dev)
    E.solve_gmres_ilu(eng, E.stop_criteria(2), 2, gp, gi, gv, T(b), x)
    assert R.testvec(x.cpu().numpy(), R.XREF5)
    c = R.NONSYM5
    b = R.dense(c) @ R.XREF5
    gp, gi, gv = T(c["pntr"]), T(c["indx"]), T(c["vals"])
    x = torch.zeros(5, dtype=torch.float64, device=dev)
    E.solve_gmres_ilu(eng, 1e-9, 6, gp, gi, gv, T(b), x)
    assert R.testvec(x.cpu().numpy(), R.XREF5)


@pytest.mark.parametrize("precond", [False, True])
@pytest.mark.parametrize("mat", ["poisson2d", "aniso3d"])
def test_cg_matches_oracle(eng, rng, precond, mat):
    p, i, v = P.poisson2d(64) if mat == "poisson2d" else P.aniso3d(24)
    n = len(p) - 1
    xt = rng.uniform(-1, 1, n)
    b = P.csr_matvec(p, i, v, xt)
    tol = 1e-10 * np.linalg.norm(b)
    fo, do, _ = O.ilu_factor(p, i, v)
    xo, ito, _ = O.cg(p, i, v, b, tol=tol, diag=do if precond else None, ilu=fo if precond else None)
    gp, gi, gv = T(p), T(i), T(v)
    ilu = E.make_ilu(eng, gp, gi, gv) if precond else None
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    it = E.solve_cg(eng, E.stop_criteria(tol), gp, gi, gv, T(b), x, ilu=ilu)
    assert within5(it, ito), (it, ito)
    xs = x.cpu().numpy()
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, xs)) < 2 * tol
    assert np.linalg.norm(xs - xo) <= 1e-8 * np.linalg.norm(xo)


def test_cg_iteration_limit(eng, rng):
    p, i, v = P.poisson2d(40)
    n = len(p) - 1
    b = rng.uniform(-1, 1, n)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    gp, gi, gv = T(p), T(i), T(v)
    it = E.solve_cg(eng, E.stop_criteria(17), gp, gi, gv, T(b), x)
    xo, ito, _ = O.cg(p, i, v, b, max_iter=17)
    assert it == ito == 17
    assert np.linalg.norm(x.cpu().numpy() - xo) <= 1e-10 * np.linalg.norm(xo)


@pytest.mark.parametrize("vdt", [torch.float64, torch.float32, torch.bfloat16])
def test_cg_persistent_small_systems(eng, eng_fused, rng, vdt):
    """unpreconditioned CG on an L2-resident system runs as one persistent cooperative launch
    (two grid barriers per iteration, Ap by recurrence): against the oracle's loop in both SpMV
    modes"""
    p, i, v = P.poisson2d(100)
    n = len(p) - 1
    b = rng.uniform(-1, 1, n)
    if vdt == torch.float64:
        vv, bb, tol = v, b, 1e-10 * np.linalg.norm(b)
    else:
        vv = v.astype(np.float32)
        bb = b.astype(np.float32)
        tol = 1e-5 * float(np.linalg.norm(bb))
    xo, ito, _ = O.cg(p, i, vv, bb, tol=tol)
    gv = T(vv) if vdt != torch.bfloat16 else T(vv).to(torch.bfloat16)   # 4 and -1 are exact in bf16
    xdt = torch.float64 if vdt == torch.float64 else torch.float32
    for e in (eng, eng_fused):
        x = torch.zeros(n, dtype=xdt, device=dev)
        info = E.solve_cg_info(e, E.make_sparse_matrix(e, n, T(p), T(i), gv), None, T(bb), x, tol)
        assert info.kernel_launches < info.iterations   # one launch per 4,096 iterations after the set-up
        xs = x.cpu().numpy().astype(np.float64)
        if vdt == torch.float64:
            assert within5(info.iterations, ito), (info.iterations, ito)
            assert np.linalg.norm(b - P.csr_matvec(p, i, v, xs)) < 2 * tol
            assert np.linalg.norm(xs - xo) <= 1e-8 * np.linalg.norm(xo)
        else:   # FP32 recurrences: the count within 10 %, the iterate near the oracle's
            assert abs(info.iterations - ito) <= max(2, ito // 10), (info.iterations, ito)
            assert np.linalg.norm(xs - xo) <= 1e-2 * np.linalg.norm(xo)


def test_gmres_matches_oracle(eng, rng):
    p, i, v = P.convdiff3d(16)
    n = len(p) - 1
    b = rng.uniform(-1, 1, n)
    fo, do, _ = O.ilu_factor(p, i, v)
    pb = O.ilu_apply(p, i, do, fo, b)
    tol = 1e-9 * np.linalg.norm(pb)
    xo, ito = O.gmres(p, i, v, b, 30, tol=tol, diag=do, ilu=fo)
    gp, gi, gv = T(p), T(i), T(v)
    ilu = E.make_ilu(eng, gp, gi, gv)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    it = E.solve_gmres(eng, E.stop_criteria(tol), 30, gp, gi, gv, T(b), x, ilu=ilu)
    assert within5(it, ito), (it, ito)
    xs = x.cpu().numpy()
    assert np.linalg.norm(xs - xo) <= 1e-7 * np.linalg.norm(xo)


@pytest.mark.parametrize("inner", [torch.float32, torch.bfloat16])
def test_ir_pcg_reaches_fp64_accuracy(eng, rng, inner):
    p, i, v = P.aniso3d(32)
    n = len(p) - 1
    xt = rng.standard_normal(n)
    b = P.csr_matvec(p, i, v, xt)
    tol = 1e-10 * np.linalg.norm(b)
    fo, do, _ = O.ilu_factor(p, i, v)
    xo, _, _ = O.cg(p, i, v, b, tol=tol, diag=do, ilu=fo)
    gp, gi, gv = T(p), T(i), T(v)
    A64 = E.make_sparse_matrix(eng, n, gp, gi, gv)
    gvi = gv.to(torch.float32 if inner == torch.float32 else torch.bfloat16)
    Ai = E.make_sparse_matrix(eng, n, gp, gi, gvi)
    Mi = E.make_ilu(eng, gp, gi, gv, store=inner)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    info = E.solve_ir_pcg(eng, A64, Ai, Mi, T(b), x, tol, inner_rtol=1e-4 if inner == torch.float32 else 1e-2)
    xs = x.cpu().numpy()
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, xs)) < tol
    assert info.outer >= 2
    # error against the exact solution, no worse than the FP64 oracle's own (same residual target;
    # both errors are conditioning x 1e-10, so they are compared rather than the two iterates)
    err, err_o = np.linalg.norm(xs - xt), np.linalg.norm(xo - xt)
    assert err <= 5 * err_o + 1e-12 * np.linalg.norm(xt), (err, err_o)
    assert np.linalg.norm(xs - xo) <= 1e-7 * np.linalg.norm(xo)


def test_fp32_cg(eng, rng):
    p, i, v = P.aniso3d(20)
    n = len(p) - 1
    v32 = v.astype(np.float32)
    b = rng.uniform(-1, 1, n).astype(np.float32)
    gp, gi, gv = T(p), T(i), T(v32)
    ilu = E.make_ilu(eng, gp, gi, gv)
    x = torch.zeros(n, dtype=torch.float32, device=dev)
    tol = 1e-5 * float(np.linalg.norm(b))
    it = E.solve_cg(eng, E.stop_criteria(tol), gp, gi, gv, T(b), x, ilu=ilu)
    fo, do, _ = O.ilu_factor(p, i, v32)
    _, ito, _ = O.cg(p, i, v32, b, tol=np.float32(tol), diag=do, ilu=fo)
    assert within5(it, ito), (it, ito)


def test_mixed_engine_host_buffers(eng, rng):
    p, i, v = P.aniso3d(16)
    n = len(p) - 1
    xt = rng.standard_normal(n)
    b = P.csr_matvec(p, i, v, xt)
    tol = 1e-10 * np.linalg.norm(b)
    ilu = E.make_ilu(eng, T(p), T(i), T(v))
    x = np.zeros(n)
    info = E.solve_cg_mixed(eng, E.stop_criteria(tol), p, i, v, ilu, b, x)
    fo, do, _ = O.ilu_factor(p, i, v)
    _, ito, _ = O.cg(p, i, v, b, tol=tol, diag=do, ilu=fo)
    assert within5(info.iterations, ito)
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, x)) < 2 * tol


@pytest.mark.parametrize("restart", [3, 8])
def test_gmres_several_cycles(eng, rng, restart):
    # short restarts: several device-resident cycles, each one graph replay
    p, i, v = P.convdiff3d(14)
    n = len(p) - 1
    b = rng.uniform(-1, 1, n)
    fo, do, _ = O.ilu_factor(p, i, v)
    tol = 1e-9 * np.linalg.norm(O.ilu_apply(p, i, do, fo, b))
    xo, ito = O.gmres(p, i, v, b, restart, tol=tol, diag=do, ilu=fo)
    gp, gi, gv = T(p), T(i), T(v)
    ilu = E.make_ilu(eng, gp, gi, gv)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    it = E.solve_gmres(eng, E.stop_criteria(tol), restart, gp, gi, gv, T(b), x, ilu=ilu)
    assert ito > restart + 1          # more than one cycle
    assert within5(it, ito), (it, ito)
    assert np.linalg.norm(x.cpu().numpy() - xo) <= 1e-7 * np.linalg.norm(xo)


def test_gmres_cycle_limit_and_unpreconditioned(eng, rng):
    p, i, v = P.convdiff3d(10)
    n = len(p) - 1
    b = rng.uniform(-1, 1, n)
    gp, gi, gv = T(p), T(i), T(v)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    # stop_criteria(int): the number of restart cycles only
    it = E.solve_gmres(eng, E.stop_criteria(3), 4, gp, gi, gv, T(b), x)
    xo, ito = O.gmres(p, i, v, b, 4, max_iter=3)
    assert it == ito == 3 * 5
    assert np.linalg.norm(x.cpu().numpy() - xo) <= 1e-9 * np.linalg.norm(xo)


def test_gmres_restart_bounds(eng):
    from hala_gb300.hgb import HgbError
    p, i, v = P.convdiff3d(4)
    gp, gi, gv = T(p), T(i), T(v)
    x = torch.zeros(len(p) - 1, dtype=torch.float64, device=dev)
    b = torch.ones(len(p) - 1, dtype=torch.float64, device=dev)
    with pytest.raises(HgbError):
        E.solve_gmres(eng, E.stop_criteria(1e-9), 513, gp, gi, gv, b, x)


@pytest.mark.parametrize("restart", [65, 150])
def test_gmres_long_restart(eng, rng, restart):
    # restarts above 64: the projection runs in groups of 64 basis columns (the reference has no cap)
    p, i, v = P.aniso3d(20)
    n = len(p) - 1
    b = rng.uniform(-1, 1, n)
    tol = 1e-10 * np.linalg.norm(b)
    xo, ito = O.gmres(p, i, v, b, restart, tol=tol, max_iter=3)
    gp, gi, gv = T(p), T(i), T(v)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    it = E.solve_gmres(eng, E.stop_criteria(tol, 3), restart, gp, gi, gv, T(b), x)
    assert ito > 65                   # the Krylov space grew past 64 columns
    assert within5(it, ito), (it, ito)
    assert np.linalg.norm(x.cpu().numpy() - xo) <= 1e-8 * np.linalg.norm(xo)


def test_gmres_fp32(eng, rng):
    p, i, v = P.convdiff3d(16)
    n = len(p) - 1
    v32 = v.astype(np.float32)
    b = rng.uniform(-1, 1, n).astype(np.float32)
    fo, do, _ = O.ilu_factor(p, i, v32)
    tol = 1e-5 * float(np.linalg.norm(O.ilu_apply(p, i, do, fo, b)))
    _, ito = O.gmres(p, i, v32, b, 30, tol=np.float32(tol), diag=do, ilu=fo)
    gp, gi, gv = T(p), T(i), T(v32)
    ilu = E.make_ilu(eng, gp, gi, gv)
    x = torch.zeros(n, dtype=torch.float32, device=dev)
    it = E.solve_gmres(eng, E.stop_criteria(tol), 30, gp, gi, gv, T(b), x, ilu=ilu)
    # FP32 vectors; the device rotations are in double, the oracle's FP32 GMRES rotates in float
    assert abs(it - ito) <= max(2, int(round(0.1 * ito))), (it, ito)
    xs = x.cpu().numpy().astype(np.float64)
    r = b - P.csr_matvec(p, i, v32.astype(np.float64), xs)
    assert np.linalg.norm(r) <= 1e-4 * np.linalg.norm(b)


@pytest.mark.parametrize("inner", [torch.float32, torch.bfloat16])
def test_ir_gmres(eng, rng, inner):
    p, i, v = P.convdiff3d(24)
    n = len(p) - 1
    b = rng.uniform(-1, 1, n)
    tol = 1e-9 * np.linalg.norm(b)
    fo, do, _ = O.ilu_factor(p, i, v)
    gp, gi, gv = T(p), T(i), T(v)
    A64 = E.make_sparse_matrix(eng, n, gp, gi, gv)
    Ai = E.make_sparse_matrix(eng, n, gp, gi, gv.to(inner))
    Mi = E.make_ilu(eng, gp, gi, gv, store=inner)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    rtol = 1e-4 if inner == torch.float32 else 1e-2
    info = E.solve_ir_gmres(eng, A64, Ai, Mi, 30, T(b), x, tol, inner_rtol=rtol)
    xs = x.cpu().numpy()
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, xs)) < tol
    assert info.outer >= 2
    xf, _ = O.gmres(p, i, v, b, 30, tol=1e-13 * np.linalg.norm(b), diag=do, ilu=fo)
    assert np.linalg.norm(xs - xf) <= 1e-7 * np.linalg.norm(xf)
    if inner == torch.float32:
        # the oracle's restatement of the same refinement: same sweeps, inner applications within 5%
        xo, tot, outer = O.ir_gmres(p, i, v, v.astype(np.float32), do, fo.astype(np.float32), fo[do], 30, b, tol,
                                    inner_rtol=rtol)
        assert info.outer == outer, (info.outer, outer)
        assert within5(info.iterations, tot), (info.iterations, tot)


@pytest.mark.parametrize("store", [torch.float32, torch.bfloat16])
def test_ru_pcg(eng, rng, store):
    p, i, v = P.aniso3d(32)
    n = len(p) - 1
    xt = rng.standard_normal(n)
    b = P.csr_matvec(p, i, v, xt)
    tol = 1e-10 * np.linalg.norm(b)
    fo, do, _ = O.ilu_factor(p, i, v)
    xo, ito, _ = O.cg(p, i, v, b, tol=tol, diag=do, ilu=fo)
    gp, gi, gv = T(p), T(i), T(v)
    A64 = E.make_sparse_matrix(eng, n, gp, gi, gv)
    A32 = E.make_sparse_matrix(eng, n, gp, gi, gv.to(torch.float32))
    M = E.make_ilu(eng, gp, gi, gv, store=store)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    info = E.solve_ru_pcg(eng, A64, A32, M, T(b), x, tol, delta=0.01)
    xs = x.cpu().numpy()
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, xs)) < tol
    assert abs(info.true_residual - np.linalg.norm(b - P.csr_matvec(p, i, v, xs))) <= 1e-3 * tol
    assert np.linalg.norm(xs - xo) <= 1e-7 * np.linalg.norm(xo)
    # the Krylov space is kept across updates: FP64 PCG's iterations (its count includes the
    # initial residual), not a restarted refinement's
    assert within5(info.iterations, ito - 1), (info.iterations, ito)
    if store == torch.float32:
        _, it_o, upd_o = O.ru_pcg(p, i, v, v.astype(np.float32), do, fo.astype(np.float32), fo[do], b, tol,
                                  delta=0.01)
        assert within5(info.iterations, it_o), (info.iterations, it_o)
        assert abs(info.outer - upd_o) <= 1, (info.outer, upd_o)


def test_ru_pcg_iteration_limit(eng, rng):
    from hala_gb300.hgb import HgbError
    p, i, v = P.aniso3d(16)
    n = len(p) - 1
    b = rng.standard_normal(n)
    fo, do, _ = O.ilu_factor(p, i, v)
    gp, gi, gv = T(p), T(i), T(v)
    A64 = E.make_sparse_matrix(eng, n, gp, gi, gv)
    A32 = E.make_sparse_matrix(eng, n, gp, gi, gv.to(torch.float32))
    M = E.make_ilu(eng, gp, gi, gv, store=torch.float32)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    with pytest.raises(HgbError):
        E.solve_ru_pcg(eng, A64, A32, M, T(b), x, 1e-12, max_iter=6)
    # the correction of the six iterations is in x: the oracle's iterate after the same six
    xo, it_o, _ = O.ru_pcg(p, i, v, v.astype(np.float32), do, fo.astype(np.float32), fo[do], b, 1e-12, max_iter=6)
    assert it_o == 6
    assert np.linalg.norm(x.cpu().numpy() - xo) <= 1e-5 * np.linalg.norm(xo)


@pytest.mark.parametrize("store", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("solver", ["ir", "ru"])
def test_mixed_host_buffers(eng, rng, solver, store):
    # host pntr/indx/vals/b/x in, x out: the end-to-end entry points of the mixed solves; the inner
    # operator is FP32 also beside a BF16-stored factor
    p, i, v = P.aniso3d(20)
    n = len(p) - 1
    xt = rng.standard_normal(n)
    b = P.csr_matvec(p, i, v, xt)
    tol = 1e-10 * np.linalg.norm(b)
    M = E.make_ilu(eng, T(p), T(i), T(v), store=store)
    x = np.zeros(n)
    if solver == "ir":
        info = E.solve_ir_pcg_mixed(eng, tol, p, i, v, M, b, x, inner_rtol=1e-4)
    else:
        info = E.solve_ru_pcg_mixed(eng, tol, p, i, v, M, b, x, delta=0.01)
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, x)) < tol
    assert info.true_residual < tol
    fo, do, _ = O.ilu_factor(p, i, v)
    xo, _, _ = O.cg(p, i, v, b, tol=tol, diag=do, ilu=fo)
    assert np.linalg.norm(x - xo) <= 1e-7 * np.linalg.norm(xo)


def test_ru_pcg_transposed(eng, rng):
    # op(A) = A^T through the cached transpose and the transposed ILU apply (the adjoint form); the
    # operator is symmetric (CG needs an SPD op(A)), so the 'T' solve must agree with the 'N' one
    n = 48
    p, i, v = P.vardiff2d(n, np.exp(P.grf2d(n, length=6.0, sigma=1.0, seed=3)))
    N = len(p) - 1
    b = rng.standard_normal(N)
    gp, gi, gv = T(p), T(i), T(v)
    A64 = E.make_sparse_matrix(eng, N, gp, gi, gv)
    A32 = E.make_sparse_matrix(eng, N, gp, gi, gv.to(torch.float32))
    M = E.make_ilu(eng, gp, gi, gv, store=torch.float32)
    tol = 1e-10 * np.linalg.norm(b)
    xs = {}
    for trans in "NT":
        x = torch.zeros(N, dtype=torch.float64, device=dev)
        info = E.solve_ru_pcg_op(eng, A64, A32, M, trans, T(b), x, tol, delta=0.01, max_iter=5000)
        xs[trans] = x.cpu().numpy()
        assert np.linalg.norm(b - P.csr_matvec(p, i, v, xs[trans])) < tol * 1.0001
        assert info.true_residual < tol
    assert np.linalg.norm(xs["T"] - xs["N"]) <= 1e-7 * np.linalg.norm(xs["N"])
