"""Differentiable solve on variable-coefficient 2D diffusion: the adjoint gradient dL/dtheta on a
512 x 512 grid against the gradient built from FP64 oracle solves, and on a 64 x 64 grid against
central finite differences (h = 1e-6, 24 random directions); plus the transposed solvers against
their 'N' forms."""
import numpy as np
import pytest
import torch

from hala_gb300 import engine as E
from hala_gb300 import problems as P
from oracle import oracle as O
from tests import adjoint_harness as H

pytestmark = pytest.mark.gpu
dev = torch.device("cuda")
N = 512
N_FD = 64


def _problem(eng, n, length):
    st = H.Stencil(n, dev)
    theta = torch.from_numpy(P.grf2d(n, length=length, sigma=1.0, seed=1)).to(dev)
    theta2 = torch.from_numpy(P.grf2d(n, length=length, sigma=1.0, seed=2)).to(dev)
    f = torch.ones(n * n, dtype=torch.float64, device=dev)
    # 3e-11: just above the FP64 residual floor of the 512 x 512 system (||A|| ||u|| eps ~ 1.3e-11 ||f||)
    solver = H.Solver(eng, st, tol=3e-11)
    with torch.no_grad():
        u_target, _ = solver.solve(H.assemble(st, theta2), f)
    return st, theta, f, u_target, solver


@pytest.fixture(scope="module")
def setup(eng):
    return _problem(eng, N, 16.0)


@pytest.fixture(scope="module")
def setup_fd(eng):
    return _problem(eng, N_FD, 4.0)


def test_forward_solve_accuracy(setup):
    st, theta, f, u_target, solver = setup
    vals = H.assemble(st, theta).detach()
    u, _ = solver.solve(vals, f)
    p, i = st.pntr, st.indx
    vn, un = vals.cpu().numpy(), u.cpu().numpy()
    r = f.cpu().numpy() - P.csr_matvec(p, i, vn, un)
    # the solver stops on its own FP64 residual; recomputing it here adds rounding of the order
    # eps * || |A| |u| ||
    floor = np.finfo(np.float64).eps * np.linalg.norm(P.csr_matvec(p, i, np.abs(vn), np.abs(un)))
    assert np.linalg.norm(r) <= 3e-11 * np.linalg.norm(f.cpu().numpy()) + 4 * floor


def test_gradient_vs_central_differences(setup_fd):
    st, theta, f, u_target, solver = setup_fd
    th = theta.clone().requires_grad_(True)
    L = H.loss(solver, st, th, f, u_target)
    (g,) = torch.autograd.grad(L, th)
    rng = np.random.default_rng(11)
    h = 1e-6
    errs = []
    with torch.no_grad():
        for _ in range(24):
            d = torch.from_numpy(rng.standard_normal(N_FD * N_FD)).to(dev)
            d /= torch.linalg.vector_norm(d)
            lp = H.loss_converged(solver, st, theta + h * d, f, u_target, sweeps=8)
            lm = H.loss_converged(solver, st, theta - h * d, f, u_target, sweeps=8)
            fd = float((lp - lm) / (2 * h))
            ad = float(torch.dot(g, d))
            errs.append(abs(fd - ad) / max(abs(ad), 1e-30 * float(L)))
    # the FD losses come from solves refined to the FP64 floor (error ~ kappa * eps); the exact
    # check of the adjoint is test_gradient_vs_fp64_oracle
    errs = np.array(errs)
    assert np.median(errs) < 1e-2 and np.quantile(errs, 0.9) < 5e-2, (np.median(errs), np.quantile(errs, 0.9))


def test_gradient_vs_fp64_oracle(setup):
    st, theta, f, u_target, solver = setup
    th = theta.clone().requires_grad_(True)
    L = H.loss(solver, st, th, f, u_target)
    (g,) = torch.autograd.grad(L, th)
    # FP64 oracle: u = A^-1 f, lam = A^-T 2(u - u_t) (A symmetric), dL/dvals = -lam_i u_j
    vals = H.assemble(st, theta).detach().cpu().numpy()
    p, i = st.pntr, st.indx
    fo, do, _ = O.ilu_factor(p, i, vals)
    fn = f.cpu().numpy()
    u, _, _ = O.cg(p, i, vals, fn, tol=1e-13 * np.linalg.norm(fn), diag=do, ilu=fo)
    gu = 2 * (u - u_target.cpu().numpy())
    lam, _, _ = O.cg(p, i, vals, gu, tol=1e-13 * np.linalg.norm(gu), diag=do, ilu=fo)
    rows = np.repeat(np.arange(len(p) - 1), np.diff(p))
    gvals = torch.from_numpy(-lam[rows] * u[i]).to(dev)
    th2 = theta.clone().requires_grad_(True)
    (g64,) = torch.autograd.grad(H.assemble(st, th2), th2, grad_outputs=gvals)
    rel = float(torch.linalg.vector_norm(g - g64) / torch.linalg.vector_norm(g64))
    assert rel < 1e-5, rel


def test_transposed_cg_matches_forward(eng, rng):
    p, i, v = P.aniso3d(20)
    n = len(p) - 1
    b = rng.standard_normal(n)
    gp, gi, gv = (torch.from_numpy(a).to(dev) for a in (p, i, v))
    A = E.make_sparse_matrix(eng, n, gp, gi, gv)
    M = E.make_ilu(eng, gp, gi, gv)
    gb = torch.from_numpy(b).to(dev)
    tol = 1e-11 * np.linalg.norm(b)
    xn = torch.zeros(n, dtype=torch.float64, device=dev)
    xt = torch.zeros(n, dtype=torch.float64, device=dev)
    inf_n = E.solve_cg_op(eng, A, M, "N", gb, xn, tol)
    inf_t = E.solve_cg_op(eng, A, M, "T", gb, xt, tol)
    # A symmetric: A^T = A and (LU)^T = LU up to rounding, so both solves agree
    assert abs(inf_n.iterations - inf_t.iterations) <= 2
    assert float(torch.linalg.vector_norm(xn - xt) / torch.linalg.vector_norm(xn)) < 1e-9
