"""Differentiable solve on variable-coefficient 2D diffusion at full size (512 x 512 cells, theta a
Gaussian random field with squared-exponential covariance, length 16 cells, sigma 1; k = exp(theta);
L = ||u(theta, f) - u_target||^2).

The GPU gradient (mixed-precision forward solve, hand-written adjoint solve A^T lam = 2(u - u_t)
with the transposed products and triangular sweeps, dL/dvals_ij = -lam_i u_j on A's pattern,
dL/dtheta through the assembly; dL/df = lam) is checked

- against central finite differences, h = 1e-6, along 64 random directions d ~ N(0, I) in theta
  and 64 directions e ~ N(0, I) in f, with a per-direction tolerance derived from the error terms
  (see test_gradients_vs_central_differences);
- against the gradient and lam built from FP64 oracle solves (the reference's CG, to 1e-13).
"""
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
H_FD = 1e-6
DIRECTIONS = 64


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
def adjoint(setup):
    """The GPU loss and its gradients dL/dtheta and dL/df (f carries requires_grad), with the GPU
    forward solution u and adjoint solution lam."""
    st, theta, f, u_target, solver = setup
    th = theta.clone().requires_grad_(True)
    ff = f.clone().requires_grad_(True)
    L = H.loss(solver, st, th, ff, u_target)
    g_th, g_f = torch.autograd.grad(L, (th, ff))
    return float(L), g_th, g_f, solver.last["u"], solver.last["lam"]


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


def test_gradients_vs_central_differences(setup, adjoint):
    """Central differences, h = 1e-6, 64 directions in theta and 64 in f.

    For each direction the check is |fd - ad| <= E_trunc + E_round + E_adj, where
      ad      = <gradient from the GPU adjoint, direction>;
      fd      = (L(+h) - L(-h)) / 2h, each L(+-h) - L(0) = <du, du + 2 w> evaluated from the
                operator change dA (exact to rounding) and (A + dA) du = -dA u solved with an FP64
                sparse LU and defect correction (adjoint_harness.LUReference);
      E_trunc = |fd(2h) - fd(h)| / 3, the Richardson estimate of the h^2 L'''/6 truncation term
                (0 in f: L is quadratic in f, so the central difference has no truncation error);
      E_round = (bound(L(+h) - L(0)) + bound(L(-h) - L(0))) / 2h, with
                bound = 2 ||ddu|| (||du|| + ||w||) + 2 ||du|| ||dw|| + the rounding of the sum,
                ||ddu||, ||dw|| <= ||(A + dA)^-1|| (||residual|| + its FP64 rounding level);
      E_adj   = the error of the GPU gradient itself, from its solves' measured errors against the
                LU solutions: ||dlam|| ||a|| + ||du_gpu|| ||b|| + second order, a_i = sum_j |u_j| |Jd_ij|,
                b_j = sum_i |lam_i| |Jd_ij| over A's pattern (Jd: the values' derivative along d);
                in f, ||dlam|| ||e||.
    """
    st, theta, f, u_target, solver = setup
    L0, g_th, g_f, u_gpu, lam_gpu = adjoint
    n = N
    th = theta.cpu().numpy()
    p, i = st.pntr, st.indx
    vals = P.vardiff2d(n, np.exp(th))[2]
    ref = H.LUReference(p, i, vals)
    fn = f.cpu().numpy()
    ut = u_target.cpu().numpy()
    u, err_u = ref.solve(fn)
    w = u - ut
    lam, err_lam = ref.solve(2.0 * w, trans="T")
    du_gpu = float(np.linalg.norm(u_gpu.cpu().numpy() - u)) + err_u
    dlam_gpu = float(np.linalg.norm(lam_gpu.cpu().numpy() - lam)) + err_lam
    rows = np.repeat(np.arange(n * n), np.diff(p))
    gth, gf = g_th.cpu().numpy(), g_f.cpu().numpy()

    def perturbed(dA_vals, h_scale):
        """L(theta + dtheta) - L(theta) and its rounding bound for the operator change dA."""
        import scipy.sparse as sp
        dA = sp.csr_matrix((dA_vals, i, p), shape=(n * n, n * n))
        rhs = -(dA @ u)
        du, e_du = ref.solve(rhs, dA=dA)
        val, e_sum = H.loss_change(du, w)
        nd, nw = float(np.linalg.norm(du)), float(np.linalg.norm(w))
        return val, 2 * e_du * (nd + nw) + 2 * nd * err_u + e_du * e_du + e_sum

    rng = np.random.default_rng(11)
    ratios, rel = [], []
    for _ in range(DIRECTIONS):
        d = rng.standard_normal(n * n)
        fd, eround = {}, 0.0
        for hs in (1, 2):
            h = hs * H_FD
            lp, ep = perturbed(P.vardiff2d_from_faces(n, *H.face_changes(n, th, h * d))[2], hs)
            lm, em = perturbed(P.vardiff2d_from_faces(n, *H.face_changes(n, th, -h * d))[2], hs)
            fd[hs] = (lp - lm) / (2 * h)
            if hs == 1:
                eround = (ep + em) / (2 * h)
        etrunc = abs(fd[2] - fd[1]) / 3
        jd = P.vardiff2d_from_faces(n, *H.face_derivs(n, th, d))[2]
        a = np.bincount(rows, np.abs(u[i]) * np.abs(jd), n * n)
        b = np.bincount(i, np.abs(lam[rows]) * np.abs(jd), n * n)
        q = -lam[rows] * u[i]
        eadj = (dlam_gpu * float(np.linalg.norm(a)) + du_gpu * float(np.linalg.norm(b))
                + 5 * dlam_gpu * du_gpu * float(np.abs(jd).max()) + 8 * H.EPS * float(np.sum(np.abs(q * jd))))
        ad = float(gth @ d)
        tol = etrunc + eround + eadj
        ratios.append(abs(fd[1] - ad) / tol)
        rel.append(abs(fd[1] - ad) / abs(ad))
    ratios, rel = np.array(ratios), np.array(rel)
    assert ratios.max() <= 1.0, (ratios.max(), np.median(rel), rel.max())
    # the tolerance is not vacuous: it is a small fraction of the directional derivative
    assert np.median(rel) < 1e-4, np.median(rel)

    ratios_f, rel_f = [], []
    for _ in range(DIRECTIONS):
        e = rng.standard_normal(n * n)
        z, e_z = ref.solve(e)
        lp, ep = H.loss_change(H_FD * z, w)
        lm, em = H.loss_change(-H_FD * z, w)
        nz, nw = H_FD * float(np.linalg.norm(z)), float(np.linalg.norm(w))
        bound = lambda es: 2 * H_FD * e_z * (nz + nw) + 2 * nz * err_u + es   # noqa: E731
        fd = (lp - lm) / (2 * H_FD)
        eround = (bound(ep) + bound(em)) / (2 * H_FD)
        ad = float(gf @ e)
        tol = eround + dlam_gpu * float(np.linalg.norm(e))
        ratios_f.append(abs(fd - ad) / tol)
        rel_f.append(abs(fd - ad) / abs(ad))
    ratios_f, rel_f = np.array(ratios_f), np.array(rel_f)
    assert ratios_f.max() <= 1.0, (ratios_f.max(), np.median(rel_f), rel_f.max())
    assert np.median(rel_f) < 1e-4, np.median(rel_f)


def test_gradient_vs_fp64_oracle(setup, adjoint):
    st, theta, f, u_target, solver = setup
    L0, g, g_f, u_gpu, lam_gpu = adjoint
    # FP64 oracle: u = A^-1 f, lam = A^-T 2(u - u_t) (A symmetric), dL/dvals = -lam_i u_j, dL/df = lam
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
    rel_lam = float(np.linalg.norm(g_f.cpu().numpy() - lam) / np.linalg.norm(lam))
    assert rel_lam < 1e-5, rel_lam


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
