"""Test harness for the differentiable solve (variable-coefficient 2D diffusion), and the accurate
CPU references of its finite-difference check.

-div(k grad u) = f on an n x n grid of unit cells (5-point finite volumes, face conductivity the
harmonic mean of the two cells, Dirichlet faces 2 k_cell), k = exp(theta).  Loss
L = ||u(theta) - u_target||^2.  The solve is a torch.autograd.Function: forward = mixed precision
ILU(0)-PCG (FP32 PCG with FP64 reliable updates) through the C ABI; backward = the hand-written adjoint:
A^T lam = dL/du by the same solver on the transposed operator, dL/df = lam and
dL/dA_ij = -lam_i u_j on A's pattern (hgb_csr_pattern_grad).  dL/dtheta follows by autograd
through the assembly below.
"""
import numpy as np
import torch

from hala_gb300 import engine as E
from hala_gb300 import problems as P
from hala_gb300.hgb import HGB_ERR_NOT_CONVERGED, HgbError


class Stencil:
    """Pattern of the 5-point operator and the mask that maps (row, offset) -> CSR position."""

    def __init__(self, n, device):
        self.n = n
        k1 = np.ones(n * n)
        p, i, _ = P.vardiff2d(n, k1)
        self.pntr, self.indx = p, i
        N = n * n
        x = np.arange(N) % n
        y = np.arange(N) // n
        # offsets in column order: south, west, diagonal, east, north (problems._stencil_csr)
        valid = np.stack([y > 0, x > 0, np.ones(N, bool), x < n - 1, y < n - 1], 1)
        self.valid = torch.from_numpy(valid.reshape(-1)).to(device)
        self.gp = torch.from_numpy(p).to(device)
        self.gi = torch.from_numpy(i).to(device)


def assemble(st, theta):
    """CSR values of the operator for conductivity exp(theta) (differentiable in theta)."""
    n = st.n
    k = torch.exp(theta).reshape(n, n)                       # [y][x]
    kx = torch.empty(n, n + 1, dtype=k.dtype, device=k.device)
    kx[:, 1:-1] = 2 * k[:, :-1] * k[:, 1:] / (k[:, :-1] + k[:, 1:])
    kx[:, 0] = 2 * k[:, 0]
    kx[:, -1] = 2 * k[:, -1]
    ky = torch.empty(n + 1, n, dtype=k.dtype, device=k.device)
    ky[1:-1, :] = 2 * k[:-1, :] * k[1:, :] / (k[:-1, :] + k[1:, :])
    ky[0, :] = 2 * k[0, :]
    ky[-1, :] = 2 * k[-1, :]
    west, east = kx[:, :-1].reshape(-1), kx[:, 1:].reshape(-1)
    south, north = ky[:-1, :].reshape(-1), ky[1:, :].reshape(-1)
    diag = west + east + south + north
    full = torch.stack([-south, -west, diag, -east, -north], 1).reshape(-1)
    return full[st.valid]


class Solver:
    def __init__(self, eng, st, tol=1e-12, inner_rtol=1e-3, max_inner=3000):
        # FP32 CG on this kappa ~ 1e6 operator stagnates near 1e-4 relative: the inner solves ask
        # for 1e-3 and the FP64 refinement carries the accuracy
        self.eng, self.st, self.tol, self.inner_rtol, self.max_inner = eng, st, tol, inner_rtol, max_inner
        self.last = None

    def _setup(self, vals):
        st = self.st
        n = st.n * st.n
        v64 = vals.detach().contiguous()
        v32 = v64.float()
        A64 = E.make_sparse_matrix(self.eng, n, st.gp, st.gi, v64)
        A32 = E.make_sparse_matrix(self.eng, n, st.gp, st.gi, v32)
        M = E.make_ilu(self.eng, st.gp, st.gi, v64, store=torch.float32)
        return (A64, A32, M, v64, v32)

    def solve(self, vals, rhs, trans="N", ops=None, sweeps=None):
        """sweeps=None: refine to tol; sweeps=k: exactly k refinement sweeps (no tolerance), which
        drives the error to the FP64 floor kappa*eps (used by the finite-difference check)."""
        ops = ops or self._setup(vals)
        A64, A32, M = ops[:3]
        x = torch.zeros_like(rhs)
        if sweeps is None:
            # to the tolerance: FP32 PCG with FP64 reliable updates (one Krylov space; on this
            # operator about 1.2x the FP64 iterations, where restarted refinement needs 1.5x and more)
            tol = self.tol * float(torch.linalg.vector_norm(rhs))
            E.solve_ru_pcg_op(self.eng, A64, A32, M, trans, rhs.contiguous(), x, tol, delta=0.01, max_iter=20000)
        else:
            try:
                E.solve_ir_pcg_op(self.eng, A64, A32, M, trans, rhs.contiguous(), x, 0.0, inner_rtol=self.inner_rtol,
                                  max_inner=self.max_inner, max_outer=sweeps)
            except HgbError as e:     # a zero tolerance is never met: the sweeps ran out, x is final
                if e.status != HGB_ERR_NOT_CONVERGED:
                    raise
        return x, ops


class DiffSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vals, f, solver):
        u, ops = solver.solve(vals, f)
        ctx.solver, ctx.ops = solver, ops
        ctx.save_for_backward(u)
        solver.last = {"u": u.detach().clone()}
        return u

    @staticmethod
    def backward(ctx, gu):
        (u,) = ctx.saved_tensors
        solver, ops = ctx.solver, ctx.ops
        lam, _ = solver.solve(None, gu.contiguous(), trans="T", ops=ops)
        gvals = torch.empty_like(ops[3])
        E.pattern_grad(ops[0], -1.0, lam, u, gvals)
        solver.last["lam"] = lam.detach().clone()
        return gvals, lam, None


def loss(solver, st, theta, f, u_target):
    vals = assemble(st, theta)
    u = DiffSolve.apply(vals, f, solver)
    return torch.sum((u - u_target) ** 2)


def loss_converged(solver, st, theta, f, u_target, sweeps=12):
    """L(theta) from a solve run for a fixed number of sweeps past convergence (no autograd)."""
    with torch.no_grad():
        u, _ = solver.solve(assemble(st, theta), f, sweeps=sweeps)
        return torch.sum((u - u_target) ** 2)


# ------------------------------------------------------------------------------------------------
# Accurate CPU references for the finite-difference check (sparse LU, FP64, refined).
#
# A central difference (L(theta + h d) - L(theta - h d)) / 2h with h = 1e-6 divides the rounding
# error of the two losses by 2h; losses evaluated separately from FP64 solves carry errors of
# about kappa * eps ~ 1e-10 relative, which would swamp the difference.  So each perturbed loss is
# evaluated as L(theta) + <du, du + 2 w> with w = u - u_target and du the solution of
# (A + dA) du = -dA u, dA the exact-to-rounding change of the operator's values (face
# conductivities changed through expm1, no cancellation) and du solved with the LU of A plus
# defect correction.  The rounding left is a few eps relative to the (small) du.
# ------------------------------------------------------------------------------------------------
EPS = float(np.finfo(np.float64).eps)


def face_changes(n, theta, dl):
    """Changes of the face conductivities of k = exp(theta) when theta -> theta + dl, without
    cancellation: interior faces H = 2 / (1/ka + 1/kb) change by -2 ds / (s (s + ds)) with
    ds = expm1(-da)/ka + expm1(-db)/kb; boundary faces 2k change by 2 k expm1(dl)."""
    k = np.exp(theta).reshape(n, n)
    dl = dl.reshape(n, n)
    inv = 1.0 / k
    e = np.expm1(-dl) * inv
    dkx = np.empty((n, n + 1))
    s, ds = inv[:, :-1] + inv[:, 1:], e[:, :-1] + e[:, 1:]
    dkx[:, 1:-1] = -2.0 * ds / (s * (s + ds))
    dkx[:, 0] = 2.0 * k[:, 0] * np.expm1(dl[:, 0])
    dkx[:, -1] = 2.0 * k[:, -1] * np.expm1(dl[:, -1])
    dky = np.empty((n + 1, n))
    s, ds = inv[:-1, :] + inv[1:, :], e[:-1, :] + e[1:, :]
    dky[1:-1, :] = -2.0 * ds / (s * (s + ds))
    dky[0, :] = 2.0 * k[0, :] * np.expm1(dl[0, :])
    dky[-1, :] = 2.0 * k[-1, :] * np.expm1(dl[-1, :])
    return dkx, dky


def face_derivs(n, theta, d):
    """Derivative of the face conductivities along d (the operator's Jacobian times d)."""
    k = np.exp(theta).reshape(n, n)
    d = d.reshape(n, n)
    inv = 1.0 / k
    dkx = np.empty((n, n + 1))
    s = inv[:, :-1] + inv[:, 1:]
    dkx[:, 1:-1] = 2.0 * (d[:, :-1] * inv[:, :-1] + d[:, 1:] * inv[:, 1:]) / (s * s)
    dkx[:, 0] = 2.0 * k[:, 0] * d[:, 0]
    dkx[:, -1] = 2.0 * k[:, -1] * d[:, -1]
    dky = np.empty((n + 1, n))
    s = inv[:-1, :] + inv[1:, :]
    dky[1:-1, :] = 2.0 * (d[:-1, :] * inv[:-1, :] + d[1:, :] * inv[1:, :]) / (s * s)
    dky[0, :] = 2.0 * k[0, :] * d[0, :]
    dky[-1, :] = 2.0 * k[-1, :] * d[-1, :]
    return dkx, dky


class LUReference:
    """FP64 sparse LU of A (SuperLU) with defect correction, for solutions accurate to about
    kappa * eps, and the a-posteriori error bounds the finite-difference tolerance uses."""

    def __init__(self, pntr, indx, vals):
        import scipy.sparse as sp
        import scipy.sparse.linalg as sla
        n = len(pntr) - 1
        self.pntr, self.indx, self.vals = pntr, indx, vals
        self.A = sp.csr_matrix((vals, indx, pntr), shape=(n, n))
        self.absA = sp.csr_matrix((np.abs(vals), indx, pntr), shape=(n, n))
        self.lu = sla.splu(self.A.tocsc(), permc_spec="MMD_AT_PLUS_A")
        self.row_len = int(np.diff(pntr).max())
        # ||A^-1||_2 (A symmetric positive definite): power iteration on A^-1, with a margin for
        # the Rayleigh quotient approaching the largest eigenvalue from below
        v = np.random.default_rng(7).standard_normal(n)
        v /= np.linalg.norm(v)
        lam = 0.0
        for _ in range(40):
            z = self.lu.solve(v)
            lam = float(v @ z)
            v = z / np.linalg.norm(z)
        self.inv_norm = 1.25 * lam

    def floor(self, x, b, dA=None):
        """Rounding level of a residual b - (A + dA) x computed in FP64."""
        t = self.absA @ np.abs(x) + np.abs(b)
        if dA is not None:
            t = t + np.abs(dA) @ np.abs(x)
        return (self.row_len + 2) * EPS * float(np.linalg.norm(t))

    def solve(self, b, dA=None, trans="N", sweeps=3):
        """x with (A + dA) x = b (or A^T x = b); returns x and a bound on ||x - x_exact||."""
        x = self.lu.solve(b, trans=trans)
        op = (lambda y: self.A @ y) if trans == "N" else (lambda y: self.A.T @ y)
        for _ in range(sweeps):
            r = b - op(x) if dA is None else b - op(x) - dA @ x
            x = x + self.lu.solve(r, trans=trans)
        r = b - op(x) if dA is None else b - op(x) - dA @ x
        # ||(A + dA)^-1|| <= ||A^-1|| / (1 - ||A^-1|| ||dA||), ||dA||_2 <= ||dA||_1,inf bound
        mu = self.inv_norm
        if dA is not None:
            nd = float(np.sqrt(abs(dA).sum(axis=0).max() * abs(dA).sum(axis=1).max()))
            mu = mu / max(1e-3, 1.0 - mu * nd)
        return x, mu * (float(np.linalg.norm(r)) + self.floor(x, b, dA))


def loss_change(du, w):
    """L(u + du) - L(u) = <du, du + 2 w> (exactly rounded sum) and its rounding bound."""
    import math
    prod = du * (du + 2.0 * w)
    val = math.fsum(prod)
    return val, 3 * EPS * float(np.sum(np.abs(du) * (np.abs(du) + 2.0 * np.abs(w)))) + EPS * abs(val)
