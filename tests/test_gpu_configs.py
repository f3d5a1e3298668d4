"""Parity at the full sizes of the benchmark workloads (the other GPU tests use scaled-down
versions of the same operators).

- 256^2 2D Poisson, unpreconditioned CG to 1e-10 relative residual (n = 65,536);
- 128^3 anisotropic 3D Poisson (1, 1, 0.01), ILU(0)-PCG to 1e-10: FP64, then mixed FP32 inner
  PCG (FP32 or BF16 ILU store) with FP64 refinement, each against the FP64 oracle solve
  (n = 2,097,152);
- 96^3 upwind convection-diffusion (v = (1, 0.5, 0.25), cell Peclet 10), ILU(0)-GMRES(30) to
  1e-9 of the preconditioned residual, then mixed FP32 / BF16 inner GMRES(30) with FP64
  refinement to a 1e-9 true relative residual (n = 884,736);
- 4,096 independent Erdos-Renyi Laplacians, n_i log-uniform on [64, 4096], FP32 values with
  FP64 refinement, 1e-8 per system.

The oracle is the reference's algorithm on the CPU (solve_cg, hex/solvers/hala_solvers_cg.hpp:92-227;
solve_gmres, hex/solvers/hala_solvers_gmres.hpp:127-267).  Reductions on the GPU are parallel, so
the Krylov recurrences agree to rounding: iteration counts within 5%, iterates within a
conditioning-scaled tolerance."""
import numpy as np
import pytest
import torch

from hala_gb300 import engine as E
from hala_gb300 import problems as P
from oracle import oracle as O

pytestmark = pytest.mark.gpu
dev = torch.device("cuda")


def T(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def within5(a, b):
    return abs(a - b) <= max(1, int(round(0.05 * b)))


def test_cg_poisson256(eng):
    p, i, v = P.poisson2d(256)
    n = len(p) - 1
    assert n == 65536 and len(i) == 326656
    xt = np.random.default_rng(1).uniform(-1, 1, n)
    b = P.csr_matvec(p, i, v, xt)
    tol = 1e-10 * np.linalg.norm(b)
    xo, ito, _ = O.cg(p, i, v, b, tol=tol)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    it = E.solve_cg(eng, E.stop_criteria(tol), T(p), T(i), T(v), T(b), x)
    assert within5(it, ito), (it, ito)
    xs = x.cpu().numpy()
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, xs)) < 2 * tol
    assert np.linalg.norm(xs - xo) <= 1e-8 * np.linalg.norm(xo)


@pytest.fixture(scope="module")
def aniso128(eng):
    p, i, v = P.aniso3d(128)
    n = len(p) - 1
    xt = np.random.default_rng(2).standard_normal(n)
    b = P.csr_matvec(p, i, v, xt)
    tol = 1e-10 * np.linalg.norm(b)
    fo, do, _ = O.ilu_factor(p, i, v)
    xo, ito, _ = O.cg(p, i, v, b, tol=tol, diag=do, ilu=fo)
    return p, i, v, xt, b, tol, xo, ito


def test_pcg_aniso128_fp64(eng, aniso128):
    p, i, v, xt, b, tol, xo, ito = aniso128
    n = len(p) - 1
    assert n == 2097152 and len(i) == 14581760
    gp, gi, gv = T(p), T(i), T(v)
    ilu = E.make_ilu(eng, gp, gi, gv)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    it = E.solve_cg(eng, E.stop_criteria(tol), gp, gi, gv, T(b), x, ilu=ilu)
    assert within5(it, ito), (it, ito)
    xs = x.cpu().numpy()
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, xs)) < 2 * tol
    assert np.linalg.norm(xs - xo) <= 1e-7 * np.linalg.norm(xo)


# The refinement's operator is FP32.  A BF16 operator does not refine at this size: BF16 rounds
# the diagonal 4.02 to 4.03125, a shift of 0.011 = 9x the smallest eigenvalue (1.2e-3), and
# refinement around (A + 0.011 I)^-1 contracts by ~0.9 per sweep (it converges on 32^3, where
# the same shift is 0.6x the smallest eigenvalue).  BF16 serves as the preconditioner's store.
@pytest.mark.parametrize("store", [torch.float32, torch.bfloat16])
def test_pcg_aniso128_mixed(eng, aniso128, store):
    p, i, v, xt, b, tol, xo, ito = aniso128
    n = len(p) - 1
    gp, gi, gv = T(p), T(i), T(v)
    A64 = E.make_sparse_matrix(eng, n, gp, gi, gv)
    Ai = E.make_sparse_matrix(eng, n, gp, gi, gv.to(torch.float32))
    Mi = E.make_ilu(eng, gp, gi, gv, store=store)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    info = E.solve_ir_pcg(eng, A64, Ai, Mi, T(b), x, tol, inner_rtol=1e-4)
    xs = x.cpu().numpy()
    # the refinement stops on the true FP64 residual
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, xs)) < tol
    # same residual target as the FP64 oracle: the iterates agree to conditioning x 1e-10
    assert np.linalg.norm(xs - xo) <= 1e-7 * np.linalg.norm(xo)
    err, err_o = np.linalg.norm(xs - xt), np.linalg.norm(xo - xt)
    assert err <= 5 * err_o + 1e-12 * np.linalg.norm(xt), (err, err_o)
    assert info.outer >= 2


def test_ru_pcg_aniso128(eng, aniso128):
    # mixed FP32 PCG with FP64 reliable updates: FP64 PCG's iteration count at 128^3
    p, i, v, xt, b, tol, xo, ito = aniso128
    n = len(p) - 1
    gp, gi, gv = T(p), T(i), T(v)
    A64 = E.make_sparse_matrix(eng, n, gp, gi, gv)
    A32 = E.make_sparse_matrix(eng, n, gp, gi, gv.to(torch.float32))
    M32 = E.make_ilu(eng, gp, gi, gv, store=torch.float32)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    info = E.solve_ru_pcg(eng, A64, A32, M32, T(b), x, tol, delta=0.01)
    xs = x.cpu().numpy()
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, xs)) < tol
    assert np.linalg.norm(xs - xo) <= 1e-7 * np.linalg.norm(xo)
    assert within5(info.iterations, ito - 1), (info.iterations, ito)


def test_pcg_aniso128_fused_spmv(eng_fused, aniso128):
    # the benchmark's forms in the default SpMV mode (one FMA per entry): FP64 PCG and the mixed
    # reliable-update PCG, against the FP64 oracle's iteration count and solution
    p, i, v, xt, b, tol, xo, ito = aniso128
    n = len(p) - 1
    gp, gi, gv = T(p), T(i), T(v)
    A64 = E.make_sparse_matrix(eng_fused, n, gp, gi, gv)
    M64 = E.make_ilu(eng_fused, gp, gi, gv)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    info = E.solve_cg_info(eng_fused, A64, M64, T(b), x, tol)
    assert within5(info.iterations, ito), (info.iterations, ito)
    xs = x.cpu().numpy()
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, xs)) < 2 * tol
    assert np.linalg.norm(xs - xo) <= 1e-7 * np.linalg.norm(xo)
    A32 = E.make_sparse_matrix(eng_fused, n, gp, gi, gv.to(torch.float32))
    M32 = E.make_ilu(eng_fused, gp, gi, gv, store=torch.float32)
    x.zero_()
    info = E.solve_ru_pcg(eng_fused, A64, A32, M32, T(b), x, tol, delta=0.01)
    xs = x.cpu().numpy()
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, xs)) < tol
    assert np.linalg.norm(xs - xo) <= 1e-7 * np.linalg.norm(xo)
    assert within5(info.iterations, ito - 1), (info.iterations, ito)


@pytest.fixture(scope="module")
def convdiff96(eng):
    p, i, v = P.convdiff3d(96)
    n = len(p) - 1
    b = np.random.default_rng(3).uniform(-1, 1, n)
    fo, do, _ = O.ilu_factor(p, i, v)
    tol = 1e-9 * np.linalg.norm(O.ilu_apply(p, i, do, fo, b))
    xo, ito = O.gmres(p, i, v, b, 30, tol=tol, diag=do, ilu=fo)
    return p, i, v, b, fo, do, tol, xo, ito


def test_gmres_convdiff96(eng, convdiff96):
    p, i, v, b, fo, do, tol, xo, ito = convdiff96
    n = len(p) - 1
    assert n == 884736 and len(i) == 6137856
    gp, gi, gv = T(p), T(i), T(v)
    ilu = E.make_ilu(eng, gp, gi, gv)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    it = E.solve_gmres(eng, E.stop_criteria(tol), 30, gp, gi, gv, T(b), x, ilu=ilu)
    assert within5(it, ito), (it, ito)
    xs = x.cpu().numpy()
    assert np.linalg.norm(xs - xo) <= 1e-7 * np.linalg.norm(xo)
    # the true relative residual of both solves is of the order of the preconditioned target
    rt = np.linalg.norm(b - P.csr_matvec(p, i, v, xs)) / np.linalg.norm(b)
    ro = np.linalg.norm(b - P.csr_matvec(p, i, v, xo)) / np.linalg.norm(b)
    assert rt <= 2 * ro + 1e-12, (rt, ro)


@pytest.mark.parametrize("inner", [torch.float32, torch.bfloat16])
def test_ir_gmres_convdiff96(eng, convdiff96, inner):
    # mixed form: FP32 / BF16 inner GMRES(30), FP64 refinement to a 1e-9 true relative residual
    p, i, v, b, fo, do, tol, xo, ito = convdiff96
    n = len(p) - 1
    gp, gi, gv = T(p), T(i), T(v)
    A64 = E.make_sparse_matrix(eng, n, gp, gi, gv)
    Ai = E.make_sparse_matrix(eng, n, gp, gi, gv.to(inner))
    Mi = E.make_ilu(eng, gp, gi, gv, store=inner)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    rtol = 1e-4 if inner == torch.float32 else 1e-2
    target = 1e-9 * np.linalg.norm(b)
    info = E.solve_ir_gmres(eng, A64, Ai, Mi, 30, T(b), x, target, inner_rtol=rtol)
    xs = x.cpu().numpy()
    assert np.linalg.norm(b - P.csr_matvec(p, i, v, xs)) < target
    # error against the FP64 oracle solve (stopped on the preconditioned residual 1e-9)
    assert np.linalg.norm(xs - xo) <= 1e-7 * np.linalg.norm(xo)
    if inner == torch.float32:
        xr, tot, outer = O.ir_gmres(p, i, v, v.astype(np.float32), do, fo.astype(np.float32), fo[do], 30, b, target,
                                    inner_rtol=rtol)
        assert info.outer == outer, (info.outer, outer)
        assert within5(info.iterations, tot), (info.iterations, tot)


def test_batch_4096_systems(eng):
    S = 4096
    sp, p, i, v = P.er_laplacian_batch(S, 64, 4096, seed=4)
    nt = len(p) - 1
    b = np.random.default_rng(5).uniform(-1, 1, nt)
    B = E.gpu_batch(eng, T(sp), T(p), T(i), T(v))
    x = torch.zeros(nt, dtype=torch.float64, device=dev)
    iters = torch.zeros(S, dtype=torch.int32, device=dev)
    rel = torch.zeros(S, dtype=torch.float64, device=dev)
    B.solve(T(b), x, rtol=1e-8, iters=iters, relres=rel)
    xs = x.cpu().numpy()
    v64 = v.astype(np.float64)       # the systems are the FP32-stored matrices
    r = b - P.csr_matvec(p, i, v64, xs)
    rn = np.sqrt(np.add.reduceat(r * r, sp[:-1]))
    bn = np.sqrt(np.add.reduceat(b * b, sp[:-1]))
    assert np.all(rn <= 1e-8 * bn * 1.0001), int(np.argmax(rn / bn))
    assert np.all(rel.cpu().numpy() <= 1e-8)
    assert np.all(iters.cpu().numpy() > 0)
    for s in range(0, S, 16):       # every 16th system against the oracle's solve_cg
        r0, r1 = sp[s], sp[s + 1]
        ps = (p[r0:r1 + 1] - p[r0]).astype(np.int32)
        iS = (i[p[r0]:p[r1]] - r0).astype(np.int32)
        bs = b[r0:r1]
        xo, _, _ = O.cg(ps, iS, v64[p[r0]:p[r1]], bs, tol=1e-12 * np.linalg.norm(bs), max_iter=20000)
        assert np.linalg.norm(xs[r0:r1] - xo) <= 1e-6 * np.linalg.norm(xo), s
