"""SpMV and BLAS-1 on the GPU, through the C ABI, against the CPU oracle.

Tolerances: in the exact SpMV mode 'N' products (and the cached transpose) are compared
BIT-EXACTLY with the oracle's sequential row loop; in the default fused mode (one FMA per entry)
within 1e-14 relative (norm-wise, and per row within the rounding bound of the row's sum) in FP64
and 1e-6 in FP32; the atomic transpose and the reductions (dot, nrm2, fused dot) within 1e-13
relative in FP64 and 1e-6 in FP32."""
import numpy as np
import pytest
import torch

from hala_gb300 import engine as E
from hala_gb300 import problems as P
from hala_gb300.hgb import HgbError, HGB_ERR_CSR
from oracle import oracle as O
from tests import refcases as R

pytestmark = pytest.mark.gpu
dev = torch.device("cuda")


def T(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def irregular(rng, n=1500):
    """rows of 0..40 entries, several empty rows, one long row (forces the global-load tile path)"""
    lens = rng.integers(0, 40, size=n)
    lens[rng.integers(0, n, 20)] = 0
    lens[7] = n  # full row
    rows, cols = [], []
    for r, L in enumerate(lens):
        c = np.sort(rng.choice(n, size=min(L, n), replace=False))
        rows.append(np.full(len(c), r))
        cols.append(c)
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    p = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(r, minlength=n), out=p[1:])
    return p.astype(np.int32), c.astype(np.int32), rng.uniform(-1, 1, len(c))


CASES = {
    "aniso3d_24": lambda rng: P.aniso3d(24, 23, 22),
    "poisson2d_100": lambda rng: P.poisson2d(100, 37),
    "convdiff3d_17": lambda rng: P.convdiff3d(17),
    "irregular": irregular,
    "one_row": lambda rng: (np.array([0, 3], np.int32), np.array([0, 1, 2], np.int32), np.array([1.0, 2.0, 3.0])),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("ab", [(1.0, 0.0), (2.0, 0.0), (-1.0, 1.0), (0.5, -0.25)])
def test_spmv_n_f64_bit_exact(eng, rng, name, ab):
    p, i, v = CASES[name](rng)
    m = len(p) - 1
    ncols = int(i.max()) + 1 if len(i) else 1
    x = rng.standard_normal(ncols)
    y0 = rng.standard_normal(m)
    alpha, beta = ab
    ref = O.spmv("N", m, ncols, alpha, p, i, v, x, beta, y0)
    gy = T(y0)
    E.sparse_gemv(eng, "N", m, ncols, alpha, T(p), T(i), T(v), T(x), beta, gy)
    assert np.array_equal(gy.cpu().numpy(), ref)


def _row_bound(p, i, v, x, alpha, beta, y0, eps):
    """Per-row bound on the difference of two roundings of alpha * sum_j a_ij x_j + beta * y_i
    (each within gamma_k * sum of |terms|, k = row length + 3)."""
    n = len(p) - 1
    s = np.zeros(n)
    lens = np.diff(p)
    rows = np.repeat(np.arange(n), lens)
    np.add.at(s, rows, np.abs(v * x[i]))
    k = lens + 3
    mag = np.abs(alpha) * s + (np.abs(beta * y0) if beta != 0 else 0.0)
    return 2 * k * eps * mag


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("ab", [(1.0, 0.0), (2.0, 0.0), (-1.0, 1.0), (0.5, -0.25)])
def test_spmv_n_fused_f64_within_1e14(eng_fused, rng, name, ab):
    p, i, v = CASES[name](rng)
    m = len(p) - 1
    ncols = int(i.max()) + 1 if len(i) else 1
    x = rng.standard_normal(ncols)
    y0 = rng.standard_normal(m)
    alpha, beta = ab
    ref = O.spmv("N", m, ncols, alpha, p, i, v, x, beta, y0)
    gy = T(y0)
    E.sparse_gemv(eng_fused, "N", m, ncols, alpha, T(p), T(i), T(v), T(x), beta, gy)
    y = gy.cpu().numpy()
    assert np.linalg.norm(y - ref) <= 1e-14 * np.linalg.norm(ref)
    assert np.all(np.abs(y - ref) <= _row_bound(p, i, v, x, alpha, beta, y0, 2.0**-53))


@pytest.mark.parametrize("name", list(CASES))
def test_spmv_n_fused_f32_within_1e6(eng_fused, rng, name):
    p, i, v = CASES[name](rng)
    m = len(p) - 1
    ncols = int(i.max()) + 1 if len(i) else 1
    x = rng.standard_normal(ncols).astype(np.float32)
    v32 = v.astype(np.float32)
    ref = O.spmv("N", m, ncols, 1.0, p, i, v32, x, 0.0)
    gy = torch.zeros(m, dtype=torch.float32, device=dev)
    E.sparse_gemv(eng_fused, "N", m, ncols, 1.0, T(p), T(i), T(v32), T(x), 0.0, gy)
    y = gy.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(y - ref) <= 1e-6 * np.linalg.norm(ref)
    bound = _row_bound(p, i, v32.astype(np.float64), x.astype(np.float64), 1.0, 0.0, None, 2.0**-24)
    assert np.all(np.abs(y - ref) <= bound)


def test_spmv_unaligned_pointers_take_plain_path(eng, eng_fused, rng):
    p, i, v = P.aniso3d(20)
    n = len(p) - 1
    x = rng.standard_normal(n)
    ref = O.spmv("N", n, n, 1.0, p, i, v, x, 0.0)
    # vals and indx views starting one element into their buffers: not 16-byte aligned
    gv = T(np.concatenate([[0.0], v]))[1:]
    gi = T(np.concatenate([np.zeros(1, np.int32), i]))[1:]
    assert gv.data_ptr() % 16 != 0
    gy = torch.zeros(n, dtype=torch.float64, device=dev)
    E.sparse_gemv(eng, "N", n, n, 1.0, T(p), gi, gv, T(x), 0.0, gy)
    assert np.array_equal(gy.cpu().numpy(), ref)
    # the fused mode takes the same plain path
    gy.zero_()
    E.sparse_gemv(eng_fused, "N", n, n, 1.0, T(p), gi, gv, T(x), 0.0, gy)
    y = gy.cpu().numpy()
    assert np.linalg.norm(y - ref) <= 1e-14 * np.linalg.norm(ref)


@pytest.mark.parametrize("name", ["aniso3d_24", "irregular"])
def test_spmv_n_f32_and_bf16_bit_exact(eng, rng, name):
    p, i, v = CASES[name](rng)
    m = len(p) - 1
    x = rng.standard_normal(m).astype(np.float32)
    v32 = v.astype(np.float32)
    ref = O.spmv("N", m, m, 1.0, p, i, v32, x, 0.0)
    gy = torch.zeros(m, dtype=torch.float32, device=dev)
    E.sparse_gemv(eng, "N", m, m, 1.0, T(p), T(i), T(v32), T(x), 0.0, gy)
    assert np.array_equal(gy.cpu().numpy(), ref)
    vb = O.f32_to_bf16(v32)
    ref = O.spmv_bf16f32("N", m, m, 1.0, p, i, vb, x, 0.0)
    gvb = torch.from_numpy(vb.view(np.int16)).to(dev).view(torch.bfloat16)
    assert np.array_equal(gvb.view(torch.int16).cpu().numpy().view(np.uint16), vb)
    gy.zero_()
    E.sparse_gemv(eng, "N", m, m, 1.0, T(p), T(i), gvb, T(x), 0.0, gy)
    assert np.array_equal(gy.cpu().numpy(), ref)


@pytest.mark.parametrize("name", ["aniso3d_24", "convdiff3d_17", "irregular"])
def test_spmv_t(eng, rng, name):
    p, i, v = CASES[name](rng)
    n = len(p) - 1
    x = rng.standard_normal(n)
    y0 = rng.standard_normal(n)
    ref = O.spmv("T", n, n, 1.5, p, i, v, x, 0.5, y0)
    # matrix object: cached transpose, same accumulation order -> identical bits
    A = E.make_sparse_matrix(eng, n, T(p), T(i), T(v))
    gy = T(y0)
    A.gemv("T", 1.5, T(x), 0.5, gy)
    assert np.array_equal(gy.cpu().numpy(), ref)
    # stateless call: atomic scatter, order not fixed
    gy = T(y0)
    E.sparse_gemv(eng, "T", n, n, 1.5, T(p), T(i), T(v), T(x), 0.5, gy)
    np.testing.assert_allclose(gy.cpu().numpy(), ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())


def test_fused_spmv_dot(eng, rng):
    p, i, v = P.aniso3d(30)
    n = len(p) - 1
    x = rng.standard_normal(n)
    A = E.make_sparse_matrix(eng, n, T(p), T(i), T(v))
    gy = torch.zeros(n, dtype=torch.float64, device=dev)
    d = torch.zeros(1, dtype=torch.float64, device=dev)
    A.gemv_dot(T(x), gy, d)
    y = O.spmv("N", n, n, 1.0, p, i, v, x, 0.0)
    assert np.array_equal(gy.cpu().numpy(), y)
    assert abs(d.item() - x @ y) <= 1e-13 * abs(x @ y)


def test_reference_gemv_goldens(eng):
    c = R.TRIDIAG5
    A = R.dense(c)
    for x in (R.make_vector(-1, 5), R.D(1, 2, 3, 4, 5)):
        for t, M in (("N", A), ("T", A.T), ("C", A.T)):
            gy = torch.zeros(5, dtype=torch.float64, device=dev)
            E.sparse_gemv(eng, t, 5, 5, 2.0, T(c["pntr"]), T(c["indx"]), T(c["vals"]), T(x), 0.0, gy)
            assert R.testvec(gy.cpu().numpy(), 2.0 * M @ x)
    # rectangular 5 x 6 product of test_sparse_matrix (tests/sparse_tests.hpp:139-148)
    pntr = R.I(0, 3, 7, 9, 13, 16)
    indx = R.I(0, 2, 5, 0, 1, 2, 5, 2, 3, 0, 2, 3, 5, 1, 3, 4)
    vals = R.D(2, 4, 5, 1, 3, 1, 5, 4, 1, 3, 4, 4, 1, 5, 1, 3)
    Ad = R.dense(dict(pntr=pntr, indx=indx, vals=vals), 6)
    x = R.make_vector(-1, 6)
    gy = torch.zeros(5, dtype=torch.float64, device=dev)
    E.sparse_gemv(eng, "N", 5, 6, 2.0, T(pntr), T(indx), T(vals), T(x), 0.0, gy)
    assert R.testvec(gy.cpu().numpy(), 2.0 * Ad @ x)
    x5 = R.make_vector(-1, 5)
    gy = torch.zeros(6, dtype=torch.float64, device=dev)
    E.sparse_gemv(eng, "T", 5, 6, 2.0, T(pntr), T(indx), T(vals), T(x5), 0.0, gy)
    assert R.testvec(gy.cpu().numpy(), 2.0 * Ad.T @ x5)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_blas1(eng, rng, dtype):
    n = 1_000_003
    npd = np.float64 if dtype == torch.float64 else np.float32
    tol = 1e-13 if dtype == torch.float64 else 1e-6
    x = rng.standard_normal(n).astype(npd)
    y = rng.standard_normal(n).astype(npd)
    gx, gy = T(x), T(y)
    ref = float(x.astype(np.float64) @ y.astype(np.float64))
    assert abs(E.dot(eng, gx, gy) - ref) <= tol * np.sqrt(n) * abs(ref) + tol
    assert abs(E.norm2(eng, gx) - np.linalg.norm(x.astype(np.float64))) <= tol * np.linalg.norm(x)
    E.axpy(eng, 0.75, gx, gy)
    np.testing.assert_allclose(gy.cpu().numpy(), y + npd(0.75) * x, rtol=tol, atol=tol)
    E.scal(eng, -2.0, gy)
    np.testing.assert_allclose(gy.cpu().numpy(), -2 * (y + npd(0.75) * x), rtol=tol, atol=tol)
    gz = torch.empty_like(gx)
    E.vcopy(eng, gx, gz)
    assert torch.equal(gz, gx)
    E.set_zero(eng, gz)
    assert int(torch.count_nonzero(gz)) == 0
    # empty vectors
    e = torch.empty(0, dtype=dtype, device=dev)
    assert E.dot(eng, e, e) == 0.0


def test_dense_gemv_krylov(eng, rng):
    m, k = 100_000, 23
    W = rng.standard_normal((k, m))        # column-major m x k == row-major k x m
    x = rng.standard_normal(m)
    c = torch.zeros(k, dtype=torch.float64, device=dev)
    E.gemv(eng, "T", m, k, 1.0, T(W), T(x), 0.0, c)
    np.testing.assert_allclose(c.cpu().numpy(), W @ x, rtol=1e-12)
    y = T(x.copy())
    E.gemv(eng, "N", m, k, -1.0, T(W), c, 1.0, y)
    np.testing.assert_allclose(y.cpu().numpy(), x - W.T @ (W @ x), rtol=1e-10, atol=1e-9)


def test_diag_index_and_csr_errors(eng, rng):
    p, i, v = P.aniso3d(8)
    d = E.get_diagonal_index(eng, T(p), T(i))
    assert np.array_equal(d.cpu().numpy(), O.diag_index(p, i))
    # drop the diagonal of row 5: the device check reports a malformed pattern
    keep = np.ones(len(i), bool)
    keep[O.diag_index(p, i)[5]] = False
    p2 = p.copy()
    p2[6:] -= 1
    with pytest.raises(HgbError) as e:
        E.get_diagonal_index(eng, T(p2), T(i[keep]))
    assert e.value.status == HGB_ERR_CSR
    # unsorted columns / out-of-range column: rejected when the matrix object is created
    i_bad = i.copy()
    i_bad[[0, 1]] = i_bad[[1, 0]]
    with pytest.raises(HgbError):
        E.make_sparse_matrix(eng, len(p) - 1, T(p), T(i_bad), T(v))
    i_bad = i.copy()
    i_bad[-1] = len(p) + 5
    with pytest.raises(HgbError):
        E.make_sparse_matrix(eng, len(p) - 1, T(p), T(i_bad), T(v))
    # the context stays usable afterwards
    d = E.get_diagonal_index(eng, T(p), T(i))
    assert np.array_equal(d.cpu().numpy(), O.diag_index(p, i))
