"""ILU(0) factorisation, level sets, ILU apply and triangular solves on the GPU vs the oracle.

The FP64 factor, the level sets and the FP64 / FP32 applies are compared BIT-EXACTLY (same
per-entry operation order, no fused multiply-add), and so is the FP32 store with FP64 pivots
against the oracle's mixed apply; the BF16 store within 2e-2 of the FP64 apply."""
import glob
import os

import numpy as np
import pytest
import torch

from hala_gb300 import engine as E
from hala_gb300 import problems as P
from hala_gb300.hgb import HgbError, HGB_ERR_CSR, HGB_ERR_TIMEOUT
from hala_gb300 import hgb as H
from oracle import oracle as O
from tests import refcases as R

pytestmark = pytest.mark.gpu
dev = torch.device("cuda")
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def T(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


MATS = {
    "aniso3d_20": lambda rng: P.aniso3d(20, 19, 18),
    "poisson2d_70": lambda rng: P.poisson2d(70, 33),
    "convdiff3d_14": lambda rng: P.convdiff3d(14),
    "random_400": lambda rng: P.random_csr(400, 0.02, rng),
    "ilu3": lambda rng: (R.ILU3["pntr"], R.ILU3["indx"], R.ILU3["vals"]),
    # several solve blocks: cross-block dependencies at block cuts that split planes / grid rows
    "aniso3d_34": lambda rng: P.aniso3d(34, 33, 32),
    "poisson2d_300": lambda rng: P.poisson2d(300, 200),
    # a chain (one row per level): blocks end at the step limit, many blocks in sequence
    "chain_40000": lambda rng: P.poisson2d(40000, 1),
    # rows with more than three dependencies in each triangle, several blocks
    "random_40000": lambda rng: P.random_csr_sparse(40000, 10, rng),
    # one level of 16384+ rows per block, every row depending on the block before (long levels)
    "shift_50000": lambda rng: shifted_diagonals(50000, 16384),
}


def shifted_diagonals(n, off):
    """Diagonal plus the two diagonals at distance off: row i couples to i - off and i + off."""
    rows, cols = [], []
    for o in (-off, 0, off):
        i = np.arange(max(0, -o), min(n, n - o))
        rows.append(i)
        cols.append(i + o)
    r, c = np.concatenate(rows), np.concatenate(cols)
    order = np.lexsort((c, r))
    r, c = r[order], c[order]
    v = np.where(r == c, 4.0, -1.0)
    p = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(r, minlength=n), out=p[1:])
    return p.astype(np.int32), c.astype(np.int32), v


@pytest.mark.parametrize("name", list(MATS))
def test_factor_levels_apply_bit_exact(eng, rng, name):
    p, i, v = MATS[name](rng)
    n = len(p) - 1
    fo, do, st = O.ilu_factor(p, i, v)
    ilu = E.make_ilu(eng, T(p), T(i), T(v))
    f, d = ilu.factor()
    assert np.array_equal(d.cpu().numpy(), do)
    assert np.array_equal(f.cpu().numpy().view(np.uint64), fo.view(np.uint64))
    for uplo in "LU":
        lev, nl = ilu.levels(uplo)
        lo, nlo = O.levels(p, i, do, uplo)
        assert nl == nlo and np.array_equal(lev.cpu().numpy(), lo)
    for _ in range(3):       # repeated applies reuse the pending-state buffers
        x = rng.standard_normal(n)
        r = ilu.apply(T(x))
        assert np.array_equal(r.cpu().numpy(), O.ilu_apply(p, i, do, fo, x))
        rt = ilu.apply(T(x), trans="T")
        assert np.array_equal(rt.cpu().numpy(), O.ilu_apply(p, i, do, fo, x, trans="T"))
    # in place
    gx = T(x)
    ilu.apply(gx, gx)
    assert np.array_equal(gx.cpu().numpy(), O.ilu_apply(p, i, do, fo, x))


def test_reference_ilu_golden(eng):
    c = R.ILU3
    ilu = E.make_ilu(eng, T(c["pntr"]), T(c["indx"]), T(c["vals"]))
    f, d = ilu.factor()
    assert np.array_equal(d.cpu().numpy(), c["diag"])
    assert R.testvec(f.cpu().numpy(), c["ilu"])
    assert R.testvec(ilu.apply(T(c["x"])).cpu().numpy(), c["apply"])


@pytest.mark.parametrize("path", sorted(f for f in glob.glob(os.path.join(GOLDEN, "*.npz"))
                                        if not os.path.basename(f).startswith("cplx_")))
def test_gpu_matches_reference_fixture(eng, path):
    g = np.load(path)
    p, i, v = g["pntr"], g["indx"], g["vals"]
    n = len(p) - 1
    ilu = E.make_ilu(eng, T(p), T(i), T(v))
    f, d = ilu.factor()
    assert np.array_equal(d.cpu().numpy(), g["diag"])
    assert np.array_equal(f.cpu().numpy().view(np.uint64), g["ilu"].view(np.uint64))
    assert np.array_equal(ilu.apply(T(g["x"])).cpu().numpy(), g["apply"])
    y = torch.zeros(n, dtype=torch.float64, device=dev)
    E.sparse_gemv(eng, "N", n, n, 1.0, T(p), T(i), T(v), T(g["x"]), 0.0, y)
    assert np.array_equal(y.cpu().numpy(), g["spmv_n"])
    A = E.make_sparse_matrix(eng, n, T(p), T(i), T(v))
    y.zero_()
    A.gemv("T", 1.0, T(g["x"]), 0.0, y)
    assert np.array_equal(y.cpu().numpy(), g["spmv_t"])


def test_f32_factor_and_apply_bit_exact(eng, rng):
    p, i, v = P.aniso3d(16)
    n = len(p) - 1
    v32 = v.astype(np.float32)
    fo, do, _ = O.ilu_factor(p, i, v32)
    ilu = E.make_ilu(eng, T(p), T(i), T(v32))
    f, _ = ilu.factor()
    assert np.array_equal(f.cpu().numpy().view(np.uint32), fo.view(np.uint32))
    x = rng.standard_normal(n).astype(np.float32)
    assert np.array_equal(ilu.apply(T(x)).cpu().numpy(), O.ilu_apply(p, i, do, fo, x))


@pytest.mark.parametrize("mat", ["aniso3d_18", "aniso3d_44", "shift_80000"])
@pytest.mark.parametrize("store", [torch.float32, torch.bfloat16])
def test_mixed_store_apply(eng, rng, store, mat):
    # aniso3d_44 and shift_80000 span several 32768-row solve blocks of the FP32 store
    p, i, v = {"aniso3d_18": lambda: P.aniso3d(18), "aniso3d_44": lambda: P.aniso3d(44),
               "shift_80000": lambda: shifted_diagonals(80000, 20000)}[mat]()
    n = len(p) - 1
    fo, do, _ = O.ilu_factor(p, i, v)
    ilu = E.make_ilu(eng, T(p), T(i), T(v), store=store)
    x = rng.standard_normal(n).astype(np.float32)
    r = ilu.apply(T(x)).cpu().numpy().astype(np.float64)
    ref = O.ilu_apply(p, i, do, fo, x.astype(np.float64))
    tol = 1e-5 if store == torch.float32 else 2e-2
    assert np.linalg.norm(r - ref) <= tol * np.linalg.norm(ref)
    if store == torch.float32:
        # FP32 sweeps in the reference's order, pivots as FP32 reciprocals of the FP64 pivots
        exact = O.ilu_apply_mixed(p, i, do, fo.astype(np.float32), fo[do], x)
        assert np.array_equal(ilu.apply(T(x)).cpu().numpy().view(np.uint32), exact.view(np.uint32))


def test_triangular_goldens(eng):
    X = R.TRSV_X
    L, U = R.TRSV_L, R.TRSV_U
    cases = [(L, L["vals"], "L", "N", "N", R.TRSV_A), (L, L["vals"], "L", "N", "T", R.TRSV_A.T),
             (L, R.TRSV_LU_VALS, "L", "U", "N", R.TRSV_AU), (U, U["vals"], "U", "N", "N", R.TRSV_A.T),
             (U, U["vals"], "U", "N", "T", R.TRSV_A)]
    for c, vals, uplo, diagc, trans, M in cases:
        tri = E.make_triangular_matrix(eng, uplo, diagc, T(c["pntr"]), T(c["indx"]), T(vals))
        x = torch.zeros(3, dtype=torch.float64, device=dev)
        E.sparse_trsv(trans, tri, 0.5, T(2.0 * M @ X), x)
        assert R.testvec(x.cpu().numpy(), X), (uplo, diagc, trans)


def test_triangular_bit_exact(eng, rng):
    p, i, v = P.random_csr(300, 0.03, rng)
    d = O.diag_index(p, i)
    up, ui, lp, li = O.split_pattern(p, i, d)
    uv, lv = O.split_values("U", "N", p, v, up, lp)
    lv = lv.copy()
    lv[lp[1:] - 1] = 1.0 + np.abs(rng.standard_normal(len(p) - 1))
    n = len(p) - 1
    b = rng.standard_normal(n)
    for tp, ti, tv, uplo in ((lp, li, lv, "L"), (up, ui, uv, "U")):
        for diagc in "NU":
            tri = E.make_triangular_matrix(eng, uplo, diagc, T(tp), T(ti), T(tv))
            for trans in "NT":
                x = torch.zeros(n, dtype=torch.float64, device=dev)
                E.sparse_trsv(trans, tri, 0.5, T(b), x)
                ref = O.trsv(uplo, diagc, trans, 0.5, tp, ti, tv, b)
                assert np.array_equal(x.cpu().numpy(), ref), (uplo, diagc, trans)
    # b and x the same buffer
    tri = E.make_triangular_matrix(eng, "L", "N", T(lp), T(li), T(lv))
    gb = T(b)
    E.sparse_trsv("N", tri, 1.0, gb, gb)
    assert np.array_equal(gb.cpu().numpy(), O.trsv("L", "N", "N", 1.0, lp, li, lv, b))


def test_zero_pivot_is_reported(eng):
    # a_11 - l*a_01 = 0 exactly: [[1,1],[1,1]] has a zero second pivot
    p, i, v = R.I(0, 2, 4), R.I(0, 1, 0, 1), R.D(1, 1, 1, 1)
    ilu = E.make_ilu(eng, T(p), T(i), T(v))
    assert ilu.zero_pivot
    f, _ = ilu.factor()
    fo, _, st = O.ilu_factor(p, i, v)
    assert st != 0 and np.array_equal(f.cpu().numpy(), fo)


def test_bounded_wait_times_out_and_context_survives(eng, rng):
    st = H.lib().hgb_selftest_wait_timeout(eng.h, 1000)
    assert st == HGB_ERR_TIMEOUT
    with pytest.raises(HgbError):
        H.check(st)
    p, i, v = P.aniso3d(10)
    ilu = E.make_ilu(eng, T(p), T(i), T(v))
    fo, do, _ = O.ilu_factor(p, i, v)
    x = rng.standard_normal(len(p) - 1)
    assert np.array_equal(ilu.apply(T(x)).cpu().numpy(), O.ilu_apply(p, i, do, fo, x))


def test_apply_bit_exact_at_bench_size(eng, rng):
    # the 128^3 workload: 128 one-plane blocks in clusters of 8 (more than are co-resident), both
    # sweeps, 'N' and 'T', against the oracle bit for bit
    p, i, v = P.aniso3d(128)
    n = len(p) - 1
    fo, do, _ = O.ilu_factor(p, i, v)
    x = rng.standard_normal(n)
    ilu = E.make_ilu(eng, T(p), T(i), T(v))
    assert np.array_equal(ilu.apply(T(x)).cpu().numpy(), O.ilu_apply(p, i, do, fo, x))
    assert np.array_equal(ilu.apply(T(x), trans="T").cpu().numpy(), O.ilu_apply(p, i, do, fo, x, trans="T"))
    ilu32 = E.make_ilu(eng, T(p), T(i), T(v), store=torch.float32)
    x32 = x.astype(np.float32)
    exact = O.ilu_apply_mixed(p, i, do, fo.astype(np.float32), fo[do], x32)
    for _ in range(2):
        assert np.array_equal(ilu32.apply(T(x32)).cpu().numpy().view(np.uint32), exact.view(np.uint32))


@pytest.mark.parametrize("store", [torch.float64, torch.float32])
def test_host_buffer_ilu_matches_device_ilu(eng, rng, store):
    # make_ilu(mixed_engine, ...): host pattern and values, copies overlapped with the host planning;
    # the factor, the level sets and the apply are those of the device-input creation, bit for bit
    p, i, v = P.aniso3d(41, 37, 23)
    n = len(p) - 1
    Md = E.make_ilu(eng, T(p), T(i), T(v), store=store)
    Mh = E.make_ilu_host(eng, p, i, v, store=store)
    fd, dd = Md.factor()
    fh, dh = Mh.factor()
    assert torch.equal(fd, fh) and torch.equal(dd, dh)
    x = torch.from_numpy(rng.standard_normal(n)).to(dev).to(store)
    rd, rh = torch.empty_like(x), torch.empty_like(x)
    Md.apply(x, rd)
    Mh.apply(x, rh)
    assert torch.equal(rd, rh)
    fo, do, _ = O.ilu_factor(p, i, v)
    assert np.array_equal(fh.cpu().numpy(), fo)


def test_host_buffer_ilu_rejects_bad_pattern(eng):
    p, i, v = P.aniso3d(6)
    i = i.copy()
    i[p[3]:p[4]] = i[p[3]:p[4]][::-1]   # unsorted row
    with pytest.raises(HgbError) as e:
        E.make_ilu_host(eng, p, i, v)
    assert e.value.status == HGB_ERR_CSR
    i[p[3]:p[4]] = np.sort(i[p[3]:p[4]])
    keep = np.ones(len(i), bool)
    keep[int(O.diag_index(p, i)[5])] = False   # drop the diagonal of row 5
    p2 = p.copy()
    p2[6:] -= 1
    with pytest.raises(HgbError) as e:
        E.make_ilu_host(eng, p2, i[keep], v[keep])
    assert e.value.status == HGB_ERR_CSR
