"""split_pattern / split_values on the device, through the C ABI, BIT-EXACTLY against the oracle
(itself pinned to the reference build) and the reference's own test_split_matrix case
(tests/sparse_tests.hpp:368-421)."""
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


def test_split_reference_case(eng):
    c = R.SPLIT6
    d = E.get_diagonal_index(eng, T(c["pntr"]), T(c["indx"]))
    assert np.array_equal(d.cpu().numpy(), c["diag"])
    up, ui, lp, li = E.split_pattern(eng, T(c["pntr"]), T(c["indx"]), d)
    for got, ref in ((up, "up"), (ui, "ui"), (lp, "lp"), (li, "li")):
        assert np.array_equal(got.cpu().numpy(), c[ref]), ref
    uv, lv = E.split_values(eng, "U", "N", T(c["pntr"]), T(c["vals"]), up, lp)
    assert np.array_equal(uv.cpu().numpy(), c["uv"]) and np.array_equal(lv.cpu().numpy(), c["lv"])


@pytest.mark.parametrize("name", ["aniso3d", "convdiff3d", "random", "one_row"])
@pytest.mark.parametrize("uplo,diag", [("U", "N"), ("L", "N"), ("U", "U"), ("L", "U")])
def test_split_matches_oracle(eng, rng, name, uplo, diag):
    if name == "aniso3d":
        p, i, v = P.aniso3d(13, 11, 9)
    elif name == "convdiff3d":
        p, i, v = P.convdiff3d(10)
    elif name == "random":
        p, i, v = P.random_csr_sparse(3000, 9, rng)
    else:
        p, i, v = np.array([0, 1], np.int32), np.array([0], np.int32), np.array([3.0])
    d = O.diag_index(p, i)
    up, ui, lp, li = O.split_pattern(p, i, d)
    uv, lv = O.split_values(uplo, diag, p, v, up, lp)
    gup, gui, glp, gli = E.split_pattern(eng, T(p), T(i), T(d))
    for got, ref in ((gup, up), (gui, ui), (glp, lp), (gli, li)):
        assert np.array_equal(got.cpu().numpy(), ref)
    for dt in (torch.float64, torch.float32):
        guv, glv = E.split_values(eng, uplo, diag, T(p), T(v).to(dt), gup, glp)
        ruv, rlv = O.split_values(uplo, diag, p, v.astype(np.float32), up, lp) if dt == torch.float32 else (uv, lv)
        assert np.array_equal(guv.cpu().numpy(), ruv) and np.array_equal(glv.cpu().numpy(), rlv)


def test_split_rejects_diagonal_outside_its_row(eng):
    p, i, v = P.aniso3d(6)
    d = O.diag_index(p, i).copy()
    d[5] = p[6]          # points into the next row
    with pytest.raises(HgbError) as e:
        E.split_pattern(eng, T(p), T(i), T(d))
    assert e.value.status == HGB_ERR_CSR
