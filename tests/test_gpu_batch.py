"""Batched independent systems on the GPU vs a per-system loop of the oracle's solve_cg
(the reference has no independent-systems batch; its solve_cg per system is the oracle)."""
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


def make(S, nmin, nmax, seed):
    sp, p, i, v = P.er_laplacian_batch(S, nmin, nmax, seed=seed)
    b = np.random.default_rng(seed + 100).uniform(-1, 1, len(p) - 1)
    return sp, p, i, v, b


@pytest.mark.parametrize("cfg", [(256, 256), (128, 0), (512, 128)])
def test_batch_matches_per_system_oracle(eng, cfg):
    sp, p, i, v, b = make(96, 16, 1500, seed=5)
    B = E.gpu_batch(eng, T(sp), T(p), T(i), T(v))
    B.set_config(*cfg)
    x = torch.zeros(len(b), dtype=torch.float64, device=dev)
    iters = torch.zeros(96, dtype=torch.int32, device=dev)
    rel = torch.zeros(96, dtype=torch.float64, device=dev)
    B.solve(T(b), x, rtol=1e-8, iters=iters, relres=rel)
    xs = x.cpu().numpy()
    v64 = v.astype(np.float64)     # the system is the FP32-stored matrix
    for s in range(96):
        r0, r1 = sp[s], sp[s + 1]
        ps = (p[r0:r1 + 1] - p[r0]).astype(np.int32)
        iS = (i[p[r0]:p[r1]] - r0).astype(np.int32)
        vS = v64[p[r0]:p[r1]]
        bs = b[r0:r1]
        res = np.linalg.norm(bs - P.csr_matvec(ps, iS, vS, xs[r0:r1]))
        assert res <= 1e-8 * np.linalg.norm(bs) * 1.0001, s
        xo, _, _ = O.cg(ps, iS, vS, bs, tol=1e-12 * np.linalg.norm(bs), max_iter=20000)
        assert np.linalg.norm(xs[r0:r1] - xo) <= 1e-6 * np.linalg.norm(xo), s
    assert np.all(rel.cpu().numpy() <= 1e-8)
    assert np.all(iters.cpu().numpy() > 0)


def test_batch_replay_and_autotune(eng, tmp_path):
    sp, p, i, v, b = make(200, 32, 2000, seed=6)
    B = E.gpu_batch(eng, T(sp), T(p), T(i), T(v))
    gb = T(b)
    x = torch.zeros(len(b), dtype=torch.float64, device=dev)
    cache = str(tmp_path / "batch_tune.txt")
    best = B.autotune(gb, x, 1e-8, cache)
    assert B.config == best
    # a second autotune of the same batch shape comes from the cache
    assert B.autotune(gb, x, 1e-8, cache) == best
    for _ in range(2):            # graph replay with the same vectors
        x.zero_()
        B.solve(gb, x, rtol=1e-8)
        r = b - P.csr_matvec(p, i, v.astype(np.float64), x.cpu().numpy())
        for s in range(0, 200, 17):
            r0, r1 = sp[s], sp[s + 1]
            assert np.linalg.norm(r[r0:r1]) <= 1e-8 * np.linalg.norm(b[r0:r1]) * 1.0001


def test_batch_rejects_coupled_systems(eng):
    sp, p, i, v, b = make(4, 16, 32, seed=7)
    i2 = i.copy()
    i2[0] = len(b) - 1        # row 0 of system 0 pointing into the last system
    order = np.argsort(i2[p[0]:p[1]], kind="stable")
    i2[p[0]:p[1]] = i2[p[0]:p[1]][order]
    v2 = v.copy()
    v2[p[0]:p[1]] = v2[p[0]:p[1]][order]
    with pytest.raises(HgbError):
        E.gpu_batch(eng, T(sp), T(p), T(i2), T(v2))
