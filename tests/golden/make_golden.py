"""Generates tests/golden/*.npz from the reference's own CPU path (oracle/_ref/libhalaref.so,
built by `make -C oracle/ref` from the unmodified reference headers).

Every output array in a fixture is computed by the reference: diagonal index, ILU(0) factor,
ILU apply, SpMV 'N' and 'T', solve_cg with the ILU preconditioner (solution + iteration count)
and solve_gmres with it.  Inputs are seeded synthetic matrices from hala_gb300.problems.
Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from hala_gb300 import problems as P  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def make(name, p, i, v, seed, spd):
    ref = O.ref()
    assert ref is not None, "build the reference CPU shim first: make -C oracle/ref"
    rng = np.random.default_rng(seed)
    n = len(p) - 1
    x = rng.standard_normal(n)
    d = np.zeros(n, np.int32)
    ref.ref_get_diagonal_index(n, p, i, d)
    f = np.zeros_like(v)
    ref.ref_factorize_ilu_d(n, p, i, v, f)
    ap = x.copy()
    ref.ref_apply_ilu_d(n, p, i, d, f, ap)
    yn = np.zeros(n)
    ref.ref_sparse_gemv_d(b"N", n, n, 1.0, p, i, v, x, 0.0, yn)
    yt = np.zeros(n)
    ref.ref_sparse_gemv_d(b"T", n, n, 1.0, p, i, v, x, 0.0, yt)
    b = yn.copy()
    cg_tol = 1e-10 * np.linalg.norm(b)
    cg_x = np.zeros(n)
    # CG only where the matrix is symmetric positive definite; capped either way
    cg_it = ref.ref_solve_cg_d(n, p, i, v, d.ctypes.data, f.ctypes.data, b, cg_x, cg_tol, 2000 if spd else 50)
    g_tol = 1e-9 * np.linalg.norm(b)
    g_x = np.zeros(n)
    g_it = ref.ref_solve_gmres_d(n, p, i, v, d.ctypes.data, f.ctypes.data, 30, b, g_x, g_tol, 200)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), pntr=p, indx=i, vals=v, x=x, diag=d, ilu=f,
                        apply=ap, spmv_n=yn, spmv_t=yt, b=b, cg_tol=cg_tol, cg_x=cg_x, cg_iters=cg_it,
                        gmres_tol=g_tol, gmres_restart=30, gmres_x=g_x, gmres_iters=g_it,
                        cg_max_iter=2000 if spd else 50, gmres_max_iter=200)
    print(name, n, len(i), "cg", cg_it, "gmres", g_it, flush=True)


if __name__ == "__main__":
    make("aniso3d_10x9x8", *P.aniso3d(10, 9, 8), seed=1, spd=True)
    make("poisson2d_24", *P.poisson2d(24), seed=2, spd=True)
    make("convdiff3d_8", *P.convdiff3d(8), seed=3, spd=False)
    make("random_200", *P.random_csr(200, 0.03, np.random.default_rng(7)), seed=4, spd=False)
