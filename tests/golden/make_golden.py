"""Generates tests/golden/*.npz from the reference's own CPU path (oracle/_ref/libhalaref.so,
built by `make -C oracle/ref` from the unmodified reference headers).

Every output array in a fixture is computed by the reference: diagonal index, ILU(0) factor,
ILU apply, SpMV 'N' and 'T', solve_cg with the ILU preconditioner (solution + iteration count)
and solve_gmres with it; the cplx_* fixtures hold the same for complex128 and complex64 values
(SpMV 'C' too), through the reference's templates instantiated on std::complex.  Inputs are seeded synthetic matrices from hala_gb300.problems.
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


def make_complex(name, p, i, v, seed, hpd):
    """Complex fixture: for complex128 and complex64 (suffix _z / _c) the reference's ILU(0)
    factor and apply, SpMV 'N' / 'T' / 'C' with complex alpha and beta, solve_cg with the ILU
    (Hermitian positive definite matrices only) and solve_gmres(30) with it."""
    assert O.ref() is not None, "build the reference CPU shim first: make -C oracle/ref"
    rng = np.random.default_rng(seed)
    n = len(p) - 1
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    y0 = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    alpha, beta = 0.5 - 0.25j, 1.0 + 0.5j
    d = np.zeros(n, np.int32)
    O.ref().ref_get_diagonal_index(n, p, i, d)
    out = dict(pntr=p, indx=i, vals=v, x=x, y0=y0, alpha=alpha, beta=beta, diag=d, hpd=hpd)
    for s, ct, rt in (("z", np.complex128, np.float64), ("c", np.complex64, np.float32)):
        r, sfx = O.zref(ct)
        vv, xx, yy = v.astype(ct), x.astype(ct), y0.astype(ct)
        ab = lambda z: np.array([z.real, z.imag], rt)  # noqa: E731
        f = np.zeros_like(vv)
        getattr(r, f"ref_factorize_ilu_{sfx}")(n, p.ctypes.data, i.ctypes.data, vv.ctypes.data, f.ctypes.data)
        ap = xx.copy()
        getattr(r, f"ref_apply_ilu_{sfx}")(n, p.ctypes.data, i.ctypes.data, d.ctypes.data, f.ctypes.data,
                                            ap.ctypes.data)
        out[f"ilu_{s}"], out[f"apply_{s}"] = f, ap
        a2, b2 = ab(alpha), ab(beta)
        for t in "NTC":
            y = yy.copy()
            getattr(r, f"ref_sparse_gemv_{sfx}")(t.encode(), n, n, a2.ctypes.data, p.ctypes.data, i.ctypes.data,
                                                  vv.ctypes.data, xx.ctypes.data, b2.ctypes.data, y.ctypes.data)
            out[f"spmv_{t.lower()}_{s}"] = y
        one, zero = ab(1.0 + 0j), ab(0j)
        b = np.zeros(n, ct)
        getattr(r, f"ref_sparse_gemv_{sfx}")(b"N", n, n, one.ctypes.data, p.ctypes.data, i.ctypes.data,
                                              vv.ctypes.data, xx.ctypes.data, zero.ctypes.data, b.ctypes.data)
        bn = float(np.linalg.norm(b.astype(np.complex128)))
        out[f"b_{s}"] = b
        tol = (1e-10 if s == "z" else 1e-4) * bn
        if hpd:
            cx = np.zeros(n, ct)
            it = getattr(r, f"ref_solve_cg_{sfx}")(n, p.ctypes.data, i.ctypes.data, vv.ctypes.data, d.ctypes.data,
                                                   f.ctypes.data, b.ctypes.data, cx.ctypes.data, tol, 2000)
            out[f"cg_x_{s}"], out[f"cg_iters_{s}"], out[f"cg_tol_{s}"] = cx, it, tol
        gx = np.zeros(n, ct)
        it = getattr(r, f"ref_solve_gmres_{sfx}")(n, p.ctypes.data, i.ctypes.data, vv.ctypes.data, d.ctypes.data,
                                                  f.ctypes.data, 30, b.ctypes.data, gx.ctypes.data, tol, 200)
        out[f"gmres_x_{s}"], out[f"gmres_iters_{s}"], out[f"gmres_tol_{s}"] = gx, it, tol
        print(name, s, n, len(i), "cg", out.get(f"cg_iters_{s}"), "gmres", it, flush=True)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **out)


if __name__ == "__main__":
    make("aniso3d_10x9x8", *P.aniso3d(10, 9, 8), seed=1, spd=True)
    make("poisson2d_24", *P.poisson2d(24), seed=2, spd=True)
    make("convdiff3d_8", *P.convdiff3d(8), seed=3, spd=False)
    make("random_200", *P.random_csr(200, 0.03, np.random.default_rng(7)), seed=4, spd=False)
    make_complex("cplx_magnetic2d_12", *P.magnetic2d(12), seed=5, hpd=True)
    make_complex("cplx_helmholtz_convdiff3d_6", *P.helmholtz_shift(*P.convdiff3d(6)), seed=6, hpd=False)
