"""Golden cases written out from the reference's own tests (inputs and expected outputs as data).

tests/sparse_tests.hpp: test_ilu (:423-440), test_split_matrix (:368-421), test_sparse_trsv
(:259-311), test_sparse_gemv (:165-191); tests/solvers_tests.hpp: test_cg (:13-55),
test_gmres (:106-137); tests/cuda_sparse_tests.hpp: sparse_matvec (:12-30).
make_vector(N) after hala_rnd = s yields s+1, s+2, ... (tests/testing_common.hpp:50-61).
The reference checks doubles with sum|x - ref| / correction < 1e-14 (testing_common.hpp:288-308).
"""
import numpy as np

I = lambda *v: np.array(v, np.int32)   # noqa: E731
D = lambda *v: np.array(v, np.float64)  # noqa: E731


def make_vector(start, n):
    return np.arange(start + 1, start + 1 + n, dtype=np.float64)


def testvec(x, y, correction=1.0, tol=1e-14):
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    return x.shape == y.shape and np.all(np.isfinite(x)) and np.abs(x - y).sum() / correction < tol


ILU3 = dict(pntr=I(0, 3, 6, 9), indx=I(0, 1, 2, 0, 1, 2, 0, 1, 2), vals=D(3, 2, 1, 2, 4, 3, 2, 1, 6),
            diag=I(0, 4, 8), ilu=D(3, 2, 1, 2 / 3, 8 / 3, 7 / 3, 2 / 3, -0.125, 5.625),
            x=D(1, 2, 3), apply=D(1 / 9, 1 / 9, 4 / 9))

_a, _d, _z = 1.0, 2.0, 0.0
SPLIT6 = dict(pntr=I(0, 2, 5, 8, 11, 13, 17), indx=I(0, 3, 0, 1, 4, 2, 3, 4, 0, 3, 4, 2, 4, 0, 1, 3, 5),
              vals=D(_d, _a, _a, _d, _a, _d, _a, _a, _a, _d, _a, _a, _d, _a, _a, _a, _d),
              diag=I(0, 3, 5, 9, 12, 16),
              up=I(0, 2, 4, 7, 9, 10, 11), ui=I(0, 3, 1, 4, 2, 3, 4, 3, 4, 4, 5),
              lp=I(0, 1, 3, 4, 6, 8, 12), li=I(0, 0, 1, 2, 0, 3, 2, 4, 0, 1, 3, 5),
              uv=D(_d, _a, _d, _a, _d, _a, _a, _d, _a, _d, _d),
              lv=D(_z, _a, _z, _z, _a, _z, _a, _z, _a, _a, _a, _z))

# 3x3 triangular systems; A is the dense lower matrix [[1,0,0],[4,2,0],[5,0,3]]
TRSV_A = np.array([[1, 0, 0], [4, 2, 0], [5, 0, 3]], np.float64)
TRSV_AU = np.array([[1, 0, 0], [1, 1, 0], [2, 0, 1]], np.float64)
TRSV_X = make_vector(-4, 3)
TRSV_L = dict(pntr=I(0, 1, 3, 5), indx=I(0, 0, 1, 0, 2), vals=D(1, 4, 2, 5, 3))
TRSV_LU_VALS = D(2, 1, 3, 2, 4)      # unit-diagonal case: diagonal values ignored
TRSV_U = dict(pntr=I(0, 3, 4, 5), indx=I(0, 1, 2, 1, 2), vals=D(1, 4, 5, 2, 3))

TRIDIAG5 = dict(pntr=I(0, 2, 5, 8, 11, 13), indx=I(0, 1, 0, 1, 2, 1, 2, 3, 2, 3, 4, 3, 4),
                vals=D(2, 1, 1, 2, 1, 1, 2, 1, 1, 2, 1, 1, 2))
CYCLIC5 = dict(pntr=I(0, 3, 6, 9, 12, 15), indx=I(0, 1, 4, 0, 1, 2, 1, 2, 3, 2, 3, 4, 0, 3, 4),
               vals=D(2, 1, 1, 1, 2, 1, 1, 2, 1, 1, 2, 1, 1, 1, 2))
NONSYM5 = dict(pntr=I(0, 2, 5, 8, 11, 12), indx=I(0, 1, 0, 1, 3, 1, 2, 3, 0, 2, 3, 4),
               vals=D(2, 1, 1, 3, 1, 1, 4, 1, 1, 1, 5, 2))
XREF5 = D(1, 2, 3, 4, 5)
CG_X0 = D(1, 3, -4, -7, 11)


def dense(c, n=None):
    n = len(c["pntr"]) - 1 if n is None else n
    A = np.zeros((len(c["pntr"]) - 1, n))
    for r in range(len(c["pntr"]) - 1):
        for p in range(c["pntr"][r], c["pntr"][r + 1]):
            A[r, c["indx"][p]] = c["vals"][p]
    return A
