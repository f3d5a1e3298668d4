"""Seeded synthetic sparse systems for the solver workloads (CSR, int32 indices, sorted columns).

All matrices are generated here; no dataset is involved.  Rows are in natural (lexicographic)
order with the first grid axis fastest, and every row holds its diagonal, as the reference's ILU
requires (sparse/hala_sparse_core.hpp:45-60).

* ``poisson2d``      2D 5-point Dirichlet Laplacian, diagonal 4, off-diagonals -1.
* ``aniso3d``        3D 7-point operator with axis coefficients (cx, cy, cz); diagonal 2(cx+cy+cz).
* ``convdiff3d``     3D 7-point diffusion plus first-order upwind convection; the cell Peclet
                     number is Pe = max|v| h / D, so the upwind weight on axis a is Pe*v_a/max|v|
                     after scaling the row by h^2/D.
* ``vardiff2d``      2D finite-volume -div(k grad u) with face conductivity the harmonic mean of
                     the two cells; a Dirichlet boundary face uses 2*k_cell (half-cell distance).
* ``er_laplacian_batch``  independent Erdos-Renyi graph Laplacians + shift*I, block-diagonal CSR.
* ``grf2d``          Gaussian random field with squared-exponential covariance (FFT sampling).
* ``magnetic2d``     complex Hermitian positive definite: the 2D 5-point Laplacian with a phase on
                     every edge (a_ij = -exp(i theta_ij), theta_ji = -theta_ij, the discrete magnetic
                     Laplacian) plus shift*I.
* ``helmholtz_shift`` complex non-Hermitian: a real operator plus (sigma_re + i sigma_im) I.
"""
from __future__ import annotations

import numpy as np


def _stencil_csr(shape, offsets):
    """Assemble a CSR matrix from a structured-grid stencil.

    ``offsets`` is a list of (axis_shift tuple, value array or scalar) in ascending column order;
    value arrays are per-row (length n).  Entries falling outside the grid are dropped."""
    shape = tuple(int(s) for s in shape)
    n = int(np.prod(shape))
    # linear index = i0 + s0*(i1 + s1*(i2 ...)) (axis 0 fastest)
    strides = [1]
    for s in shape[:-1]:
        strides.append(strides[-1] * s)
    coords = np.indices(shape[::-1]).reshape(len(shape), -1)[::-1]  # axis-0 fastest ordering
    cols, vals, valid = [], [], []
    rows = np.arange(n, dtype=np.int64)
    for shift, v in offsets:
        ok = np.ones(n, bool)
        off = 0
        for ax, d in enumerate(shift):
            if d:
                c = coords[ax] + d
                ok &= (c >= 0) & (c < shape[ax])
                off += d * strides[ax]
        cols.append(rows + off)
        vals.append(np.broadcast_to(np.asarray(v, np.float64), (n,)))
        valid.append(ok)
    cols = np.stack(cols, 1)
    vals = np.stack(vals, 1)
    valid = np.stack(valid, 1)
    counts = valid.sum(1)
    pntr = np.zeros(n + 1, np.int64)
    np.cumsum(counts, out=pntr[1:])
    indx = cols[valid].astype(np.int32)
    v = vals[valid].astype(np.float64)
    return pntr.astype(np.int32), indx, v


def _axis_shift(ndim, ax, d):
    s = [0] * ndim
    s[ax] = d
    return tuple(s)


def poisson2d(nx, ny=None):
    ny = nx if ny is None else ny
    offs = [((0, -1), -1.0), ((-1, 0), -1.0), ((0, 0), 4.0), ((1, 0), -1.0), ((0, 1), -1.0)]
    return _stencil_csr((nx, ny), offs)


def aniso3d(nx, ny=None, nz=None, coef=(1.0, 1.0, 0.01)):
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    cx, cy, cz = coef
    offs = [((0, 0, -1), -cz), ((0, -1, 0), -cy), ((-1, 0, 0), -cx), ((0, 0, 0), 2.0 * (cx + cy + cz)),
            ((1, 0, 0), -cx), ((0, 1, 0), -cy), ((0, 0, 1), -cz)]
    return _stencil_csr((nx, ny, nz), offs)


def convdiff3d(n, velocity=(1.0, 0.5, 0.25), peclet=10.0):
    vmax = max(abs(v) for v in velocity)
    P = [peclet * v / vmax for v in velocity]       # upwind weights after the h^2/D scaling
    offs = []
    # ascending column order: -z, -y, -x, 0, +x, +y, +z
    for ax in (2, 1, 0):
        up = P[ax] if velocity[ax] > 0 else 0.0
        offs.append((_axis_shift(3, ax, -1), -1.0 - up))
    offs.append(((0, 0, 0), 6.0 + sum(abs(p) for p in P)))
    for ax in (0, 1, 2):
        up = -P[ax] if velocity[ax] < 0 else 0.0
        offs.append((_axis_shift(3, ax, 1), -1.0 - up))
    return _stencil_csr((n, n, n), offs)


def grf2d(n, length=16.0, sigma=1.0, seed=1):
    """Stationary Gaussian random field on an n x n periodic grid with covariance
    sigma^2 exp(-r^2 / (2 length^2)), sampled by spectral (FFT) synthesis."""
    rng = np.random.default_rng(seed)
    k = np.fft.fftfreq(n) * n
    kx, ky = np.meshgrid(k, k, indexing="ij")
    # spectral density of the squared-exponential kernel on the discrete torus
    spec = (2 * np.pi * length ** 2) * np.exp(-2 * np.pi ** 2 * length ** 2 * (kx ** 2 + ky ** 2) / n ** 2)
    noise = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    field = np.fft.ifft2(noise * np.sqrt(spec)).real * n
    field *= sigma / field.std()
    return field.T.reshape(-1).astype(np.float64)    # axis-0 (x) fastest


def vardiff2d_faces(n, kcell):
    """Face conductivities (harmonic mean) for an n x n cell grid, x fastest.
    Returns kx (n+1, n) over x-faces and ky (n, n+1) over y-faces, as [y][x] arrays, with the
    boundary faces set to 2*k_cell (Dirichlet at half-cell distance)."""
    k = kcell.reshape(n, n)                         # [y][x]
    kx = np.empty((n, n + 1))
    kx[:, 1:-1] = 2 * k[:, :-1] * k[:, 1:] / (k[:, :-1] + k[:, 1:])
    kx[:, 0] = 2 * k[:, 0]
    kx[:, -1] = 2 * k[:, -1]
    ky = np.empty((n + 1, n))
    ky[1:-1, :] = 2 * k[:-1, :] * k[1:, :] / (k[:-1, :] + k[1:, :])
    ky[0, :] = 2 * k[0, :]
    ky[-1, :] = 2 * k[-1, :]
    return kx, ky


def vardiff2d(n, kcell):
    """5-point finite-volume -div(k grad u) on n x n unit cells (h = 1)."""
    kx, ky = vardiff2d_faces(n, kcell)
    return vardiff2d_from_faces(n, kx, ky)


def vardiff2d_from_faces(n, kx, ky):
    """The 5-point operator's CSR for given face conductivities kx (n, n+1) and ky (n+1, n),
    [y][x] arrays.  Linear in the faces, so face changes give the operator's change."""
    west = kx[:, :-1].reshape(-1)
    east = kx[:, 1:].reshape(-1)
    south = ky[:-1, :].reshape(-1)
    north = ky[1:, :].reshape(-1)
    diag = west + east + south + north
    offs = [((0, -1), -south), ((-1, 0), -west), ((0, 0), diag), ((1, 0), -east), ((0, 1), -north)]
    return _stencil_csr((n, n), offs)


def er_laplacian(n, rng, mean_degree=8.0, wlo=0.1, whi=1.0, shift=0.01):
    """Weighted Erdos-Renyi graph Laplacian + shift*I as local CSR (sorted columns)."""
    p = min(1.0, mean_degree / max(n - 1, 1))
    m = rng.binomial(n * (n - 1) // 2, p)
    a = rng.integers(0, n, size=2 * m + 16)
    b = rng.integers(0, n, size=2 * m + 16)
    keep = a != b
    a, b = a[keep], b[keep]
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    key = np.unique(lo.astype(np.int64) * n + hi)[:m]
    rng.shuffle(key)
    lo, hi = key // n, key % n
    w = rng.uniform(wlo, whi, size=len(key))
    r = np.concatenate([lo, hi, np.arange(n)])
    c = np.concatenate([hi, lo, np.arange(n)])
    deg = np.bincount(lo, w, n) + np.bincount(hi, w, n)
    v = np.concatenate([-w, -w, deg + shift])
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    pntr = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(r, minlength=n), out=pntr[1:])
    return pntr, c.astype(np.int64), v


def er_laplacian_batch(num_systems=4096, nmin=64, nmax=4096, seed=4, mean_degree=8.0,
                       shift=0.01, dtype=np.float32):
    """Block-diagonal CSR of independent systems with sizes log-uniform in [nmin, nmax].
    Returns (sys_ptr[num_systems+1] row offsets, pntr, indx (global columns), vals)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(nmin), np.log(nmax), size=num_systems)).astype(np.int64)
    sizes = np.clip(sizes, nmin, nmax)
    sys_ptr = np.zeros(num_systems + 1, np.int64)
    np.cumsum(sizes, out=sys_ptr[1:])
    P, I, V = [np.zeros(1, np.int64)], [], []
    nnz = 0
    for s, n in enumerate(sizes):
        p, c, v = er_laplacian(int(n), rng, mean_degree=mean_degree, shift=shift)
        P.append(p[1:] + nnz)
        I.append(c + sys_ptr[s])
        V.append(v)
        nnz += int(p[-1])
    pntr = np.concatenate(P).astype(np.int32)
    indx = np.concatenate(I).astype(np.int32)
    vals = np.concatenate(V).astype(dtype)
    return sys_ptr.astype(np.int32), pntr, indx, vals


def csr_to_dense(pntr, indx, vals, ncols=None):
    n = len(pntr) - 1
    ncols = n if ncols is None else ncols
    A = np.zeros((n, ncols), vals.dtype)
    for i in range(n):
        A[i, indx[pntr[i]:pntr[i + 1]]] = vals[pntr[i]:pntr[i + 1]]
    return A


def csr_matvec(pntr, indx, vals, x):
    """Vectorised A @ x in float64 (fixture helper; not an oracle of the summation order)."""
    n = len(pntr) - 1
    prod = vals.astype(np.float64) * x[indx]
    out = np.add.reduceat(prod, pntr[:-1].astype(np.int64)) if len(prod) else np.zeros(n)
    out[np.diff(pntr) == 0] = 0
    return out


def random_csr_sparse(n, per_row, rng):
    """Random square pattern with about per_row uniformly placed entries per row plus the diagonal
    (sorted columns, diagonally dominant), built without a dense mask."""
    rows = np.repeat(np.arange(n, dtype=np.int64), per_row)
    cols = rng.integers(0, n, size=n * per_row)
    key = np.unique(np.concatenate([rows * n + cols, np.arange(n, dtype=np.int64) * (n + 1)]))
    r, c = key // n, key % n
    v = rng.uniform(-1, 1, size=len(r))
    rowsum = np.bincount(r, np.abs(v), n)
    d = r == c
    v[d] = rowsum[r[d]] + 1.0
    pntr = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(r, minlength=n), out=pntr[1:])
    return pntr.astype(np.int32), c.astype(np.int32), v


def random_csr(n, density, rng, with_diag=True, dominant=True, ncols=None):
    """Random sparse matrix with sorted columns; optional full diagonal (diagonally dominant)."""
    ncols = n if ncols is None else ncols
    mask = rng.random((n, ncols)) < density
    if with_diag:
        mask[np.arange(min(n, ncols)), np.arange(min(n, ncols))] = True
    r, c = np.nonzero(mask)
    v = rng.uniform(-1, 1, size=len(r))
    if with_diag and dominant:
        rowsum = np.bincount(r, np.abs(v), n)
        d = r == c
        v[d] = rowsum[r[d]] + 1.0
    pntr = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(r, minlength=n), out=pntr[1:])
    return pntr.astype(np.int32), c.astype(np.int32), v.astype(np.float64)


def magnetic2d(nx, ny=None, flux=0.3, shift=0.05):
    """Hermitian positive definite complex matrix: 5-point Laplacian whose edge (i, j) carries the
    phase exp(i theta_ij), theta_ij = flux * (x_i + y_j) * sign, theta_ji = -theta_ij; diagonal
    4 + shift (the Gershgorin disks stay in the right half plane)."""
    p, i, v = poisson2d(nx, ny)
    nxx = nx
    vals = v.astype(np.complex128)
    for r in range(len(p) - 1):
        for q in range(p[r], p[r + 1]):
            c = int(i[q])
            if c == r:
                vals[q] = 4.0 + shift
            else:
                lo, hi = min(r, c), max(r, c)
                th = flux * ((lo % nxx) + 0.5 * (hi // nxx) + 0.25 * (hi - lo))
                vals[q] = -np.exp(1j * th) if r < c else -np.exp(-1j * th)
    return p, i, vals


def helmholtz_shift(p, i, v, sigma=(0.5, 0.5)):
    """v + (sigma_re + i sigma_im) on the diagonal, complex128."""
    vals = np.asarray(v, np.complex128).copy()
    s = complex(*sigma)
    for r in range(len(p) - 1):
        for q in range(p[r], p[r + 1]):
            if i[q] == r:
                vals[q] += s
    return p, i, vals
