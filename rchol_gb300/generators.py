"""Synthetic SDDM test matrices (CSR with sorted columns), vectorised numpy.

``laplace_3d`` reproduces the reference's 7-point Dirichlet Laplacian
(c++/util/laplace_3d.hpp:8-61: diagonal 6, off-diagonals -1, vertex
k + j*n + i*n^2).  The others build the weighted grid Laplacians the
benchmarks use; every random draw comes from ``numpy.random.default_rng(seed)``
in a fixed order, so a (shape, seed) pair always gives the same matrix.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def _assemble(n, ei, ej, w, diag):
    """Symmetric CSR from undirected edges (ei < ej, weights w > 0) and a diagonal."""
    rows = np.concatenate([ei, ej, np.arange(n)])
    cols = np.concatenate([ej, ei, np.arange(n)])
    vals = np.concatenate([-w, -w, diag])
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    A.sum_duplicates()
    A.sort_indices()
    return A


def _grid_edges_3d(nx, ny, nz):
    """Edges of an nx*ny*nz grid, vertex id = k + j*nz + i*ny*nz (k fastest)."""
    idx = np.arange(nx * ny * nz, dtype=np.int64).reshape(nx, ny, nz)
    out = []
    for a, b in ((idx[:-1, :, :], idx[1:, :, :]), (idx[:, :-1, :], idx[:, 1:, :]), (idx[:, :, :-1], idx[:, :, 1:])):
        out.append((a.ravel(), b.ravel()))
    return out


def laplace_3d(n: int) -> sp.csr_matrix:
    """7-point Laplacian with Dirichlet boundary on an n^3 grid (diag 6, off -1)."""
    N = n ** 3
    edges = _grid_edges_3d(n, n, n)
    ei = np.concatenate([e[0] for e in edges])
    ej = np.concatenate([e[1] for e in edges])
    return _assemble(N, ei, ej, np.ones(len(ei)), np.full(N, 6.0))


def laplace_3d_weighted(n: int, sigma: float = 1.0, shift: float = 1e-3, seed: int = 0) -> sp.csr_matrix:
    """7-point graph Laplacian on an n^3 grid with edge weights exp(sigma*N(0,1))
    plus ``shift`` on the diagonal (diag = sum of incident weights + shift)."""
    rng = np.random.default_rng(seed)
    N = n ** 3
    edges = _grid_edges_3d(n, n, n)
    ei = np.concatenate([e[0] for e in edges])
    ej = np.concatenate([e[1] for e in edges])
    w = np.exp(sigma * rng.standard_normal(len(ei)))
    deg = np.bincount(ei, w, N) + np.bincount(ej, w, N)
    return _assemble(N, ei, ej, w, deg + shift)


def grid_2d_weighted(nx: int, ny: int, weights: str = "lognormal", sigma: float = 0.5,
                     shift: float = 0.0, dirichlet: bool = True, seed: int = 0,
                     rng: np.random.Generator | None = None) -> sp.csr_matrix:
    """5-point weighted Laplacian on an nx*ny grid (vertex j + i*ny).

    weights: "lognormal" -> exp(sigma*N(0,1)); "loguniform" -> 10**U(-2, 2).
    dirichlet: every missing neighbour across the boundary is a grounded node
    joined by an edge of the same distribution, whose weight is added to the
    diagonal.  ``shift`` is added to every diagonal entry."""
    rng = rng if rng is not None else np.random.default_rng(seed)
    N = nx * ny
    idx = np.arange(N, dtype=np.int64).reshape(nx, ny)
    ei = np.concatenate([idx[:-1, :].ravel(), idx[:, :-1].ravel()])
    ej = np.concatenate([idx[1:, :].ravel(), idx[:, 1:].ravel()])

    def draw(m):
        if weights == "lognormal":
            return np.exp(sigma * rng.standard_normal(m))
        if weights == "loguniform":
            return 10.0 ** rng.uniform(-2.0, 2.0, m)
        raise ValueError("unknown weight distribution " + weights)

    w = draw(len(ei))
    deg = np.bincount(ei, w, N) + np.bincount(ej, w, N)
    if dirichlet:
        nb = np.zeros((nx, ny))
        nb[0, :] += 1
        nb[-1, :] += 1
        nb[:, 0] += 1
        nb[:, -1] += 1
        cnt = nb.ravel().astype(np.int64)
        owner = np.repeat(np.arange(N), cnt)
        deg += np.bincount(owner, draw(len(owner)), N)
    return _assemble(N, ei, ej, w, deg + shift)


def checkerboard_3d(n: int, block: int = 8, lo: float = 1.0, hi: float = 1e4) -> sp.csr_matrix:
    """7-point Laplacian on an n^3 grid whose cell coefficients form a
    block^3 checkerboard of ``lo`` and ``hi``.  An edge takes the harmonic mean
    of its two cells' coefficients; each Dirichlet boundary face adds the
    cell's own coefficient to the diagonal."""
    N = n ** 3
    c = np.arange(n) // block
    coef = np.where(((c[:, None, None] + c[None, :, None] + c[None, None, :]) & 1) == 0, lo, hi).ravel()
    edges = _grid_edges_3d(n, n, n)
    ei = np.concatenate([e[0] for e in edges])
    ej = np.concatenate([e[1] for e in edges])
    a, b = coef[ei], coef[ej]
    w = 2.0 * a * b / (a + b)
    deg = np.bincount(ei, w, N) + np.bincount(ej, w, N)
    i = np.arange(n)
    faces = ((i == 0).astype(int) + (i == n - 1))
    nf = (faces[:, None, None] + faces[None, :, None] + faces[None, None, :]).ravel()
    deg += nf * coef
    return _assemble(N, ei, ej, w, deg)


def sddm_to_laplacian(M: sp.spmatrix) -> sp.csr_matrix:
    """Extended Laplacian [[M, -M1], [-1^T M, 1^T M 1]] (python/rchol/util.py:22-29)."""
    one_row = -np.asarray(M.sum(axis=0)).ravel()
    total = -one_row.sum()
    M = sp.vstack([M, one_row], format="csr")
    one_col = np.append(one_row, total)
    return sp.hstack([M, one_col.reshape(-1, 1)], format="csr")
