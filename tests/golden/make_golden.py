"""Generates the golden fixtures in this directory from the UNMODIFIED
reference C++ (built by oracle/Makefile into oracle/_ref/librchol_ref.so with
the fixed-seed shim).  Run where the reference sources are available:

    python tests/golden/make_golden.py

Each fixture holds, for one small SDDM matrix: the reference's ordering
(find_separator + result_idx), the permuted matrix, the extended Laplacian,
the factor G (CSR of G^T) for a fixed sampler seed, and the reference PCG's
solution, relative residual and iteration count for a fixed right-hand side.
"""

from __future__ import annotations

import os
import platform
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from rchol_gb300 import generators  # noqa: E402

CASES = [
    # name, matrix builder, threads (0 = sequential rchol(A, G)), seed, tol
    ("lap6_seq", lambda R: R.laplace_3d(6), 0, 11, 1e-10),
    ("lap6_t4", lambda R: R.laplace_3d(6), 4, 5, 1e-10),
    ("lap10_t8", lambda R: R.laplace_3d(10), 8, 3, 1e-10),
    ("lap12_t2", lambda R: R.laplace_3d(12), 2, 21, 1e-8),
    ("weighted7_t4", lambda R: _csr(generators.laplace_3d_weighted(7, sigma=1.0, shift=1e-3, seed=4)), 4, 9, 1e-8),
    ("grid2d_t8", lambda R: _csr(generators.grid_2d_weighted(20, 17, "loguniform", shift=1e-4, dirichlet=False, seed=2)), 8, 13, 1e-8),
]


def _csr(A):
    return (A.indptr.astype(np.uint64), A.indices.astype(np.uint64), A.data.astype(np.float64))


def main():
    if not oracle.Reference.available():
        oracle.build(with_ref=True)
    R = oracle.Reference()
    for name, make, threads, seed, tol in CASES:
        A = make(R)
        n = len(A[0]) - 1
        G, perm = R.rchol(A, threads, seed)
        if threads:
            perm2, ridx = R.order(A, threads)
            assert np.array_equal(perm, perm2)
            Ap = R.reorder(A, perm)
        else:
            ridx = np.array([0, n + 1], dtype=np.uint64)
            Ap = A
        L = R.extend(Ap)
        b = np.random.default_rng(1000 + seed).uniform(-1, 1, n)
        x, relres, itr = R.pcg(Ap, b, tol, 200, G)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            A_rp=A[0], A_ci=A[1], A_v=A[2], threads=threads, seed=seed, tol=tol,
            perm=perm, ridx=ridx, Ap_rp=Ap[0], Ap_ci=Ap[1], Ap_v=Ap[2],
            L_rp=L[0], L_ci=L[1], L_v=L[2], G_rp=G[0], G_ci=G[1], G_v=G[2],
            b=b, x=x, relres=relres, itr=itr, arch=platform.machine())
        print(f"{name}: n={n} nnz(A)={len(A[1])} nnz(G)={len(G[1])} itr={itr} relres={relres:.2e}")


if __name__ == "__main__":
    main()
