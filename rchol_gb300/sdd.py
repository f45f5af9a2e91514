"""SDD systems through the SDDM preconditioner: host-side input adapters.

rchol needs an SDDM matrix (non-positive off-diagonals).  A symmetric
diagonally dominant matrix with some positive off-diagonals is brought into
that form in one of two ways, as the reference's MATLAB examples do:

* the sign-flip reduction (matlab/ex_sdd_opt.m): if a diagonal sign matrix S
  makes every off-diagonal of S A S non-positive, solve (S A S) y = S b and
  return x = S y -- same size as A;
* the extension (matlab/rchol/sdd_to_sddm.m, matlab/ex_sdd.m): with A = D + N + P
  (diagonal, negative and positive off-diagonal parts), the 2n x 2n matrix
  [[D + N, -P], [-P, D + N]] is SDDM; solve it with [b; -b] and return
  x = (x_1 - x_2) / 2.

``solve_sdd`` tries the reduction and falls back to the extension.  Both are
exact transformations; everything after them is the ordinary GPU path.
"""

from __future__ import annotations

from collections import deque

import numpy as np
import scipy.sparse as sp


def sdd_3d(n: int) -> sp.csr_matrix:
    """The reference's 3D SDD test matrix (matlab/rchol/sdd_3d.m): the 7-point
    Laplacian with the couplings along one axis flipped to +1, plus 4 I."""
    e = np.ones(n)
    I = sp.identity(n, format="csr")
    D = sp.diags([-e[:-1], 2 * e, -e[:-1]], [-1, 0, 1], format="csr")
    A1 = sp.kron(D, I, format="csr")
    A2 = sp.kron(I, D, format="csr")
    A = sp.kron(A1, -I) + sp.kron(I, A1) + sp.kron(I, A2) + 4 * sp.identity(n ** 3)
    A = sp.csr_matrix(A)
    A.sum_duplicates()
    A.eliminate_zeros()
    A.sort_indices()
    return A


def _split(A):
    A = sp.csr_matrix(A, dtype=np.float64)
    d = A.diagonal()
    off = A - sp.diags(d)
    off = sp.csr_matrix(off)
    off.eliminate_zeros()
    pos = off.multiply(off > 0).tocsr()
    neg = off.multiply(off < 0).tocsr()
    return d, neg, pos


def sdd_to_sddm(A) -> sp.csr_matrix:
    """[[D + N, -P], [-P, D + N]] (matlab/rchol/sdd_to_sddm.m)."""
    d, neg, pos = _split(A)
    DN = sp.diags(d) + neg
    E = sp.bmat([[DN, -pos], [-pos, DN]], format="csr")
    E.sum_duplicates()
    E.eliminate_zeros()
    E.sort_indices()
    return E


def sign_flip(A):
    """Signs s (+1/-1) with every off-diagonal of diag(s) A diag(s) non-positive,
    found by a breadth-first 2-colouring (an edge with a positive entry joins
    opposite signs, a negative one equal signs); None if no such signs exist
    (a cycle with an odd number of positive entries)."""
    A = sp.csr_matrix(A)
    n = A.shape[0]
    s = np.zeros(n, dtype=np.int8)
    rp, ci, v = A.indptr, A.indices, A.data
    for root in range(n):
        if s[root]:
            continue
        s[root] = 1
        q = deque([root])
        while q:
            i = q.popleft()
            for k in range(rp[i], rp[i + 1]):
                j = ci[k]
                if j == i or v[k] == 0:
                    continue
                want = -s[i] if v[k] > 0 else s[i]
                if s[j] == 0:
                    s[j] = want
                    q.append(j)
                elif s[j] != want:
                    return None
    return s.astype(np.float64)


def solve_sdd(A, b, tol=1e-8, maxit=200, nt=1, precision="fp64", seed=0):
    """Solve the SDD system A x = b with the GPU preconditioner.  Returns
    (x, relres, iters, method) with method "sddm", "sign_flip" or "extension"."""
    from . import pcg, rchol

    A = sp.csr_matrix(A, dtype=np.float64)
    A.sort_indices()
    b = np.asarray(b, dtype=np.float64)
    _, _, pos = _split(A)
    if pos.nnz == 0:
        M, rhs, back, method = A, b, (lambda y: y), "sddm"
    else:
        s = sign_flip(A)
        if s is not None:
            S = sp.diags(s)
            M = sp.csr_matrix(S @ A @ S)
            rhs, back, method = s * b, (lambda y, s=s: s * y), "sign_flip"
        else:
            n = A.shape[0]
            M = sdd_to_sddm(A)
            rhs = np.concatenate([b, -b])
            back, method = (lambda y, n=n: (y[:n] - y[n:]) / 2), "extension"
    M.sort_indices()
    G, perm, part = rchol(M, nt, seed=seed, precision=precision)
    Mp = M[perm][:, perm]
    y, relres, itr = pcg(Mp, rhs[perm], tol, maxit, G)
    yy = np.empty_like(y)
    yy[perm] = y
    x = back(yy)
    return x, relres, itr, method
