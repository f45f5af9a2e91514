"""SDD -> SDDM input adapters (matlab/rchol/sdd_to_sddm.m, matlab/ex_sdd.m,
matlab/ex_sdd_opt.m): the transformations are exact (checked with a direct
solve on the CPU), and SDD systems solve through the GPU path."""

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from rchol_gb300 import sdd


def _odd_cycle_sdd(n=31, seed=0):
    """An SDD matrix whose positive couplings form an odd cycle (no sign flip)."""
    rng = np.random.default_rng(seed)
    rows, cols, vals = [], [], []
    for i in range(n):  # ring of positive couplings, n odd -> odd cycle
        j = (i + 1) % n
        w = rng.uniform(0.5, 1.5)
        rows += [i, j]
        cols += [j, i]
        vals += [w, w]
    for i in range(n - 2):  # some negative couplings
        w = rng.uniform(0.5, 1.5)
        rows += [i, i + 2]
        cols += [i + 2, i]
        vals += [-w, -w]
    M = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    d = np.asarray(abs(M).sum(axis=1)).ravel() + 0.1
    return sp.csr_matrix(M + sp.diags(d))


def test_sdd_3d_is_sdd_with_positive_couplings():
    A = sdd.sdd_3d(6)
    assert (A - A.T).nnz == 0
    d = A.diagonal()
    off = A - sp.diags(d)
    assert np.all(d >= np.asarray(abs(off).sum(axis=1)).ravel())
    assert (off > 0).nnz > 0


def test_sign_flip_makes_sddm_and_is_exact():
    A = sdd.sdd_3d(6)
    s = sdd.sign_flip(A)
    assert s is not None
    Ag = sp.diags(s) @ A @ sp.diags(s)
    off = Ag - sp.diags(Ag.diagonal())
    assert (off > 0).nnz == 0
    b = np.random.default_rng(1).uniform(0, 1, A.shape[0])
    xg = spla.spsolve(sp.csc_matrix(Ag), s * b)
    assert np.linalg.norm(A @ (s * xg) - b) <= 1e-10 * np.linalg.norm(b)


def test_extension_is_sddm_and_exact():
    A = _odd_cycle_sdd()
    assert sdd.sign_flip(A) is None
    E = sdd.sdd_to_sddm(A)
    off = E - sp.diags(E.diagonal())
    assert (off > 0).nnz == 0 and E.shape == (2 * A.shape[0],) * 2
    b = np.random.default_rng(2).uniform(-1, 1, A.shape[0])
    y = spla.spsolve(sp.csc_matrix(E), np.concatenate([b, -b]))
    n = A.shape[0]
    x = (y[:n] - y[n:]) / 2
    assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["sign_flip", "extension", "sddm"])
def test_solve_sdd_on_gpu(cuda, which):
    if which == "sign_flip":
        A = sdd.sdd_3d(10)
    elif which == "extension":
        A = _odd_cycle_sdd(301)
    else:
        from rchol_gb300 import laplace_3d
        A = laplace_3d(10)
    b = np.random.default_rng(3).uniform(-1, 1, A.shape[0])
    x, relres, itr, method = sdd.solve_sdd(A, b, tol=1e-10, maxit=300, nt=2)
    assert method == which
    assert np.linalg.norm(A @ x - b) <= 1e-8 * np.linalg.norm(b)
