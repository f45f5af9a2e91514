"""rchol_gb300: rchol's preconditioned-solve path on one GB300 GPU.

Front end over the C ABI in include/rchol_gpu.h (librchol_gb300.so), shaped
like the reference's Python package (python/rchol/rchol.py, util.py):

    G, perm, part = rchol(A, nt, perm, part)      # python/rchol/rchol.py:8-45
    x, relres, itr = pcg(A, b, tol, maxit, G, Gt)  # python/rchol/util.py:32-61

``A`` is a scipy.sparse SDDM matrix; ``G`` comes back as the lower-triangular
scipy CSR matrix the reference returns (G = L sqrt(D)) and also carries the
GPU-resident factor, so pcg() reuses it without a copy.  ``Solver`` keeps A
and G on the device for repeated solves with torch tensors, and
``autograd.solve`` differentiates x = A^-1 b.  Ordering (METIS nested
dissection) runs on the host; factorization and solves run on the GPU.  There
is no CPU fallback: without the CUDA library every call raises.
"""

from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp

from . import _lib
from ._lib import PREC_FP32, PREC_FP64, Factor, Matrix, RcholError, Tree
from .batch import Batch
from .generators import (checkerboard_3d, grid_2d_weighted, laplace_3d, laplace_3d_weighted,
                         sddm_to_laplacian)

__all__ = ["rchol", "pcg", "Solver", "Batch", "Tree", "Matrix", "Factor", "RcholError", "laplace_3d",
           "laplace_3d_weighted", "grid_2d_weighted", "checkerboard_3d", "sddm_to_laplacian",
           "PREC_FP64", "PREC_FP32", "precision_code"]


def precision_code(precision) -> int:
    if precision in (PREC_FP64, "fp64", "float64", "double", np.float64):
        return PREC_FP64
    if precision in (PREC_FP32, "fp32", "float32", "float", np.float32):
        return PREC_FP32
    raise ValueError(f"unknown precision {precision!r}")


def _csr(A):
    A = sp.csr_matrix(A)
    A.sum_duplicates()
    A.sort_indices()
    return A


def rchol(A, nt=1, perm=np.array([]), part=np.array([]), seed=0, precision="fp64", order="python",
          leaf_order="natural"):
    """Randomized Cholesky preconditioner of an SDDM matrix on the GPU.

    Mirrors python/rchol/rchol.py:8-45.  ``nt`` is the number of leaf
    subdomains of the nested-dissection tree (the reference's thread count,
    a power of two); ``perm``/``part`` reuse an earlier ordering and must be
    given together.  ``order="python"`` is the Python front end's nested
    dissection (the last vertex goes into the root separator,
    python/rchol_lap/find_separator.pyx:27-28), ``"c++"`` the C++ front
    end's.  ``leaf_order`` ("natural", "nd", "md") reorders inside the leaf
    subdomains as the MATLAB front end does with amd
    (matlab/rchol/find_separator.m:6): less fill, usually more PCG
    iterations.  Returns ``(G, perm, part)`` with G lower triangular such
    that G G^T approximates A[perm][:, perm].
    """
    if order not in ("python", "c++"):
        raise ValueError("order must be 'python' or 'c++'")
    if nt < 1:
        raise Exception("number of threads must be at least 1")
    perm = np.asarray(perm)
    part = np.asarray(part)
    if (perm.size > 0) ^ (part.size > 0):
        raise Exception("permutation and partition must be given together")
    if not math.log2(nt).is_integer():
        nt = 2 ** int(math.floor(math.log2(nt)))
        print("number of threads rounded down to {}".format(nt))
    A = _csr(A)
    if perm.size == 0:
        tree = Tree.build(A.indptr, A.indices, nt, last_in_root=(order == "python"), leaf_order=leaf_order)
    else:
        tree = Tree.from_partition(perm, part)
    perm, part = tree.arrays()
    Ad = Matrix.create(A.indptr, A.indices, A.data, tree)
    F = Factor.compute(Ad, tree, seed=seed, precision=precision_code(precision))
    G = factor_to_scipy(F)
    G._rchol_factor = F
    G._rchol_tree = tree
    return G, perm, part


def factor_to_scipy(F: Factor) -> sp.csr_matrix:
    """Lower-triangular G (scipy CSR) from a device factor."""
    rp, ci, v = F.export()
    n = len(rp) - 1
    Gt = sp.csr_matrix((v, ci, rp), shape=(n, n))
    return Gt.transpose().tocsr()


def pcg(A, b, epsilon, maxitr, G, Gt=None):
    """Preconditioned CG with M = G G^T on the GPU (python/rchol/util.py:32-61,
    c++/util/pcg.cpp:57-127).  ``b`` may be a vector or an n x k array (k
    right-hand sides, each with its own stopping test).  Returns
    (x, relres, niters); with k > 1, relres and niters are arrays."""
    A = _csr(A)
    b = np.asarray(b, dtype=np.float64)
    n = A.shape[0]
    k = 1 if b.ndim == 1 else b.shape[1]
    F = getattr(G, "_rchol_factor", None)
    if F is None:
        Gt_ = sp.csr_matrix(Gt) if Gt is not None else sp.csr_matrix(G).transpose().tocsr()
        Gt_.sort_indices()
        F = Factor.from_host(Gt_.indptr, Gt_.indices, Gt_.data)
    Ad = Matrix.create(A.indptr, A.indices, A.data)
    x, relres, itr = _pcg_host(Ad, F, b.reshape(n, k), epsilon, maxitr)
    if b.ndim == 1:
        return x[:, 0], float(relres[0]), int(itr[0])
    return x, relres, itr


def _pcg_host(Ad, F, B, tol, maxit):
    n, k = B.shape
    B = np.ascontiguousarray(B, dtype=np.float64)
    X = np.zeros((n, k))
    relres = np.zeros(k)
    itr = np.zeros(k, dtype=np.int32)
    _lib.check(_lib.lib().rchol_gpu_pcg(Ad.ptr, F.ptr, _lib.pd(B), _lib.pd(X), k, float(tol), int(maxit),
                                        _lib.pd(relres), itr.ctypes.data_as(_lib._ip)))
    return X, relres, itr


class Solver:
    """A and G resident on the GPU for repeated solves.

    Builds the ordering (host), uploads A(p,p) and factors it on the GPU.
    ``solve`` takes right-hand sides in the ORIGINAL ordering (numpy or torch,
    shape (n,) or (n, k)) and returns x in the original ordering.
    """

    def __init__(self, A, nt=64, seed=0, precision="fp64", perm=None, part=None):
        A = _csr(A)
        self.n = A.shape[0]
        if perm is None:
            self.tree = Tree.build(A.indptr, A.indices, nt)
        else:
            self.tree = Tree.from_partition(perm, part)
        self.perm, self.part = self.tree.arrays()
        self.A = Matrix.create(A.indptr, A.indices, A.data, self.tree)
        self.G = Factor.compute(self.A, self.tree, seed=seed, precision=precision_code(precision))
        self.iperm = np.empty_like(self.perm)
        self.iperm[self.perm] = np.arange(self.n)

    def solve(self, b, tol=1e-8, maxit=200, return_info=False):
        try:
            import torch
        except ImportError:  # numpy-only path
            torch = None
        if torch is not None and isinstance(b, torch.Tensor):
            return self._solve_torch(b, tol, maxit, return_info)
        b = np.asarray(b, dtype=np.float64)
        B = b.reshape(self.n, -1)[self.perm]
        X, relres, itr = _pcg_host(self.A, self.G, B, tol, maxit)
        x = X[self.iperm].reshape(b.shape)
        return (x, relres, itr) if return_info else x

    def _solve_torch(self, b, tol, maxit, return_info):
        import torch
        if not b.is_cuda:
            raise ValueError("torch right-hand sides must be CUDA tensors")
        shape = b.shape
        B = b.reshape(self.n, -1).to(torch.float64)
        perm = torch.as_tensor(self.perm, device=b.device)
        Bp = B.index_select(0, perm).contiguous()
        Xp = torch.empty_like(Bp)
        k = Bp.shape[1]
        relres = np.zeros(k)
        itr = np.zeros(k, dtype=np.int32)
        stream = torch.cuda.current_stream(b.device).cuda_stream
        _lib.check(_lib.lib().rchol_gpu_pcg_d(self.A.ptr, self.G.ptr, Bp.data_ptr(), Xp.data_ptr(), k,
                                              float(tol), int(maxit), _lib.pd(relres),
                                              itr.ctypes.data_as(_lib._ip), stream))
        X = torch.empty_like(Xp)
        X.index_copy_(0, perm, Xp)
        x = X.reshape(shape)
        return (x, relres, itr) if return_info else x
