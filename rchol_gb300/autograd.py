"""Differentiable SDDM solves: x = A(w)^-1 b with gradients for b and w.

    A(w) = sum_e w_e (u_i - u_j)(u_i - u_j)^T + diag(shift)

on a fixed graph with edges e = (i, j).  The forward pass factors A(w) with
the GPU randomized Cholesky (ordering computed once per graph) and solves with
PCG; the backward pass solves the adjoint system A lambda = dL/dx with the SAME
factor (A is symmetric) and evaluates the edge gradients with a CUDA kernel:

    dL/db = lambda,        dL/dw_e = -(lambda_i - lambda_j) (x_i - x_j).

The reference has no differentiable front end; this module is an addition on
top of the same C ABI (rchol_gpu_pcg_d, rchol_gpu_edge_grad_d).
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib
from ._lib import Factor, Matrix, PREC_FP64, Tree


class LaplacianOperator:
    """A(w) on a fixed graph, resident on one GPU."""

    def __init__(self, n, ei, ej, shift=0.0, nt=64, seed=0, precision=PREC_FP64, device="cuda"):
        ei = np.asarray(ei, dtype=np.int64)
        ej = np.asarray(ej, dtype=np.int64)
        if np.any(ei == ej):
            raise ValueError("self loops are not edges")
        self.n, self.m = int(n), len(ei)
        self.device = torch.device(device)
        self.shift = np.broadcast_to(np.asarray(shift, dtype=np.float64), (self.n,)).copy()
        rows = np.concatenate([ei, ej, np.arange(self.n)])
        cols = np.concatenate([ej, ei, np.arange(self.n)])
        tag = np.arange(len(rows))  # position of each (row, col) in the COO list
        P = sp.csr_matrix((tag + 1.0, (rows, cols)), shape=(self.n, self.n))
        P.sum_duplicates()
        if P.nnz != len(rows):
            raise ValueError("duplicate edges")
        P.sort_indices()
        where = np.empty(len(rows), dtype=np.int64)
        where[(P.data - 1).astype(np.int64)] = np.arange(P.nnz)
        self.pos_ij, self.pos_ji, self.pos_d = where[: self.m], where[self.m: 2 * self.m], where[2 * self.m:]
        self.ei, self.ej = ei, ej
        self.indptr, self.indices = P.indptr.astype(np.int64), P.indices.astype(np.int64)
        self.tree = Tree.build(self.indptr, self.indices, nt)
        self.perm, self.part = self.tree.arrays()
        iperm = np.empty_like(self.perm)
        iperm[self.perm] = np.arange(self.n)
        self.iperm = iperm
        self.perm_t = torch.as_tensor(self.perm, device=self.device)
        self.iperm_t = torch.as_tensor(self.iperm, device=self.device)
        self.ei_p = torch.as_tensor(iperm[ei], device=self.device)
        self.ej_p = torch.as_tensor(iperm[ej], device=self.device)
        self.seed, self.precision = seed, precision
        self.A = None
        self.F = None
        self._w = None

    def values(self, w):
        """CSR values of A(w) (the pattern of self.indptr / self.indices)."""
        w = np.asarray(w, dtype=np.float64)
        data = np.empty(len(self.indices))
        data[self.pos_ij] = -w
        data[self.pos_ji] = -w
        data[self.pos_d] = self.shift + np.bincount(self.ei, w, self.n) + np.bincount(self.ej, w, self.n)
        return data

    def matrix(self, w):
        return sp.csr_matrix((self.values(w), self.indices, self.indptr), shape=(self.n, self.n))

    def update(self, w: torch.Tensor):
        """Assemble and factor A(w) unless w is the current weight vector."""
        wn = w.detach().to("cpu", torch.float64).numpy()
        if self._w is not None and np.array_equal(wn, self._w):
            return
        data = self.values(wn)
        if self.A is None:
            self.A = Matrix.create(self.indptr, self.indices, data, self.tree)
        else:
            self.A.set_values(data)
        self.F = Factor.compute(self.A, self.tree, seed=self.seed, precision=self.precision)
        self._w = wn.copy()

    def solve_permuted(self, bp: torch.Tensor, tol, maxit):
        """PCG on A(p,p) x = b(p) with device tensors already in the permuted order."""
        bp = bp.to(torch.float64).contiguous()
        xp = torch.empty_like(bp)
        k = 1 if bp.dim() == 1 else bp.shape[1]
        relres = np.zeros(k)
        itr = np.zeros(k, dtype=np.int32)
        stream = torch.cuda.current_stream(self.device).cuda_stream
        _lib.check(_lib.lib().rchol_gpu_pcg_d(self.A.ptr, self.F.ptr, bp.data_ptr(), xp.data_ptr(), k, float(tol),
                                              int(maxit), _lib.pd(relres), itr.ctypes.data_as(_lib._ip), stream))
        self.last_relres, self.last_iters = relres.copy(), itr.copy()
        return xp

    def edge_grad(self, lam_p: torch.Tensor, x_p: torch.Tensor):
        g = torch.empty(self.m, dtype=torch.float64, device=self.device)
        stream = torch.cuda.current_stream(self.device).cuda_stream
        _lib.check(_lib.lib().rchol_gpu_edge_grad_d(self.m, self.ei_p.data_ptr(), self.ej_p.data_ptr(),
                                                    lam_p.data_ptr(), x_p.data_ptr(), g.data_ptr(), stream))
        return g


class _LaplacianSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, w, b, op, tol, maxit):
        op.update(w)
        xp = op.solve_permuted(b.index_select(0, op.perm_t), tol, maxit)
        ctx.op, ctx.tol, ctx.maxit = op, tol, maxit
        ctx.save_for_backward(w, xp)
        return xp.index_select(0, op.iperm_t)

    @staticmethod
    def backward(ctx, gx):
        w, xp = ctx.saved_tensors
        op = ctx.op
        op.update(w)  # the adjoint needs A(w) of this forward pass
        lam_p = op.solve_permuted(gx.index_select(0, op.perm_t), ctx.tol, ctx.maxit)
        gb = lam_p.index_select(0, op.iperm_t) if ctx.needs_input_grad[1] else None
        gw = op.edge_grad(lam_p, xp).to(w.dtype) if ctx.needs_input_grad[0] else None
        return gw, gb, None, None, None


def laplacian_solve(w: torch.Tensor, b: torch.Tensor, op: LaplacianOperator, tol=1e-12, maxit=1000):
    """x = A(w)^-1 b, differentiable in w and b."""
    return _LaplacianSolve.apply(w, b, op, tol, maxit)
