"""Many independent SDDM systems solved together on one GPU.

The systems become the diagonal blocks of one matrix.  Each is ordered on its
own (nested dissection with ``threads`` leaves), the per-system trees hang
below empty separators of one tree, and one factorization, one SpMV and one
preconditioner apply per iteration serve every system, while PCG keeps
separate scalars, stopping tests and iteration counts per system
(rchol_gpu_pcg_batch).  No counterpart in the reference, which solves one
system per call (c++/util/pcg.cpp:14-55).
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from . import _lib
from ._lib import PREC_FP32, Factor, Matrix, Tree


def autotune_threads(mats, candidates=(1, 2, 4, 8, 16), sample=8, seed=0, precision=PREC_FP32, reps=3):
    """Leaves per system (the ``threads`` of Batch) chosen by measurement: the
    largest ``sample`` systems are factored with every candidate and the
    preconditioner apply (the dominant cost of a PCG iteration) is timed on
    the GPU with CUDA events; the fastest candidate wins.  Returns
    (best, {candidate: ms})."""
    import torch

    mats = list(mats)
    order = np.argsort([-A.shape[0] for A in mats])[: max(1, sample)]
    probe = [mats[i] for i in order]
    timings = {}
    stream = torch.cuda.current_stream()
    for t in candidates:
        if min(A.shape[0] for A in probe) < 4 * t:
            continue
        b = Batch(probe, threads=t, seed=seed, precision=precision)
        n = int(b.sys_ptr[-1])
        d_r = torch.as_tensor(np.random.default_rng(seed).standard_normal(n), device="cuda")
        d_z = torch.empty_like(d_r)

        def apply():
            _lib.check(_lib.lib().rchol_gpu_precond_d(b.F.ptr, d_r.data_ptr(), d_z.data_ptr(), 1,
                                                      stream.cuda_stream))

        apply()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            apply()
        e1.record(stream)
        torch.cuda.synchronize()
        timings[t] = e0.elapsed_time(e1) / reps
        del b
    return min(timings, key=timings.get), timings


class Batch:
    """Factor of a list of SDDM matrices (scipy.sparse, any sizes).  With
    ``threads=0`` the leaves per system are chosen by autotune_threads."""

    def __init__(self, mats, threads=4, seed=0, precision=PREC_FP32, G=None):
        if threads == 0:
            threads, self.tuning = autotune_threads(mats, seed=seed, precision=precision)
        self.threads = threads
        mats = [sp.csr_matrix(A) for A in mats]
        for A in mats:
            A.sum_duplicates()
            A.sort_indices()
        self.sizes = np.array([A.shape[0] for A in mats], dtype=np.int64)
        self.sys_ptr = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        U = sp.block_diag(mats, format="csr")
        U.sort_indices()
        self.U = U
        self.tree = Tree.build_batch(self.sys_ptr, U.indptr, U.indices, threads)
        self.perm, self.part = self.tree.arrays()
        self.A = Matrix.create(U.indptr, U.indices, U.data, self.tree)
        if G is None:
            self.F = Factor.compute(self.A, self.tree, seed=seed, precision=precision)
        else:  # a given factor of the permuted block-diagonal matrix (CSR of G^T)
            self.F = Factor.from_host(G[0], G[1], G[2], self.tree, precision=precision)

    @property
    def nsys(self):
        return len(self.sizes)

    def solve(self, bs, tol=1e-8, maxit=200):
        """Solve A_s x_s = b_s for every system; returns (xs, relres, iters)."""
        b = np.concatenate([np.asarray(v, dtype=np.float64) for v in bs])
        if b.shape[0] != self.sys_ptr[-1]:
            raise ValueError("right-hand sides do not match the systems")
        bp = np.ascontiguousarray(b[self.perm])
        xp = np.zeros_like(bp)
        relres = np.zeros(self.nsys)
        itr = np.zeros(self.nsys, dtype=np.int32)
        _lib.check(_lib.lib().rchol_gpu_pcg_batch(self.A.ptr, self.F.ptr, self.nsys, _lib.p64(self.sys_ptr),
                                                  _lib.pd(bp), _lib.pd(xp), float(tol), int(maxit),
                                                  _lib.pd(relres), itr.ctypes.data_as(_lib._ip)))
        x = np.empty_like(xp)
        x[self.perm] = xp
        xs = [x[self.sys_ptr[s]:self.sys_ptr[s + 1]] for s in range(self.nsys)]
        return xs, relres, itr
