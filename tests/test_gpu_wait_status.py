"""Bounded waits of the triangular-solve kernels report through a status flag.

A record copy that never lands is made on purpose only in the self-test
kernel (an mbarrier nothing arrives at, polled a bounded number of times):
the wait gives up, the flag is set, rchol_gpu_solve_status returns
RCHOL_ERR_TIMEOUT and clears it, and the context stays usable -- a solve run
afterwards matches the oracle and reports RCHOL_OK.
"""

import numpy as np
import pytest

from rchol_gb300 import _lib, generators

pytestmark = pytest.mark.gpu


def test_wait_timeout_is_reported_and_cleared(cuda, R, O):
    import torch

    L = _lib.lib()
    st = torch.cuda.current_stream().cuda_stream
    assert L.rchol_gpu_solve_status(st) == _lib.OK
    assert L.rchol_gpu_wait_selftest(2000, st) == _lib.ERR_TIMEOUT
    assert "gave up" in L.rchol_gpu_last_error().decode()
    assert L.rchol_gpu_solve_status(st) == _lib.OK  # read once, then cleared

    # the context is still usable: a solve after the timeout is correct
    A = generators.laplace_3d(12)
    tree = R.Tree.build(A.indptr, A.indices, 4)
    Ad = R.Matrix.create(A.indptr, A.indices, A.data, tree)
    F = R.Factor.compute(Ad, tree, seed=0)
    n = A.shape[0]
    r = torch.tensor(np.random.default_rng(0).standard_normal(n), device=cuda)
    z = torch.empty_like(r)
    _lib.check(L.rchol_gpu_trsv_d(F.ptr, 0, r.data_ptr(), z.data_ptr(), 1, st))
    assert L.rchol_gpu_solve_status(st) == _lib.OK
    G = F.export()
    y = O.trsv_lower(G, r.cpu().numpy())
    assert np.max(np.abs(z.cpu().numpy() - y)) <= 1e-12 * max(1.0, np.max(np.abs(y)))
