"""The allocation-free preconditioner entry point (rchol_gpu_precond_noalloc_d).

It serves callers that cannot allocate device memory at solve time; its two
scratch vectors live in a fixed device array inside the library.  Checked
through the C ABI against rchol_gpu_precond_d on two calls in a row (the
array keeps the previous call's contents, which must not leak into the next
result), for FP64 and FP32 factors, plus the size limit.  This file is
collected last so that a failure here stops a -x run only after every other
test has run; it also passes alone in a fresh process.
"""

import numpy as np
import pytest

from rchol_gb300 import _lib, generators

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _precond(torch, fn, F, r):
    z = torch.empty_like(r)
    stream = torch.cuda.current_stream().cuda_stream
    if fn == "noalloc":
        _lib.check(_lib.lib().rchol_gpu_precond_noalloc_d(F.ptr, r.data_ptr(), z.data_ptr(), stream))
    else:
        _lib.check(_lib.lib().rchol_gpu_precond_d(F.ptr, r.data_ptr(), z.data_ptr(), 1, stream))
    torch.cuda.synchronize()
    return z.cpu().numpy()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_noalloc_matches_allocating_entry_point(cuda, R, precision):
    import torch

    A = generators.laplace_3d_weighted(20, sigma=1.0, seed=7)
    tree = R.Tree.build(A.indptr, A.indices, 16)
    Ad = R.Matrix.create(A.indptr, A.indices, A.data, tree)
    F = R.Factor.compute(Ad, tree, seed=3, precision=precision)
    rng = np.random.default_rng(11)
    for call in range(2):  # two calls in a row through the shared scratch array
        r = torch.tensor(rng.standard_normal(A.shape[0]), device=cuda)
        z_new = _precond(torch, "noalloc", F, r)
        z_ref = _precond(torch, "alloc", F, r)
        assert np.linalg.norm(z_new - z_ref) <= TOL * np.linalg.norm(z_ref), call


def test_noalloc_rejects_sizes_beyond_its_array(cuda, R):
    import torch

    n = (16 << 20) // 16 + 1  # one more unknown than an FP64 factor fits
    rp = np.arange(n + 1, dtype=np.int64)
    F = R.Factor.from_host(rp, np.arange(n, dtype=np.int64), np.ones(n))
    r = torch.ones(n, dtype=torch.float64, device=cuda)
    with pytest.raises(ValueError, match="scratch"):
        _precond(torch, "noalloc", F, r)
