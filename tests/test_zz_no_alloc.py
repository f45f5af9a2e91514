"""The allocation-free preconditioner entry point (rchol_gpu_precond_noalloc_d).

It serves callers that cannot allocate device memory at solve time (a memory
budget fixed at start-up, allocator-free real-time loops, hosts that own all
device memory); its two scratch vectors live in a fixed device array inside
the library.  Checked through the C ABI against rchol_gpu_precond_d on two
calls in a row (the array keeps the previous call's contents, which must not
leak into the next result), for FP64 and FP32 factors; free device memory
does not drop across its first call on a fresh factor; and the size limit
holds exactly (n at the limit works, one more is rejected) for both
precisions.  This file is collected last so that a failure here stops a -x
run only after every other test has run; it also passes alone in a fresh
process.
"""

import numpy as np
import pytest

from rchol_gb300 import _lib, generators

pytestmark = pytest.mark.gpu

TOL = 1e-12
SCRATCH_BYTES = 16 << 20
LIMIT = {0: SCRATCH_BYTES // 16, 1: SCRATCH_BYTES // 8}  # largest n: two vectors of 8 (FP64) or 4 (FP32) bytes


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
    rs = [torch.tensor(rng.standard_normal(A.shape[0]), device=cuda) for _ in range(2)]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    z_first = _precond(torch, "noalloc", F, rs[0])  # first call on this factor
    assert torch.cuda.mem_get_info()[0] >= free0, "the allocation-free entry point took device memory"
    for call in range(2):  # two calls in a row through the shared scratch array
        z_new = z_first if call == 0 else _precond(torch, "noalloc", F, rs[call])
        z_ref = _precond(torch, "alloc", F, rs[call])
        assert np.linalg.norm(z_new - z_ref) <= TOL * np.linalg.norm(z_ref), call


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_noalloc_size_limit_is_exact(cuda, R, precision):
    """n at the limit gives the allocating entry point's result (a diagonal
    factor); n one past it raises ValueError naming the scratch size."""
    import torch

    for n, ok in ((LIMIT[precision], True), (LIMIT[precision] + 1, False)):
        rp = np.arange(n + 1, dtype=np.int64)
        d = np.random.default_rng(n).uniform(0.5, 2.0, n)
        F = R.Factor.from_host(rp, np.arange(n, dtype=np.int64), d, precision=precision)
        r = torch.tensor(np.random.default_rng(1).standard_normal(n), device=cuda)
        if ok:
            z_new = _precond(torch, "noalloc", F, r)
            z_ref = _precond(torch, "alloc", F, r)
            assert np.linalg.norm(z_new - z_ref) <= TOL * np.linalg.norm(z_ref)
        else:
            with pytest.raises(ValueError, match="scratch"):
                _precond(torch, "noalloc", F, r)
        del F
