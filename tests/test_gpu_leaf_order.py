"""Factor and PCG with a fill-reducing order inside the leaves (the MATLAB
front end orders its leaves with amd, matlab/rchol/find_separator.m:6; here
METIS nested dissection "nd" or the minimum-degree order "md", see
tests/test_host.py for the orderings themselves).

With the leaf order applied, the GPU factor equals the oracle's device
contract bit for bit on the same permutation, and the GPU PCG matches the
oracle PCG (c++/util/pcg.cpp:57-127) to 1e-12 with the same iteration count.
"""

import numpy as np
import pytest

import oracle
from rchol_gb300 import generators
from conftest import csr_u64

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("leaf_order", ["nd", "md"])
@pytest.mark.parametrize("case", ["laplace20", "weighted16"])
def test_leaf_order_factor_and_pcg(cuda, O, R, leaf_order, case):
    A = generators.laplace_3d(20) if case == "laplace20" else generators.laplace_3d_weighted(16, sigma=1.0, seed=4)
    Au = csr_u64(A)
    threads = 8
    tree = R.Tree.build(A.indptr, A.indices, threads, leaf_order=leaf_order)
    perm, part = tree.arrays()
    po, ro = O.order(Au, threads, leaf_order=leaf_order)
    assert np.array_equal(perm, po.astype(np.int64)) and np.array_equal(part, ro.astype(np.int64))
    Ad = R.Matrix.create(A.indptr, A.indices, A.data, tree)
    F = R.Factor.compute(Ad, tree, seed=11)
    grp, gci, gv = F.export()
    Ap = O.reorder(Au, po)
    Go, _, singular = O.factor(O.extend(Ap), ro, oracle.MODE_DEVICE, 11)
    assert not singular
    assert np.array_equal(grp, Go[0].astype(np.int64))
    assert np.array_equal(gci, Go[1].astype(np.int64))
    assert np.array_equal(gv, Go[2])
    n = A.shape[0]
    bp = np.random.default_rng(5).uniform(-1, 1, n)[perm]
    x, relres, itr = R._pcg_host(Ad, F, bp.reshape(n, 1), 1e-10, 200)
    xo, rro, ito = O.pcg(Ap, bp, 1e-10, 200, Go)
    assert int(itr[0]) == ito
    assert np.linalg.norm(x[:, 0] - xo) / np.linalg.norm(xo) < 1e-12
