"""Host side of the product (no GPU needed): ordering, reorder, generators,
argument checking -- bit-exact against the oracle."""

import numpy as np
import pytest

from rchol_gb300 import _lib, generators
from conftest import csr_u64


@pytest.mark.parametrize("n,threads", [(6, 1), (6, 2), (8, 4), (12, 8), (16, 32), (24, 64)])
def test_ordering_bit_exact(O, R, n, threads):
    A = R.laplace_3d(n)
    tree = R.Tree.build(A.indptr, A.indices, threads)
    perm, part = tree.arrays()
    po, ro = O.order(csr_u64(A), threads)
    assert np.array_equal(perm, po.astype(np.int64))
    assert np.array_equal(part, ro.astype(np.int64))
    assert part[-1] == A.shape[0] + 1 and len(part) == 2 * threads


@pytest.mark.parametrize("n,threads", [(8, 2), (12, 8), (16, 32)])
def test_ordering_python_front_end_variant(O, R, n, threads):
    """The Python front end's ordering (last vertex forced into the root
    separator, python/rchol_lap/find_separator.pyx:27-28), bit-exact."""
    A = R.laplace_3d(n)
    tree = R.Tree.build(A.indptr, A.indices, threads, last_in_root=True)
    perm, part = tree.arrays()
    po, ro = O.order(csr_u64(A), threads, last_in_root=True)
    assert np.array_equal(perm, po.astype(np.int64))
    assert np.array_equal(part, ro.astype(np.int64))
    root = perm[part[-2]:part[-1] - 1]  # the root separator (ground excluded)
    assert A.shape[0] - 1 in root
    plain, _ = R.Tree.build(A.indptr, A.indices, threads).arrays()
    assert not np.array_equal(plain, perm) or A.shape[0] - 1 in plain[part[-2]:]


def test_ordering_python_variant_matches_reference_fixture(O, R):
    """Against the reference's own Cython find_separator, run as
    python/rchol/rchol.py does (tests/golden/make_python_order.py)."""
    import os

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "python_order.npz"))
    cases = sorted({k.split("_", 1)[1] for k in g.files})
    assert cases
    for case in cases:
        n, nt = (int(x) for x in case.split("_"))
        A = R.laplace_3d(n)
        perm, part = R.Tree.build(A.indptr, A.indices, nt, last_in_root=True).arrays()
        assert np.array_equal(perm, g["perm_" + case]), case
        assert np.array_equal(part, g["part_" + case]), case
        po, ro = O.order(csr_u64(A), nt, last_in_root=True)
        assert np.array_equal(po.astype(np.int64), g["perm_" + case]), case


@pytest.mark.parametrize("leaf_order", ["nd", "md"])
@pytest.mark.parametrize("n,threads", [(8, 1), (10, 2), (12, 8)])
def test_leaf_orderings_bit_exact_and_fill_reducing(O, R, n, threads, leaf_order):
    """Fill-reducing order inside the leaves (the MATLAB front end's amd step,
    matlab/rchol/find_separator.m:6): host and oracle agree bit for bit, the
    separators are untouched, and the factor has less fill than with the
    natural leaf order."""
    import oracle

    A = R.laplace_3d(n)
    Au = csr_u64(A)
    perm, part = R.Tree.build(A.indptr, A.indices, threads, leaf_order=leaf_order).arrays()
    po, ro = O.order(Au, threads, leaf_order=leaf_order)
    assert np.array_equal(perm, po.astype(np.int64)) and np.array_equal(part, ro.astype(np.int64))
    nat, part0 = R.Tree.build(A.indptr, A.indices, threads).arrays()
    assert np.array_equal(part, part0)
    for a, b in zip(part[:-1], part[1:]):  # same vertex set per segment
        b = min(b, A.shape[0])
        assert np.array_equal(np.sort(perm[a:b]), np.sort(nat[a:b]))
    fill = {}
    for name, p_ in (("natural", nat), (leaf_order, perm)):
        Ap = O.reorder(Au, p_.astype(np.uint64))
        G, d, _ = O.factor(O.extend(Ap), part.astype(np.uint64), oracle.MODE_DEVICE, 3)
        fill[name] = len(G[1])
    assert fill[leaf_order] < fill["natural"], fill


def test_ordering_forked_workers_match_serial(O, R, monkeypatch):
    """Large enough that subtrees go to forked worker processes."""
    A = R.laplace_3d(40)
    tree = R.Tree.build(A.indptr, A.indices, 16)
    perm, part = tree.arrays()
    po, ro = O.order(csr_u64(A), 16)
    assert np.array_equal(perm, po.astype(np.int64)) and np.array_equal(part, ro.astype(np.int64))


@pytest.mark.parametrize("maker", [
    lambda: generators.laplace_3d_weighted(9, sigma=1.0, seed=1),
    lambda: generators.grid_2d_weighted(31, 17, "loguniform", shift=1e-4, dirichlet=False, seed=3),
    lambda: generators.checkerboard_3d(12, block=4),
])
def test_ordering_weighted(O, R, maker):
    A = maker()
    tree = R.Tree.build(A.indptr, A.indices, 8)
    perm, part = tree.arrays()
    po, ro = O.order(csr_u64(A), 8)
    assert np.array_equal(perm, po.astype(np.int64)) and np.array_equal(part, ro.astype(np.int64))


def test_reorder_matches_oracle(O, R):
    A = generators.laplace_3d_weighted(7, seed=9)
    perm = np.random.default_rng(0).permutation(A.shape[0])
    got = _lib.reorder(A.indptr, A.indices, A.data, perm)
    want = O.reorder(csr_u64(A), perm.astype(np.uint64))
    for g, w in zip(got, want):
        assert np.array_equal(g, w.astype(g.dtype))


def test_generator_matches_reference_layout(O):
    for n in (3, 5, 9):
        A = generators.laplace_3d(n)
        rp, ci, v = O.laplace_3d(n)
        assert np.array_equal(A.indptr, rp.astype(A.indptr.dtype))
        assert np.array_equal(A.indices, ci.astype(A.indices.dtype))
        assert np.array_equal(A.data, v)


@pytest.mark.parametrize("maker", [
    lambda: generators.laplace_3d_weighted(6, sigma=1.0, shift=1e-3, seed=0),
    lambda: generators.grid_2d_weighted(9, 13, "lognormal", sigma=0.5, seed=0),
    lambda: generators.grid_2d_weighted(9, 13, "loguniform", shift=1e-4, dirichlet=False, seed=0),
    lambda: generators.checkerboard_3d(16, block=8),
])
def test_generators_are_sddm(maker):
    A = maker()
    assert (A != A.T).nnz == 0
    d = A.diagonal()
    rowsum = np.asarray(A.sum(axis=1)).ravel()
    assert (d > 0).all()
    # weakly diagonally dominant everywhere, strictly somewhere (shift or Dirichlet)
    assert (rowsum > -1e-12 * d).all() and (rowsum > 1e-12 * d).any()
    A2 = A.tocoo()
    offd = A2.data[A2.row != A2.col]
    assert (offd < 0).all()


def test_checkerboard_values():
    A = generators.checkerboard_3d(16, block=8)
    # an edge inside a block has weight = coefficient, across blocks the harmonic mean
    w = -A[0, 1]
    assert w == 1.0
    w2 = -A[7, 8]  # k=7 -> k=8 crosses into the 1e4 block
    assert abs(w2 - 2 * 1e4 / (1 + 1e4)) < 1e-12


def test_argument_errors(R):
    A = R.laplace_3d(3)
    with pytest.raises(ValueError, match="power of 2"):
        R.Tree.build(A.indptr, A.indices, 3)
    with pytest.raises(ValueError, match="positive"):
        R.Tree.build(A.indptr, A.indices, 0)
    with pytest.raises(ValueError, match="too many threads"):
        R.Tree.build(A.indptr, A.indices, 512)
    bad = A.indices.copy()
    bad[0] = 10 ** 6
    with pytest.raises(ValueError, match="out of range"):
        R.Tree.build(A.indptr, bad, 2)
    with pytest.raises(ValueError):
        R.Tree.from_partition(np.arange(27), np.array([0, 5, 28]))  # length not 2*power of 2
    with pytest.raises(ValueError, match="permutation"):
        R.Tree.from_partition(np.zeros(27, np.int64), np.array([0, 28]))
    with pytest.raises(Exception, match="given together"):
        R.rchol(A, 2, perm=np.arange(27))


def test_tree_from_partition_roundtrip(R):
    A = R.laplace_3d(10)
    t = R.Tree.build(A.indptr, A.indices, 8)
    perm, part = t.arrays()
    t2 = R.Tree.from_partition(perm, part)
    p2, q2 = t2.arrays()
    assert np.array_equal(perm, p2) and np.array_equal(part, q2)
