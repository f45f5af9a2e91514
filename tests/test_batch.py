"""Many independent systems in one block-diagonal matrix (rchol_gpu_tree_build_batch,
rchol_gpu_pcg_batch): the ordering keeps every system in its own row range and
matches the per-system ordering, the factor of the union is block diagonal and
bit-exact with the oracle's device contract, and the batched PCG reproduces
the reference PCG of every system (identical iteration counts, iterates to
1e-12 or the reference's own rounding-order spread)."""

import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from conftest import csr_u64
from rchol_gb300 import generators

SIDES = [(12, 9), (20, 17), (7, 31), (25, 25), (16, 5)]


def _systems(seed=3):
    rng = np.random.default_rng(seed)
    return [generators.grid_2d_weighted(nx, ny, "lognormal", sigma=0.5, rng=rng) for nx, ny in SIDES]


def _union(mats):
    sizes = np.array([A.shape[0] for A in mats], dtype=np.int64)
    sys_ptr = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    U = sp.block_diag(mats, format="csr")
    U.sort_indices()
    return U, sys_ptr


@pytest.mark.parametrize("threads", [1, 2, 4])
def test_batch_ordering_keeps_systems(R, threads):
    mats = _systems()
    U, sys_ptr = _union(mats)
    T = R.Tree.build_batch(sys_ptr, U.indptr, U.indices, threads)
    perm, part = T.arrays()
    pad = 1 << int(np.ceil(np.log2(len(mats))))
    assert len(part) == 2 * pad * threads
    assert part[0] == 0 and part[-1] == U.shape[0] + 1
    for s, A in enumerate(mats):
        a, b = sys_ptr[s], sys_ptr[s + 1]
        ps = perm[a:b] - a
        assert np.array_equal(np.sort(ps), np.arange(b - a))
        # the same ordering as the system on its own
        Ts = R.Tree.build(A.indptr, A.indices, threads)
        assert np.array_equal(ps, Ts.arrays()[0])


def test_batch_rejects_coupled_systems(R):
    mats = _systems()
    U, sys_ptr = _union(mats)
    bad = sys_ptr.copy()
    bad[1] += 3  # cuts system 1 so that its edges cross the boundary
    with pytest.raises(ValueError, match="block diagonal"):
        R.Tree.build_batch(bad, U.indptr, U.indices, 2)


def test_batch_oracle_factor_is_block_diagonal(R, O):
    mats = _systems()
    U, sys_ptr = _union(mats)
    T = R.Tree.build_batch(sys_ptr, U.indptr, U.indices, 2)
    perm, part = T.arrays()
    Up = O.reorder(csr_u64(U), perm.astype(np.uint64))
    G, d, singular = O.factor(O.extend(Up), part.astype(np.uint64), oracle.MODE_DEVICE, 5)
    assert not singular
    n = U.shape[0]
    rows = np.repeat(np.arange(n), np.diff(G[0].astype(np.int64)))
    sys_of = np.searchsorted(sys_ptr, np.arange(n), side="right") - 1
    assert np.array_equal(sys_of[rows], sys_of[G[1].astype(np.int64)])


@pytest.mark.gpu
def test_batch_factor_matches_device_contract(cuda, R, O):
    mats = _systems()
    U, sys_ptr = _union(mats)
    T = R.Tree.build_batch(sys_ptr, U.indptr, U.indices, 2)
    perm, part = T.arrays()
    Ad = R.Matrix.create(U.indptr, U.indices, U.data, T)
    F = R.Factor.compute(Ad, T, seed=5)
    rp, ci, v = F.export()
    Up = O.reorder(csr_u64(U), perm.astype(np.uint64))
    G, d, _ = O.factor(O.extend(Up), part.astype(np.uint64), oracle.MODE_DEVICE, 5)
    assert np.array_equal(rp, G[0].astype(np.int64))
    assert np.array_equal(ci, G[1].astype(np.int64))
    assert np.array_equal(v, G[2])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_batch_pcg_matches_per_system_reference(cuda, R, O, precision):
    mats = _systems()
    U, sys_ptr = _union(mats)
    T = R.Tree.build_batch(sys_ptr, U.indptr, U.indices, 2)
    perm, part = T.arrays()
    Up = O.reorder(csr_u64(U), perm.astype(np.uint64))
    G, d, _ = O.factor(O.extend(Up), part.astype(np.uint64), oracle.MODE_REF, 11)
    B = R.Batch(mats, threads=2, precision=precision, G=G)
    assert np.array_equal(B.perm, perm)
    rng = np.random.default_rng(8)
    bs = [rng.standard_normal(A.shape[0]) for A in mats]
    tol = 1e-8
    xs, relres, itr = B.solve(bs, tol=tol, maxit=200)
    Gm = sp.csr_matrix((G[2], G[1].astype(np.int64), G[0].astype(np.int64)))
    Upm = sp.csr_matrix((Up[2], Up[1].astype(np.int64), Up[0].astype(np.int64)))
    bperm = np.concatenate(bs)[perm]
    for s, A in enumerate(mats):
        a, b = sys_ptr[s], sys_ptr[s + 1]
        Gs = csr_u64(Gm[a:b, a:b].tocsr())
        As = csr_u64(Upm[a:b, a:b].tocsr())
        bs_p = bperm[a:b].copy()
        xo, rro, ito = O.pcg(As, bs_p, tol, 200, Gs)
        x_p = np.concatenate(xs)[perm][a:b]
        if precision == 0:
            assert int(itr[s]) == ito, s
            spread = 0.0
            for th in (8, -8):
                xv, _, _ = O.pcg(As, bs_p, tol, 200, Gs, threads=th)
                spread = max(spread, np.linalg.norm(xv - xo) / np.linalg.norm(xo))
            assert np.linalg.norm(x_p - xo) / np.linalg.norm(xo) < max(1e-12, 4 * spread), s
        else:  # G applied in FP32: same convergence within a few iterations
            assert abs(int(itr[s]) - ito) <= max(2, ito // 10), s
            assert relres[s] <= tol
        # the reported residual is the true one
        true = np.linalg.norm(A @ xs[s] - bs[s]) / np.linalg.norm(bs[s])
        assert abs(true - relres[s]) <= 1e-10, s


@pytest.mark.gpu
def test_batch_autotuned_leaves(cuda, R):
    """threads=0 picks the leaves per system by timing the preconditioner on
    the largest systems; the chosen setting solves every system."""
    from rchol_gb300.batch import autotune_threads

    mats = _systems()
    best, timings = autotune_threads(mats, candidates=(1, 2, 4), sample=3)
    assert best in timings and all(v > 0 for v in timings.values())
    B = R.Batch(mats, threads=0)
    assert B.threads in timings
    rng = np.random.default_rng(2)
    bs = [rng.standard_normal(A.shape[0]) for A in mats]
    xs, relres, itr = B.solve(bs, tol=1e-8, maxit=200)
    for s, A in enumerate(mats):
        assert np.linalg.norm(A @ xs[s] - bs[s]) <= 1.5e-8 * np.linalg.norm(bs[s])
