"""The oracle restatement against the live reference (oracle/_ref, compiled
from the reference's own sources).  Skipped where the sources are absent; the
golden fixtures carry the same pin to other machines."""

import numpy as np
import pytest

import oracle
from rchol_gb300 import generators
from conftest import csr_u64


def _eq(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("n", [4, 7, 11])
@pytest.mark.parametrize("threads", [0, 1, 2, 4, 8])
def test_factor_bit_exact(O, Ref, n, threads):
    A = Ref.laplace_3d(n)
    assert _eq(A, O.laplace_3d(n))
    for seed in (1, 99):
        Gr, Pr = Ref.rchol(A, threads, seed)
        Go, Po, ridx, d = O.rchol(A, threads, seed, oracle.MODE_REF)
        assert np.array_equal(Pr, Po)
        assert _eq(Gr, Go)


@pytest.mark.parametrize("threads", [2, 4, 16])
def test_weighted_and_2d(O, Ref, threads):
    for A in (csr_u64(generators.laplace_3d_weighted(9, sigma=1.0, seed=2)),
              csr_u64(generators.grid_2d_weighted(23, 19, "lognormal", seed=5)),
              csr_u64(generators.checkerboard_3d(10, block=2))):
        pr, rr = Ref.order(A, threads)
        po, ro = O.order(A, threads)
        assert np.array_equal(pr, po) and np.array_equal(rr, ro)
        Ap = Ref.reorder(A, pr)
        assert _eq(Ap, O.reorder(A, po))
        assert _eq(Ref.extend(Ap), O.extend(Ap))
        Gr, _ = Ref.rchol(A, threads, 17)
        Go, _, _, _ = O.rchol(A, threads, 17, oracle.MODE_REF)
        assert _eq(Gr, Go)
        b = np.random.default_rng(3).uniform(-1, 1, len(pr))
        xr, rrr, itr = Ref.pcg(Ap, b, 1e-9, 200, Gr)
        xo, rro, ito = O.pcg(Ap, b, 1e-9, 200, Go)
        assert itr == ito and rrr == rro and np.array_equal(xr, xo)


def test_order_errors_match(O, Ref):
    A = Ref.laplace_3d(2)
    for bad in (3, 6):
        with pytest.raises(ValueError):
            O.order(A, bad)
    with pytest.raises(ValueError, match="too many threads"):
        Ref.order(A, 64)
    with pytest.raises(ValueError, match="too many threads"):
        O.order(A, 64)
