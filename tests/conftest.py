import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# reference path fixtures (tests/golden/make_golden.py); python_order.npz is
# the ordering-only fixture of tests/golden/make_python_order.py
GOLDEN = sorted(p for p in glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz"))
                if not os.path.basename(p).startswith("python_order"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Product library and CPU checkers, built in place."""
    import __graft_entry__

    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def O(built):
    import oracle

    return oracle.Oracle()


@pytest.fixture(scope="session")
def Ref(built):
    import oracle

    if not oracle.Reference.available():
        pytest.skip("reference sources not available on this machine")
    return oracle.Reference()


@pytest.fixture(scope="session")
def R(built):
    import rchol_gb300

    return rchol_gb300


@pytest.fixture(scope="session")
def cuda(built):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def load_golden(path):
    d = np.load(path)
    return {k: d[k] for k in d.files}


def csr_u64(A):
    return (A.indptr.astype(np.uint64), A.indices.astype(np.uint64), A.data.astype(np.float64))
