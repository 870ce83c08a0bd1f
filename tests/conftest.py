import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and libcuvgls.so")


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def lib():
    from cuvarbase_gb300 import _lib
    from cuvarbase_gb300 import build as B
    B.build()
    return _lib.load()


@pytest.fixture(scope="session")
def handle(lib):
    from cuvarbase_gb300 import _lib
    h = _lib.Handle(sigma=2.0, m=8)
    yield h
    h.close()
