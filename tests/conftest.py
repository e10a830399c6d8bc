import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libmbe.so")


@pytest.fixture(scope="session")
def built():
    """Builds libmbe.so (nvcc cross-compiles without a GPU) and the oracle."""
    from cumbe_gb300 import build as b
    import oracle
    b.build()
    oracle.build()
    return True


@pytest.fixture(scope="session")
def engine(built):
    import cumbe_gb300 as cm
    e = cm.Engine(0)
    yield e
    e.close()


def random_csr(rng, nr, nc, p):
    M = rng.random((nr, nc)) < p
    rp = np.zeros(nr + 1, np.uint64)
    rp[1:] = np.cumsum(M.sum(1))
    return nr, nc, rp, np.nonzero(M)[1].astype(np.uint32)
