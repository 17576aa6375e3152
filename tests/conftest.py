import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libdfm2g.so")


@pytest.fixture(scope="session")
def port():
    """The plain-C oracle (built on demand)."""
    from oracle import port as _port
    return _port()


@pytest.fixture(scope="session")
def built_lib():
    """libdfm2g.so, building it if needed (the CPU suite only loads it)."""
    from delfem2_gb300 import build as B
    B.build()
    from delfem2_gb300 import _native
    return _native.load()


@pytest.fixture(scope="session")
def gpu(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return built_lib


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / den)
