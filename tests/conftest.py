import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "weno-cfd-solver_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); run with -m gpu")


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def golden_twin():
    import numpy as np
    return np.load(os.path.join(GOLDEN, "twin_cons_hlle.npz"))


@pytest.fixture(scope="session")
def golden_drivers():
    import numpy as np
    return np.load(os.path.join(GOLDEN, "drivers.npz"))


@pytest.fixture(scope="session")
def wx():
    """The product module, with its CUDA library built; skips nothing -- GPU tests
    must fail loudly if the library cannot be built or loaded."""
    import weno_ext
    from weno_ext import _lib
    _lib.load()
    return weno_ext
