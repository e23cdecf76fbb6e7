import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native_lib():
    """The library, built if needed (no GPU is touched by loading it)."""
    from cosma_gb300 import build
    build.build()
    from cosma_gb300 import _native
    return _native.load()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def colmajor(t):
    """Column-major view helper: a (rows x cols) torch tensor with stride(0) == 1."""
    return t.t().contiguous().t()


@pytest.fixture
def rng():
    import numpy as np
    return np.random.default_rng(int(os.environ.get("COSMA_TEST_SEED", "1234")))
