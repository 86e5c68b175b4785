import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device")


@pytest.fixture(scope="session")
def built_lib():
    """Build (if needed) and load the CUDA library."""
    from dynamix_gb300 import build
    build.build(force=False)
    from dynamix_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def cuda_device():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name + ".npz"))
