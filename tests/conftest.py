import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built extension")


def golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library; a GPU test fails (not skips) when it is missing on a GPU machine."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from edelweissfe_gb300 import _lib

    return _lib.lib()
