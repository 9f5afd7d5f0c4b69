import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgbnufft.so")


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built if needed; skips nothing -- GPU tests fail
    loudly when the GPU or the library is missing."""
    import torch

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from mrrt.nufft_gb300 import _build, _lib

    _build.build()
    return _lib.load()
