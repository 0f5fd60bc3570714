import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def native():
    """libfasttau.so, built in-tree (nvcc cross-compiles without a GPU)."""
    from fast_gb300 import build
    build.build()
    from fast_gb300 import _native
    return _native.lib()


@pytest.fixture(scope="session")
def gpu(native):
    if not has_gpu():
        pytest.fail("this test needs a CUDA GPU")
    return native
