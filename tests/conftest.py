import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")


def gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cuda_lib():
    """Build (if stale) and load the CUDA library; GPU tests only."""
    if not gpu_available():
        pytest.fail("GPU test collected without a CUDA device")
    from tskit_gb300 import _build, _native

    _build.build_all()
    return _native.load()


@pytest.fixture(scope="session")
def cuda_lib_cpu():
    """Build (if stale) and load the library for host-only calls (no GPU
    needed: file reading, error strings)."""
    from tskit_gb300 import _build, _native

    _build.build_all()
    return _native.load()
