import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the engine through the C ABI")


@pytest.fixture(scope="session")
def built_lib():
    """Builds libltpg.so (nvcc cross-compiles without a GPU) and the oracle."""
    from ltpg_gb300 import build as b
    import oracle
    path = b.build()
    oracle.build()
    return path


def _gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu(built_lib):
    if not _gpu_available():
        pytest.skip("no CUDA device")
    return 0
