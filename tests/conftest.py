import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN


@pytest.fixture(scope="session")
def rbrp_lib():
    """The built CUDA library (built in-tree on first use when missing)."""
    from robust_blockwise_random_pivoting_gb300 import _lib, build
    import os
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.load()


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
