import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build libopflow_gpu.so (cross-compiles without a GPU) and the oracle once per session."""
    from opflow_gb300 import build
    build.build()
    import oracle_lib
    oracle_lib.lib()
    yield


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def ctx():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from opflow_gb300 import default_context
    return default_context(0)
