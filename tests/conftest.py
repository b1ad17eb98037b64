import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads the CUDA library; GPU tests only."""
    from fringe_gb300 import build, _lib
    build.build()
    return _lib.load()
