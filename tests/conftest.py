import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path")
    config.addinivalue_line("markers", "slow: long-running parity case")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load libphafd_gpu.so; GPU tests fail loudly without it."""
    from phafd_gb300 import build as B
    B.build()
    from phafd_gb300 import gpu
    return gpu.load()
