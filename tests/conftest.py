import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgategpu.so")


@pytest.fixture(scope="session")
def built_lib():
    """Builds libgategpu.so once per session (nvcc, sm_103a)."""
    from opengate_gb300 import build

    return build.build()
