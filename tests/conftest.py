import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library; building it is part of the test run."""
    from edxraster_gb300 import build
    build.build()
    from edxraster_gb300 import _lib
    return _lib.load()
