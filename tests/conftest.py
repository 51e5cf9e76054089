import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libnpgpu.so")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads libnpgpu.so; GPU tests fail loudly without it."""
    from nphysics_gb300 import build
    build.build()
    from nphysics_gb300 import world
    return world.lib()
