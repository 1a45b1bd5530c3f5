import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libvct.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def vct():
    """The engine's Python mirror; builds libvct.so if needed (GPU tests)."""
    from voxel_cone_tracing_gb300 import build, renderer
    build.build()
    renderer.lib()
    return renderer
