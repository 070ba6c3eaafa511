import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def ctx():
    """A library context on cuda:0 (GPU tests only; fails loudly without a GPU)."""
    from isosurface_gb300 import build as gbuild
    gbuild.build()
    from isosurface_gb300 import Context
    c = Context(0)
    yield c
    c.close()
