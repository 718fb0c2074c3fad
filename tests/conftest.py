import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built engine library")


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle library (built on demand)."""
    import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def engine():
    """The engine library (built on demand): GPU tests, and CPU tests of its host-only entry
    points (file formats, box scalers)."""
    from rampack_gb300 import build as _build
    _build.build()
    from rampack_gb300 import _lib
    _lib.load()
    return _lib
