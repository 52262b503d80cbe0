import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libcrg.so")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle

    pyoracle.build()
    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def gpu():
    """libcrg.so loaded on a machine with a GPU; fails (not skips) if the library is missing."""
    from cellular_raza_gb300 import _native, build

    build.build_library()
    return _native.load()
