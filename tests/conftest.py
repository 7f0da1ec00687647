import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built native library")


@pytest.fixture(scope="session")
def native_lib():
    """The built product library (built on demand; the GPU tests need it)."""
    from calchem_gb300 import _native

    return _native.load(build_if_missing=True)


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.lib()
    return O
