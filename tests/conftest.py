import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def built_lib():
    """Builds (if needed) and returns the path of libppmpa_gb300.so."""
    from ppmpa_gb300 import build as lib_build
    return lib_build.build()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import binding
    return binding.lib()
