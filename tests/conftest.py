import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and runs the device kernels")


@pytest.fixture(scope="session")
def mblib():
    """The product library, built in-tree if missing."""
    from mandelbulber_gb300 import _build, library
    _build.build()
    return library()


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle (test infrastructure), built by oracle/Makefile if missing."""
    from tests import oracle_lib
    return oracle_lib.load()


@pytest.fixture(scope="session")
def gpu_ctx(mblib):
    import mandelbulber_gb300 as mb
    ctx = mb.Context(0)
    yield ctx
    ctx.close()
