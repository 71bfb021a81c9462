import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the device kernels)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def fgpu_lib():
    from feelpp_gb300 import _ffi
    from feelpp_gb300 import build
    build.build()
    return _ffi.load()


@pytest.fixture(scope="session")
def env(fgpu_lib):
    import feelpp_gb300 as fpp
    e = fpp.Environment(profile=False)
    yield e
