import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def native_lib():
    from polyred_gb300 import _abi, build, native
    build.build()
    return _abi.bind_testing(native.load())


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    return oracle.load()


@pytest.fixture(scope="session")
def device(native_lib):
    from polyred_gb300 import render
    d = render.Device(0)
    yield d
    d.close()
