import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 and the built CUDA library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def lib():
    from jetshow_gb300 import _capi, build
    build.build()
    return _capi.load_library()


@pytest.fixture(scope="session")
def ctx(lib):
    from jetshow_gb300.runtime import Context
    c = Context(0)
    yield c
    c.close()
