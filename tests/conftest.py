"""Shared fixtures. GPU tests are marked ``gpu`` and run on a GB300; everything else runs on CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libarc_trace.so")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on CPU")


@pytest.fixture(scope="session")
def orc():
    from oracle import pyorc

    pyorc.build()
    return pyorc


@pytest.fixture(scope="session")
def native_lib():
    from arcadia_gb300 import build, native

    build.build()
    return native


_worlds = {}


@pytest.fixture(scope="session")
def world_cache(orc):
    """Oracle-built worlds by scene name (built once per session)."""
    from arcadia_gb300.layout import SCENES

    def get(name):
        if name not in _worlds:
            _worlds[name] = orc.build_world(SCENES[name])
        return _worlds[name]

    return get
