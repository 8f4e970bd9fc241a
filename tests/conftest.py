import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and libb2r.so")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def orc():
    from oracle import orc as o
    o.lib()
    return o


@pytest.fixture(scope="session")
def b2r():
    """The product package; on a machine with a GPU the library must load (no
    fallback).  A fresh checkout compiles it (and the host program) first."""
    import b2r_gb300
    from b2r_gb300 import build as pkg_build
    if not os.path.exists(b2r_gb300.LIB_PATH) or not os.path.exists(pkg_build.MAIN):
        pkg_build.build()
    b2r_gb300.lib()
    return b2r_gb300
