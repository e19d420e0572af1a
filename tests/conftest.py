import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def port_lib():
    from oracle import oracle
    assert oracle.build_port(), "oracle port failed to build"
    return oracle


@pytest.fixture(scope="session")
def ref_lib():
    from oracle import oracle
    if not oracle.ref_available():
        pytest.skip("reference Box2D checkout not present on this machine")
    assert oracle.build_ref(), "reference library failed to build"
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    import __graft_entry__ as g
    from forge2d_gb300 import build
    build()
    from forge2d_gb300 import native
    return native.load()
