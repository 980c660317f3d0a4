import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def pytest_configure(config):
    config.addinivalue_line("markers",
                            "gpu: needs a GB300 and the built CUDA library")


@pytest.fixture(scope="session")
def port():
    from oracle import oracle
    return oracle.load_port()


@pytest.fixture(scope="session")
def ref():
    from oracle import oracle
    lib = oracle.load_ref()
    if lib is None:
        pytest.skip("reference core not built here (no reference tree)")
    return lib


@pytest.fixture(scope="session", params=["ref", "port"])
def oracle_lib(request):
    from oracle import oracle
    lib = oracle.load_ref() if request.param == "ref" else oracle.load_port()
    if lib is None:
        pytest.skip("reference core not built here")
    return lib


@pytest.fixture(scope="session")
def gpu():
    """The GB300 library; fails (does not skip) when it cannot load."""
    from crux_gb300 import _native
    lib = _native.load()
    import ctypes
    buf = ctypes.create_string_buffer(256)
    lib.cxgInfo(buf, 256)
    assert b"no device" not in buf.value, buf.value
    return lib
