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
    """The GB300 library; fails (does not skip) when it cannot load.  Every
    device allocation it makes in the tests carries a canary (see
    canaries_intact)."""
    from crux_gb300 import _native
    lib = _native.load()
    import ctypes
    buf = ctypes.create_string_buffer(256)
    lib.cxgInfo(buf, 256)
    assert b"no device" not in buf.value, buf.value
    assert lib.cxgDebugCanaries(1) == 0
    return lib


@pytest.fixture(autouse=True)
def canaries_intact(request):
    """After every GPU test: no kernel wrote past the end of a library
    allocation (each carries a 256-byte canary, read back here and at every
    synchronous free).  A memory checker may not run on the GPUs."""
    yield
    if request.node.get_closest_marker("gpu") is None or \
            "gpu" not in request.fixturenames:
        return
    import ctypes
    lib = request.getfixturevalue("gpu")
    checked, bad = ctypes.c_ulonglong(), ctypes.c_ulonglong()
    assert lib.cxgDebugCheckCanaries(ctypes.byref(checked),
                                     ctypes.byref(bad)) == 0
    assert bad.value == 0, "%d of %d canaries overwritten" % (bad.value,
                                                              checked.value)
