"""ORACLE TEST INFRASTRUCTURE -- not part of the product.

Loaders for the two CPU oracles that export the reference's C entry points
(CxLikQDecomp, CxLikPt, CxLikExecute) over the struct ABI of
include/cxlik_gpu.h:

* ``load_ref()``: oracle/_ref/libcxlik_ref.so, the reference's own
  lib/Crux/Tree/CxLik.c built unchanged by ``make -C oracle ref``.  Its
  LAPACK calls (CxLik.c:194-226) are routed to scipy's cython_lapack.
  Present only where the reference tree was available at build time.
* ``load_port()``: oracle/_build/libcxlik_port.so, this repository's C
  restatement (oracle/cxlik_port.c), built by ``make -C oracle port``.
* ``load_best()``: the reference build when present, else the port.
"""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SO = os.path.join(HERE, "_ref", "libcxlik_ref.so")
PORT_SO = os.path.join(HERE, "_build", "libcxlik_port.so")
STAGED = os.path.join(HERE, "_ref", "src", "lib", "Crux", "Tree", "CxLik.c")

_cache = {}


def build(ref_tree=None):
    """Build the port, and the reference core when its sources exist: from
    `ref_tree` (or $CRUX_REF), a crux source tree, which also stages the
    files under oracle/_ref/src; else from a staged copy made earlier."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    ref_tree = ref_tree or os.environ.get("CRUX_REF")
    if ref_tree and os.path.isdir(os.path.join(ref_tree, "lib", "Crux", "Tree")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + ref_tree],
                       check=True)
    elif os.path.exists(STAGED):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF="], check=True)


def _capsule_pointer(capsule):
    get_name = ctypes.pythonapi.PyCapsule_GetName
    get_name.restype = ctypes.c_char_p
    get_name.argtypes = [ctypes.py_object]
    get_ptr = ctypes.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = ctypes.c_void_p
    get_ptr.argtypes = [ctypes.py_object, ctypes.c_char_p]
    return get_ptr(capsule, get_name(capsule))


def _declare(lib):
    from crux_gb300 import _abi
    _abi.declare_core(lib)
    return lib


def load_ref():
    """The reference's own CxLik.c core, or None if it was not built."""
    if "ref" in _cache:
        return _cache["ref"]
    lib = None
    if os.path.exists(REF_SO):
        lib = ctypes.CDLL(REF_SO, mode=ctypes.RTLD_LOCAL)
        from scipy.linalg import cython_lapack
        caps = cython_lapack.__pyx_capi__
        lib.oracle_set_lapack.argtypes = [ctypes.c_void_p] * 3
        lib.oracle_set_lapack(_capsule_pointer(caps["dgeev"]),
                              _capsule_pointer(caps["dgetrf"]),
                              _capsule_pointer(caps["dgetri"]))
        lib.CxThreaded.argtypes = []
        lib.CxThreaded.restype = None
        lib.kind = "reference"
        lib.plan_natively = False
        _declare(lib)
    _cache["ref"] = lib
    return lib


def ref_threaded(lib):
    """Enable the reference's pthread stripe pool (Cx.c:63-66)."""
    lib.CxThreaded()


def ref_ncpus(lib):
    return ctypes.c_uint.in_dll(lib, "CxNcpus").value


def load_port():
    if "port" in _cache:
        return _cache["port"]
    if not os.path.exists(PORT_SO):
        subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    lib = ctypes.CDLL(PORT_SO, mode=ctypes.RTLD_LOCAL)
    lib.port_set_threads.argtypes = [ctypes.c_int]
    lib.port_set_threads.restype = None
    lib.port_get_threads.argtypes = []
    lib.port_get_threads.restype = ctypes.c_int
    lib.kind = "port"
    lib.plan_natively = False
    _declare(lib)
    _cache["port"] = lib
    return lib


def load_best():
    return load_ref() or load_port()
