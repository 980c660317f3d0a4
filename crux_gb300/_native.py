"""Loader for the GB300 library (crux_gb300/_lib/libcxlik_gpu.so).

There is no CPU fallback: if the library is missing or no GPU is present the
load raises, so a likelihood is never computed silently elsewhere.
"""
import ctypes
import os

from . import _abi

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib",
                        "libcxlik_gpu.so")
_lib = None


class NativeUnavailable(RuntimeError):
    pass


CXG_ENOMEM = -2
CXG_ETIMEOUT = -4


class DeviceTimeout(RuntimeError):
    """A bounded device wait gave up (CXG_ETIMEOUT)."""


def error(lib, rc, what):
    """The exception for return code `rc` of the library call `what`:
    MemoryError for CXG_ENOMEM (the reference raises MemoryError when an
    allocation fails, Lik.pyx:66-84), DeviceTimeout for CXG_ETIMEOUT,
    RuntimeError otherwise."""
    msg = "%s: %s" % (what, lib.cxgLastError().decode(errors="replace"))
    if rc == CXG_ENOMEM:
        return MemoryError(msg)
    if rc == CXG_ETIMEOUT:
        return DeviceTimeout(msg)
    return RuntimeError(msg)


def declare(lib):
    """Declare every entry point of include/cxlik_gpu.h on `lib`."""
    _abi.declare_core(lib)
    P = ctypes.POINTER
    c_int, c_uint, c_double = ctypes.c_int, ctypes.c_uint, ctypes.c_double
    lib.cxgLastError.argtypes = []
    lib.cxgLastError.restype = ctypes.c_char_p
    lib.cxgInfo.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    lib.cxgInfo.restype = c_int
    lib.cxgLikClSetLeafMasks.argtypes = [P(_abi.CxtLikCL), P(ctypes.c_uint8),
                                         c_uint]
    lib.cxgLikClSetLeafMasks.restype = c_int
    lib.cxgLikClForget.argtypes = [P(c_double)]
    lib.cxgLikClForget.restype = c_int
    lib.cxgLikReset.argtypes = []
    lib.cxgLikReset.restype = c_int
    lib.cxgLikSetPatternWeights.argtypes = [P(c_uint), c_uint]
    lib.cxgLikSetPatternWeights.restype = c_int
    lib.cxgLikForgetPatternWeights.argtypes = [P(c_uint), c_uint]
    lib.cxgLikForgetPatternWeights.restype = c_int
    lib.cxgLikExecuteLnL.argtypes = [P(_abi.CxtLik), c_int, P(c_double),
                                     P(c_double)]
    lib.cxgLikExecuteLnL.restype = c_int
    lib.cxgLikLastIo.argtypes = [P(ctypes.c_size_t), P(ctypes.c_size_t)]
    lib.cxgLikLastIo.restype = c_int
    lib.cxgLikDeviceBytes.argtypes = [P(ctypes.c_size_t)]
    lib.cxgLikDeviceBytes.restype = c_int
    vp = ctypes.c_void_p
    lib.cxgPlanCreate.argtypes = [P(_abi.CxtLik), c_int, P(vp)]
    lib.cxgPlanCreate.restype = c_int
    lib.cxgPlanRun.argtypes = [vp, P(c_double), P(c_double)]
    lib.cxgPlanRun.restype = c_int
    lib.cxgPlanTime.argtypes = [vp, c_int, P(c_double), P(c_double),
                                P(c_double)]
    lib.cxgPlanTime.restype = c_int
    lib.cxgPlanInfo.argtypes = [vp, P(c_double), P(c_double), P(c_uint),
                                P(c_uint)]
    lib.cxgPlanInfo.restype = c_int
    lib.cxgPlanDestroy.argtypes = [vp]
    lib.cxgPlanDestroy.restype = c_int
    lib.cxgPlanShape.argtypes = [vp, P(c_uint), P(c_uint), P(c_uint), P(c_uint),
                                 P(c_uint)]
    lib.cxgPlanShape.restype = c_int
    u32p = P(ctypes.c_uint32)
    lib.cxgPlanSnapRun.argtypes = [P(_abi.CxgPlanSnap), P(c_double), c_int,
                                   vp, ctypes.c_uint32, u32p, u32p, u32p]
    lib.cxgPlanSnapRun.restype = c_int
    lib.cxgTune.argtypes = [c_uint, c_uint, c_uint, ctypes.c_size_t]
    lib.cxgTune.restype = c_int
    lib.cxgTuneGet.argtypes = [P(c_uint), P(c_uint), P(c_uint),
                               P(ctypes.c_size_t)]
    lib.cxgTuneGet.restype = c_int
    lib.cxgTuneLanes.argtypes = [c_uint]
    lib.cxgTuneLanes.restype = c_int
    lib.cxgTuneLanesGet.argtypes = [P(c_uint)]
    lib.cxgTuneLanesGet.restype = c_int
    lib.cxgPlanLanes.argtypes = [vp, P(c_uint)]
    lib.cxgPlanLanes.restype = c_int
    lib.cxgLikExecuteNoAlloc.argtypes = [P(_abi.CxtLik), c_int,
                                         P(ctypes.c_uint32), P(c_double),
                                         vp, P(c_double)]
    lib.cxgLikExecuteNoAlloc.restype = c_int
    lib.cxgBatchCreate.argtypes = [P(P(_abi.CxtLik)), c_uint, c_int, c_uint,
                                   P(vp)]
    lib.cxgBatchCreate.restype = c_int
    lib.cxgBatchRun.argtypes = [vp, P(c_double)]
    lib.cxgBatchRun.restype = c_int
    lib.cxgBatchTime.argtypes = [vp, c_int, P(c_double), P(c_double)]
    lib.cxgBatchTime.restype = c_int
    lib.cxgBatchInfo.argtypes = [vp, P(c_double), P(c_double), P(c_uint),
                                 P(c_uint), P(ctypes.c_ulonglong)]
    lib.cxgBatchInfo.restype = c_int
    lib.cxgBatchDestroy.argtypes = [vp]
    lib.cxgBatchDestroy.restype = c_int
    lib.cxgDebugSetSpinLimit.argtypes = [c_uint, P(c_uint)]
    lib.cxgDebugSetSpinLimit.restype = c_int
    lib.cxgDebugFailAllocs.argtypes = [ctypes.c_longlong]
    lib.cxgDebugFailAllocs.restype = c_int
    lib.cxgDebugCanaries.argtypes = [c_int]
    lib.cxgDebugCanaries.restype = c_int
    lib.cxgDebugCheckCanaries.argtypes = [P(ctypes.c_ulonglong),
                                          P(ctypes.c_ulonglong)]
    lib.cxgDebugCheckCanaries.restype = c_int
    lib.cxgDebugCanarySelfTest.argtypes = [P(c_int)]
    lib.cxgDebugCanarySelfTest.restype = c_int
    return lib


def load(path=LIB_PATH):
    """Load and declare the library; raise NativeUnavailable if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise NativeUnavailable(
            "%s is missing: build it with `python -m crux_gb300.build`" % path)
    lib = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
    declare(lib)
    _lib = lib
    return lib


def last_error(lib=None):
    lib = lib or load()
    return lib.cxgLastError().decode(errors="replace")
