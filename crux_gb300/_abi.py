"""ctypes mirror of the drop-in structures in include/cxlik_gpu.h.

The layouts are those of the reference's lib/Crux/Tree/CxLik.h:9-273 (built
without CxmMpi), so a ``CxtLik`` filled here can be handed to any library that
exports ``CxLikExecute``: the GPU library, or the CPU oracles used by tests.
"""
import ctypes
from ctypes import (POINTER, Structure, c_bool, c_double, c_int, c_uint,
                    c_uint32, c_void_p)

import numpy as np


class CxtLikCL(Structure):
    pass


class CxtLikModel(Structure):
    pass


CxtLikCL._fields_ = [
    ("cLMat", POINTER(c_double)),
    ("lnScale", POINTER(c_double)),
    ("valid", c_bool),
    ("parent", POINTER(CxtLikCL)),
    ("nSibs", c_uint),
    ("edgeLen", c_double),
]


class CxtLikComp(Structure):
    _fields_ = [
        ("model", POINTER(CxtLikModel)),
        ("weightScaled", c_double),
        ("cweight", c_double),
        ("cmult", c_double),
    ]


CxtLikModel._fields_ = [
    ("decomp", c_bool),
    ("weight", c_double),
    ("qNorm", c_double),
    ("rmult", c_double),
    ("rclass", POINTER(c_uint)),
    ("rTri", POINTER(c_double)),
    ("piDiag", POINTER(c_double)),
    ("piDiagNorm", POINTER(c_double)),
    ("qEigVecCube", POINTER(c_double)),
    ("qEigVals", POINTER(c_double)),
    ("alpha", c_double),
    ("catMedian", c_bool),
    ("invar", c_bool),
    ("comp0", c_uint),
    ("clen", c_uint),
]

# CxeLikStep (CxLik.h:150-155).
ComputeL, ComputeI, MergeL, MergeI = 0, 1, 2, 3


class CxtLikStep(Structure):
    _fields_ = [
        ("variant", c_int),
        ("ntrail", c_uint),
        ("parentCL", POINTER(CxtLikCL)),
        ("childCL", POINTER(CxtLikCL)),
        ("edgeLen", c_double),
    ]


# numpy view of a CxtLikStep array (the planner writes a plan's steps in
# one assignment).
STEP_DTYPE = np.dtype({
    "names": ["variant", "ntrail", "parentCL", "childCL", "edgeLen"],
    "formats": ["<i4", "<u4", "<u8", "<u8", "<f8"],
    "offsets": [CxtLikStep.variant.offset, CxtLikStep.ntrail.offset,
                CxtLikStep.parentCL.offset, CxtLikStep.childCL.offset,
                CxtLikStep.edgeLen.offset],
    "itemsize": ctypes.sizeof(CxtLikStep)})


class CxtLik(Structure):
    _fields_ = [
        ("polarity", c_uint),
        ("dim", c_uint),
        ("rlen", c_uint),
        ("cbase", c_uint),
        ("nchars", c_uint),
        ("mschars", c_uint),
        ("npad", c_uint),
        ("charFreqs", POINTER(c_uint)),
        ("stripeWidth", c_uint),
        ("nstripes", c_uint),
        ("invalidate", c_bool),
        ("resize", c_bool),
        ("reweight", c_bool),
        ("wNorm", c_double),
        ("models", POINTER(POINTER(CxtLikModel))),
        ("modelsLen", c_uint),
        ("modelsMax", c_uint),
        ("comps", POINTER(CxtLikComp)),
        ("compsLen", c_uint),
        ("compsMax", c_uint),
        ("rootCLC", POINTER(CxtLikCL)),
        ("siteLnL", POINTER(c_double)),
        ("stripeLnL", POINTER(c_double)),
        ("steps", POINTER(CxtLikStep)),
        ("stepsLen", c_uint),
        ("stepsMax", c_uint),
    ]


class CxgPlanSnap(Structure):
    """cxgPlanSnap (include/cxlik_gpu.h): one rooted traversal, flattened in
    the planner's post-order, for the native planner cxgPlanSnapRun."""
    _fields_ = [
        ("nvis", c_uint32),
        ("nkid", c_uint32),
        ("cl", c_void_p),
        ("up", c_void_p),
        ("nsibs", c_void_p),
        ("edge", c_void_p),
        ("kid0", c_void_p),
        ("nkids", c_void_p),
        ("kid_cl", c_void_p),
        ("kid_int", c_void_p),
        ("kid_edge", c_void_p),
        ("valid", c_void_p),
        ("cvalid", c_void_p),
        ("m_parent", c_void_p),
        ("m_nsibs", c_void_p),
        ("m_elen", c_void_p),
    ]


def declare_core(lib):
    """Declare the three drop-in entry points on a loaded library."""
    dp = POINTER(c_double)
    lib.CxLikQDecomp.argtypes = [c_int, dp, dp, dp, dp, dp, dp]
    lib.CxLikQDecomp.restype = c_bool
    lib.CxLikPt.argtypes = [c_int, dp, dp, dp, c_double]
    lib.CxLikPt.restype = None
    lib.CxLikExecute.argtypes = [POINTER(CxtLik)]
    lib.CxLikExecute.restype = None
    return lib


def dptr(arr):
    """POINTER(c_double) to the data of a float64 numpy array."""
    return arr.ctypes.data_as(POINTER(c_double))


def uptr(arr):
    """POINTER(c_uint) to the data of a uint32 numpy array."""
    return arr.ctypes.data_as(POINTER(c_uint))


def vptr(arr):
    return c_void_p(arr.ctypes.data)
