"""Batches: many likelihoods evaluated by one persistent GPU launch.

Wrapper over cxgBatchCreate / cxgBatchRun / cxgBatchTime / cxgBatchInfo
(include/cxlik_gpu.h).  Each Lik contributes its current plan; call
``lik.prepare_plan()`` (a full or dirty-path plan) before building the
batch.  All Liks must use the same number of active mixture components.
"""
import ctypes

import numpy as np

from . import _abi, _native

PER_NODE = 1


class Batch:
    def __init__(self, liks, precision="fp32", per_node=False):
        self.liks = list(liks)
        self.lib = self.liks[0].lib
        arr = (ctypes.POINTER(_abi.CxtLik) * len(self.liks))()
        for i, lk in enumerate(self.liks):
            arr[i] = ctypes.pointer(lk.lik)
        self.h = ctypes.c_void_p()
        code = 1 if precision == "fp32" else 0
        rc = self.lib.cxgBatchCreate(arr, len(self.liks), code,
                                     PER_NODE if per_node else 0,
                                     ctypes.byref(self.h))
        if rc != 0:
            raise _native.error(self.lib, rc, "cxgBatchCreate")

    def _check(self, rc, what):
        if rc != 0:
            raise _native.error(self.lib, rc, what)

    def run(self):
        out = np.zeros(len(self.liks))
        self._check(self.lib.cxgBatchRun(self.h, _abi.dptr(out)),
                    "cxgBatchRun")
        return out

    def time(self, iters):
        ms, walk = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.cxgBatchTime(self.h, iters, ctypes.byref(ms),
                                          ctypes.byref(walk)), "cxgBatchTime")
        return {"ms_per_run": ms.value, "walk_ms": walk.value}

    def info(self):
        up, by = ctypes.c_double(), ctypes.c_double()
        ni, gr, la = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        self._check(self.lib.cxgBatchInfo(self.h, ctypes.byref(up),
                                          ctypes.byref(by), ctypes.byref(ni),
                                          ctypes.byref(gr), ctypes.byref(la)),
                    "cxgBatchInfo")
        return {"updates": up.value, "alg_bytes": by.value,
                "items": ni.value, "grid": gr.value,
                "launches_per_run": la.value}

    def close(self):
        if self.h:
            self.lib.cxgBatchDestroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
