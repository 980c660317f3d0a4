"""Translated plans: run one Lik's current step list repeatedly on the GPU.

Thin wrapper over cxgPlanCreate / cxgPlanRun / cxgPlanTime / cxgPlanInfo
(include/cxlik_gpu.h).  The Lik must have been planned (``lik._prep(root)``)
and its CL buffers must stay alive while the Plan exists.
"""
import ctypes


class Plan:
    def __init__(self, lik, precision="fp64"):
        self.lib = lik.lib
        self.lik = lik
        self.h = ctypes.c_void_p()
        code = 1 if precision == "fp32" else 0
        rc = self.lib.cxgPlanCreate(ctypes.byref(lik.lik), code,
                                    ctypes.byref(self.h))
        if rc != 0:
            raise _native.error(self.lib, rc, "cxgPlanCreate")

    def _check(self, rc, what):
        if rc != 0:
            raise _native.error(self.lib, rc, what)

    def run(self):
        out = ctypes.c_double()
        self._check(self.lib.cxgPlanRun(self.h, ctypes.byref(out), None),
                    "cxgPlanRun")
        return out.value

    def time(self, iters):
        ms, kern, lnl = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.cxgPlanTime(self.h, iters, ctypes.byref(ms),
                                         ctypes.byref(kern), ctypes.byref(lnl)),
                    "cxgPlanTime")
        return {"ms_per_run": ms.value, "kernel_ms": kern.value,
                "lnL": lnl.value}

    def info(self):
        up, by = ctypes.c_double(), ctypes.c_double()
        nops, nk = ctypes.c_uint(), ctypes.c_uint()
        self._check(self.lib.cxgPlanInfo(self.h, ctypes.byref(up),
                                         ctypes.byref(by), ctypes.byref(nops),
                                         ctypes.byref(nk)), "cxgPlanInfo")
        return {"updates": up.value, "alg_bytes": by.value,
                "nops": nops.value, "kernels_per_run": nk.value}

    def shape(self):
        t, g, p = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint()
        n, l = ctypes.c_uint(), ctypes.c_uint()
        self._check(self.lib.cxgPlanShape(self.h, ctypes.byref(t),
                                          ctypes.byref(g), ctypes.byref(p),
                                          ctypes.byref(n), ctypes.byref(l)),
                    "cxgPlanShape")
        lanes = ctypes.c_uint()
        self._check(self.lib.cxgPlanLanes(self.h, ctypes.byref(lanes)),
                    "cxgPlanLanes")
        return {"tile": t.value, "threads_per_pattern": g.value,
                "patterns_per_thread": p.value, "nslot": n.value,
                "nleaf": l.value, "lanes": lanes.value}

    def close(self):
        if self.h:
            self.lib.cxgPlanDestroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
