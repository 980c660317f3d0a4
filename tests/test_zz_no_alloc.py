"""cxgLikExecuteNoAlloc: the plan walker for callers that cannot allocate.

Some callers own all device memory themselves. It may come from their own
pool, or from a framework's caching allocator. They may run a
latency-critical loop that must not stall on cudaMalloc. This entry point
takes every buffer from the caller, and its scratch is a fixed array
inside the library.  The test
plays such a caller: it allocates device buffers itself (through the CUDA
runtime, as the caller would), lays out the CLs and leaf masks, and checks
that two calls in a row give the same lnL as the allocating entry point
cxgLikExecuteLnL, within the parity tolerances of the other GPU tests
(1e-11 relative for FP64, 1e-6 for FP32).

This file is collected last, so a run that stops at the first failure has
already run every other test.
"""
import ctypes
import math

import numpy as np
import pytest

from crux_gb300 import _abi, synth

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-11, "fp32": 1e-6}
H2D, D2H = 1, 2


def _cudart():
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            rt = None
    assert rt is not None, "CUDA runtime not found"
    rt.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
    rt.cudaFree.argtypes = [ctypes.c_void_p]
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_size_t, ctypes.c_int]
    rt.cudaMemset.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t]
    return rt


class DeviceArena:
    """The caller's own device allocations."""

    def __init__(self, rt):
        self.rt = rt
        self.ptrs = []

    def alloc(self, nbytes):
        p = ctypes.c_void_p()
        assert self.rt.cudaMalloc(ctypes.byref(p), max(nbytes, 16)) == 0
        assert self.rt.cudaMemset(p, 0, max(nbytes, 16)) == 0
        self.ptrs.append(p)
        return p.value

    def upload(self, arr):
        arr = np.ascontiguousarray(arr)
        p = self.alloc(arr.nbytes)
        assert self.rt.cudaMemcpy(p, arr.ctypes.data, arr.nbytes, H2D) == 0
        return p

    def free(self):
        for p in self.ptrs:
            self.rt.cudaFree(p)
        self.ptrs = []


def device_copy_of_plan(lik, arena, kact, precision):
    """A CxtLik whose CLs are the caller's device buffers.

    Mirrors lik's current plan: each distinct CxtLikCL of the plan gets a
    new struct pointing at device memory -- internal CLs [kact][U][ppad]
    16-byte units plus 8 bytes of scaler per pattern, leaves uint8 masks.
    """
    L = lik.lik
    npat = L.mschars
    ppad = (npat + 127) // 128 * 128
    elt = 4 if precision == "fp32" else 8
    made = {}
    keep = []

    def dev_cl(cl_ptr, leaf):
        key = ctypes.addressof(cl_ptr.contents)
        if key in made:
            return made[key]
        s = _abi.CxtLikCL()
        if leaf:
            host_cl = cl_ptr.contents
            masks = np.full(ppad, 15, dtype=np.uint8)
            owner = None
            for ring_cl in lik._leaf_masks:
                if ring_cl[0] == key:
                    owner = ring_cl[1]
            assert owner is not None
            masks[:npat] = owner
            s.cLMat = ctypes.cast(arena.upload(masks), ctypes.POINTER(ctypes.c_double))
            s.lnScale = None
            del host_cl
        else:
            s.cLMat = ctypes.cast(arena.alloc(kact * 4 * ppad * elt),
                                  ctypes.POINTER(ctypes.c_double))
            s.lnScale = ctypes.cast(arena.alloc(ppad * 8),
                                    ctypes.POINTER(ctypes.c_double))
        made[key] = s
        keep.append(s)
        return s

    steps = (_abi.CxtLikStep * max(L.stepsLen, 1))()
    for i in range(L.stepsLen):
        st = L.steps[i]
        leaf = st.variant in (_abi.ComputeL, _abi.MergeL)
        steps[i].variant = st.variant
        steps[i].ntrail = st.ntrail
        steps[i].edgeLen = st.edgeLen
        steps[i].parentCL = ctypes.pointer(dev_cl(st.parentCL, False))
        steps[i].childCL = ctypes.pointer(dev_cl(st.childCL, leaf))
    d = _abi.CxtLik()
    ctypes.pointer(d)[0] = L
    d.steps = ctypes.cast(steps, ctypes.POINTER(_abi.CxtLikStep))
    d.rootCLC = ctypes.pointer(dev_cl(L.rootCLC, False))
    freqs = arena.upload(np.ascontiguousarray(lik._freqs[:npat]))
    return d, (steps, keep, made), freqs


def leaf_mask_table(lik):
    """(host CxtLikCL address, masks) for every leaf of lik's tree."""
    out = []
    L = lik.lik
    for e in lik.tree.edges:
        for ring in (e.ring, e.ring.other):
            cl = ring.aux
            if cl is not None and cl.leaf:
                ind = lik.alignment.taxaMap.indGet(ring.node.taxon)
                row = lik.alignment.getRow(ind)[:L.mschars]
                vals = lik.char_.val_table[row]
                vals = np.where(vals == 0, lik.char_.any, vals).astype(np.uint8)
                out.append((ctypes.addressof(cl.c[0]), vals))
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_no_alloc_matches_allocating_entry_point(gpu, precision):
    rt = _cudart()
    case = synth.Case(48, 3000, 0.1, 77, pinv=0.0, gap_frac=0.01)
    lik = case.lik(lib=gpu, precision=precision)
    want = lik.lnL()                       # allocating path (cxgLikExecuteLnL)
    # Re-plan the whole tree so every CL is recomputed from leaves.
    lik.lik.invalidate = True
    lik._prep(None)
    lik._leaf_masks = leaf_mask_table(lik)
    kact = sum(1 for i in range(lik.lik.compsLen)
               if lik.lik.comps[i].weightScaled != 0.0)
    arena = DeviceArena(rt)
    try:
        d, keep, freqs = device_copy_of_plan(lik, arena, kact, precision)
        code = 1 if precision == "fp32" else 0
        site = arena.alloc(lik.lik.mschars * 8)
        got = []
        for _ in range(2):                 # two calls in a row
            out = ctypes.c_double()
            rc = gpu.cxgLikExecuteNoAlloc(
                ctypes.byref(d), code,
                ctypes.cast(freqs, ctypes.POINTER(ctypes.c_uint32)),
                ctypes.cast(site, ctypes.POINTER(ctypes.c_double)), None,
                ctypes.byref(out))
            assert rc == 0, gpu.cxgLastError().decode()
            got.append(out.value)
        sites = np.zeros(lik.lik.mschars)
        assert rt.cudaMemcpy(sites.ctypes.data, site, sites.nbytes, D2H) == 0
    finally:
        arena.free()
    for g in got:
        assert math.isfinite(g)
        assert abs(g - want) <= TOL[precision] * abs(want), (g, want)
    want_sites = np.array(lik.siteLnLs())
    n = len(want_sites)
    assert np.all(np.abs(sites[:n] - want_sites) <=
                  TOL[precision] * np.maximum(1.0, np.abs(want_sites)) * 10)


def test_no_alloc_rejects_oversized_plans(gpu):
    case = synth.Case(8, 200, 0.1, 5)
    lik = case.lik(lib=gpu)
    lik.lnL()
    d = _abi.CxtLik()
    ctypes.pointer(d)[0] = lik.lik
    d.mschars = (1 << 20) + 1
    out = ctypes.c_double()
    one = (ctypes.c_uint32 * 1)()
    rc = gpu.cxgLikExecuteNoAlloc(ctypes.byref(d), 0, one, None, None,
                                  ctypes.byref(out))
    assert rc != 0
    assert b"2^20" in gpu.cxgLastError()
