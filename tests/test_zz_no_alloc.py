"""cxgLikExecuteNoAlloc: the plan walker for callers that cannot allocate.

Some callers own all device memory themselves. It may come from their own
pool, or from a framework's caching allocator. They may run a
latency-critical loop that must not stall on cudaMalloc. This entry point
takes every buffer from the caller, and its scratch is a fixed array
inside the library.  The tests play such a caller: they allocate device
buffers themselves (through the CUDA runtime, as the caller would), lay out
the CLs and leaf masks, and check that two calls in a row give the same
lnL as the allocating entry point cxgLikExecuteLnL and as the FP64 oracle,
within the parity tolerances of the other GPU tests (1e-11 relative for
FP64, 1e-6 for FP32): on a binary tree, and on a tree with degree-4 and
degree-5 nodes walked with shared-memory stack slots.  A record wait that
gives up returns CXG_ETIMEOUT, and malformed or oversized plans are
rejected on the host before anything is launched.

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


def run_no_alloc(gpu, lik, precision, calls=2):
    """Re-plan `lik` in full and evaluate it `calls` times through
    cxgLikExecuteNoAlloc on buffers this test allocates.  Returns the
    return codes, the lnLs and the site lnLs of the last call."""
    rt = _cudart()
    lik.lik.invalidate = True
    lik._prep(None)
    lik._leaf_masks = leaf_mask_table(lik)
    kact = sum(1 for i in range(lik.lik.compsLen)
               if lik.lik.comps[i].weightScaled != 0.0)
    arena = DeviceArena(rt)
    rcs, got = [], []
    try:
        d, keep, freqs = device_copy_of_plan(lik, arena, kact, precision)
        code = 1 if precision == "fp32" else 0
        site = arena.alloc(lik.lik.mschars * 8)
        for _ in range(calls):
            out = ctypes.c_double()
            rcs.append(gpu.cxgLikExecuteNoAlloc(
                ctypes.byref(d), code,
                ctypes.cast(freqs, ctypes.POINTER(ctypes.c_uint32)),
                ctypes.cast(site, ctypes.POINTER(ctypes.c_double)), None,
                ctypes.byref(out)))
            got.append(out.value)
        sites = np.zeros(lik.lik.mschars)
        assert rt.cudaMemcpy(sites.ctypes.data, site, sites.nbytes, D2H) == 0
    finally:
        arena.free()
    return rcs, got, sites


def check(gpu, lik, want_oracle, precision):
    # The allocating path (cxgLikExecuteLnL), every CL recomputed: a plan
    # made for the no-allocation call marks CLs valid without computing
    # them on the allocating path.
    lik.lik.invalidate = True
    want = lik.lnL()
    rcs, got, sites = run_no_alloc(gpu, lik, precision)
    assert rcs == [0, 0], gpu.cxgLastError().decode()
    for g in got:
        assert math.isfinite(g)
        assert abs(g - want) <= TOL[precision] * abs(want), (g, want)
        assert abs(g - want_oracle) <= TOL[precision] * abs(want_oracle), \
            (g, want_oracle)
    want_sites = np.array(lik.siteLnLs())
    n = len(want_sites)
    assert np.all(np.abs(sites[:n] - want_sites) <=
                  TOL[precision] * np.maximum(1.0, np.abs(want_sites)) * 10)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_no_alloc_matches_allocating_entry_point(gpu, port, precision):
    case = synth.Case(48, 3000, 0.1, 77, pinv=0.0, gap_frac=0.01)
    check(gpu, case.lik(lib=gpu, precision=precision),
          case.lik(lib=port).lnL(), precision)


class tuned:
    """Context: a walker launch shape for plans translated meanwhile."""

    def __init__(self, lib, tile, budget):
        self.lib, self.tile, self.budget = lib, tile, budget

    def __enter__(self):
        t, g, p, b = (ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint(),
                      ctypes.c_size_t())
        self.lib.cxgTuneGet(ctypes.byref(t), ctypes.byref(g), ctypes.byref(p),
                            ctypes.byref(b))
        self.old = (t.value, g.value, p.value, b.value)
        assert self.lib.cxgTune(self.tile, 1, 1, self.budget) == 0
        return self

    def __exit__(self, *exc):
        assert self.lib.cxgTune(*self.old) == 0
        return False


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_no_alloc_polytomies_with_stack_slots(gpu, port, precision):
    """Degree-4 and degree-5 nodes (Merge steps with ntrail counting down)
    and results kept in shared-memory stack slots between ops (a stack
    budget of 48 KiB), with +I (five components) and gaps."""
    import kat_cases as K
    from crux_gb300.alignment import Alignment, CTMatrix
    from crux_gb300.lik import Lik
    rng = np.random.default_rng(81)
    names = ["t%d" % i for i in range(11)]
    fasta = "".join(">%s\n%s\n" % (n, "".join(rng.choice(list("ACGTACGTN-"),
                                                          2500)))
                    for n in names)
    newick = ("(t0:0.1,t1:0.2,(t2:0.1,t3:0.3,t4:0.05,t5:0.2):0.15,"
              "(t6:0.1,t7:0.2,t8:0.3):0.1,(t9:0.05,t10:0.4):0.2);")
    aln = Alignment(CTMatrix(fasta))
    aln.compact()

    def make(lib, prec="fp64"):
        lk = Lik(K.tree_for(newick, aln), aln, ncat=4, invar=True, lib=lib,
                 precision=prec)
        lk.setAlpha(0, 0.6)
        lk.setWVar(0, 0.75)
        lk.setWInvar(0, 0.25)
        return lk

    lg = make(gpu, precision)
    assert max(n.getDegree() for n in lg.tree.nodes) >= 5
    with tuned(gpu, 64, 48 << 10):
        check(gpu, lg, make(port).lnL(), precision)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_no_alloc_wait_that_gives_up(gpu, port, precision):
    """With every record wait set to give up at once the call returns
    CXG_ETIMEOUT (-4); with the default bound back, the next calls match."""
    case = synth.Case(20, 1500, 0.1, 78)
    lik = case.lik(lib=gpu, precision=precision)
    prev = ctypes.c_uint()
    assert gpu.cxgDebugSetSpinLimit(0, ctypes.byref(prev)) == 0
    try:
        rcs, _, _ = run_no_alloc(gpu, lik, precision, calls=1)
    finally:
        assert gpu.cxgDebugSetSpinLimit(prev.value, None) == 0
    assert rcs == [-4]
    check(gpu, lik, case.lik(lib=port).lnL(), precision)


def _fake_plan(steps_spec, ncomps=1, mschars=100, leaf_addr=0x10000):
    """A CxtLik whose CL pointers are dummies (never dereferenced: every
    case below is rejected on the host before anything is launched).
    `steps_spec`: (variant, ntrail, parent index, child index) tuples."""
    keep = []
    cls = []
    for i in range(64):
        c = _abi.CxtLikCL()
        c.cLMat = ctypes.cast(ctypes.c_void_p(0x100000 + 0x1000 * i),
                              ctypes.POINTER(ctypes.c_double))
        c.lnScale = ctypes.cast(ctypes.c_void_p(0x800000 + 0x1000 * i),
                                ctypes.POINTER(ctypes.c_double))
        cls.append(c)
    leaf = _abi.CxtLikCL()
    leaf.cLMat = ctypes.cast(ctypes.c_void_p(leaf_addr),
                             ctypes.POINTER(ctypes.c_double))
    model = _abi.CxtLikModel()
    comps = (_abi.CxtLikComp * ncomps)()
    for k in range(ncomps):
        comps[k].model = ctypes.pointer(model)
        comps[k].weightScaled = 1.0 / ncomps
        comps[k].cmult = 1.0
    steps = (_abi.CxtLikStep * max(1, len(steps_spec)))()
    for i, (v, nt, par, ch) in enumerate(steps_spec):
        steps[i].variant = v
        steps[i].ntrail = nt
        steps[i].parentCL = ctypes.pointer(cls[par])
        steps[i].childCL = ctypes.pointer(leaf if ch < 0 else cls[ch])
        steps[i].edgeLen = 0.1
    d = _abi.CxtLik()
    d.dim = 4
    d.mschars = mschars
    d.comps = comps
    d.compsLen = ncomps
    d.steps = ctypes.cast(steps, ctypes.POINTER(_abi.CxtLikStep))
    d.stepsLen = len(steps_spec)
    d.rootCLC = ctypes.pointer(cls[0])
    keep += [cls, leaf, model, comps, steps]
    return d, keep


def _reject(gpu, d, precision=0):
    out = ctypes.c_double()
    one = ctypes.cast(ctypes.c_void_p(0x200000), ctypes.POINTER(ctypes.c_uint32))
    rc = gpu.cxgLikExecuteNoAlloc(ctypes.byref(d), precision, one, None, None,
                                  ctypes.byref(out))
    assert rc == -1, rc                    # CXG_EINVAL
    return gpu.cxgLastError().decode()


def test_no_alloc_rejects_malformed_plans(gpu):
    C, CI, M, MI = _abi.ComputeL, _abi.ComputeI, _abi.MergeL, _abi.MergeI
    # A Merge step with no Compute step before it.
    d, k = _fake_plan([(M, 0, 1, -1)])
    assert "Merge" in _reject(gpu, d)
    # A Merge step of another parent, and an ntrail that does not count down.
    d, k = _fake_plan([(C, 1, 1, -1), (M, 0, 2, -1)])
    assert "Merge" in _reject(gpu, d)
    d, k = _fake_plan([(C, 2, 1, -1), (M, 0, 1, -1)])
    assert "Merge" in _reject(gpu, d)
    # A plan that ends in the middle of a node, and a Compute step there.
    d, k = _fake_plan([(C, 1, 1, -1)])
    assert "mid-node" in _reject(gpu, d)
    d, k = _fake_plan([(C, 1, 1, -1), (CI, 0, 2, 3)])
    assert "Compute" in _reject(gpu, d)
    # More than 8 active components.
    d, k = _fake_plan([(C, 0, 1, -1)], ncomps=9)
    assert "8 active" in _reject(gpu, d)
    # A leaf mask array that is not 16-byte aligned.
    d, k = _fake_plan([(C, 1, 1, -1), (M, 0, 1, -1)], leaf_addr=0x10008)
    assert "aligned" in _reject(gpu, d)


def test_no_alloc_rejects_plans_beyond_its_limits(gpu):
    C, CI, MI = _abi.ComputeL, _abi.ComputeI, _abi.MergeI
    # More than 1024 node updates.
    spec = [(C, 0, 1 + (i % 60), -1) for i in range(1025)]
    d, k = _fake_plan(spec)
    assert "1024" in _reject(gpu, d)
    # More than 2048 children (1000 ops of three).
    spec = []
    for i in range(1000):
        p = 1 + (i % 60)
        spec += [(CI, 2, p, 2), (MI, 1, p, 3), (MI, 0, p, 4)]
    d, k = _fake_plan(spec)
    assert "2048" in _reject(gpu, d)
    # A node of degree 17.
    spec = [(CI if j == 0 else MI, 16 - j, 1, 2 + j) for j in range(17)]
    d, k = _fake_plan(spec)
    assert "16" in _reject(gpu, d)
    # Op records above their 1.5 MiB budget: FP64, eight components, 750
    # binary ops of 32 + 2 x (32 + 8 x 128) bytes each.
    spec = []
    for i in range(750):
        p = 1 + (i % 60)
        spec += [(CI, 1, p, 2), (MI, 0, p, 3)]
    d, k = _fake_plan(spec, ncomps=8)
    assert "1.5 MiB" in _reject(gpu, d)


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
