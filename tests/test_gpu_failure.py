"""Failure paths on the GPU, made without faulting it.

* Bounded waits: cxgDebugSetSpinLimit(0) makes every op-record wait of the
  plan walkers give up at its first check.  The walker then drains the
  copies it has in flight and sets the run's error word; the call returns
  CXG_ETIMEOUT (DeviceTimeout in Python), and the next call, with the
  default bound back, recomputes the CLs and matches the FP64 oracle.  This
  covers the single-plan entry point, the batched walker, MC3 and the
  server.
* Allocation failure: cxgDebugFailAllocs(k) lets k more allocations of the
  library succeed and fails the rest as an out-of-memory (MemoryError in
  Python, as the reference raises when an allocation fails, Lik.pyx:66-84).
  CL-registry growth, batch creation and server admission fail cleanly at
  every point: the device memory they hold goes back to what it was, and
  the next call succeeds with the oracle's result.
"""
import ctypes
import gc

import pytest

from crux_gb300 import synth
from crux_gb300._native import DeviceTimeout
from crux_gb300.batch import Batch

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-11, "fp32": 1e-6}
DEFAULT_SPIN = 1 << 26


def rel(a, b):
    return abs(a - b) / abs(b)


class spin_limit:
    """Context: the walkers' record waits give up after `n` attempts."""

    def __init__(self, lib, n):
        self.lib, self.n = lib, n

    def __enter__(self):
        prev = ctypes.c_uint()
        assert self.lib.cxgDebugSetSpinLimit(self.n, ctypes.byref(prev)) == 0
        assert prev.value == DEFAULT_SPIN
        return self

    def __exit__(self, *exc):
        assert self.lib.cxgDebugSetSpinLimit(DEFAULT_SPIN, None) == 0
        return False


class fail_allocs:
    """Context: `k` more allocations of the library succeed, then none."""

    def __init__(self, lib, k):
        self.lib, self.k = lib, k

    def __enter__(self):
        self.lib.cxgDebugFailAllocs(self.k)
        return self

    def __exit__(self, *exc):
        self.lib.cxgDebugFailAllocs(-1)
        return False


def registry_bytes(lib):
    n = ctypes.c_size_t()
    assert lib.cxgLikDeviceBytes(ctypes.byref(n)) == 0
    return n.value


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_walker_wait_that_gives_up_is_reported(gpu, port, precision):
    case = synth.Case(24, 2000, 0.1, 71)
    lg = case.lik(lib=gpu, precision=precision)
    lo = case.lik(lib=port)
    assert rel(lg.lnL(), lo.lnL()) <= TOL[precision]
    for lk in (lg, lo):
        lk.tree.edges[5].length *= 1.7
    with spin_limit(gpu, 0):
        with pytest.raises(DeviceTimeout):
            lg.lnL()                      # a dirty path
        lg.lik.invalidate = True
        with pytest.raises(DeviceTimeout):
            lg.lnL()                      # a full plan
    # The bound is back: the next call recomputes every CL it needs.
    assert rel(lg.lnL(), lo.lnL()) <= TOL[precision]
    for lk in (lg, lo):
        lk.tree.edges[2].length *= 0.6
    assert rel(lg.lnL(), lo.lnL()) <= TOL[precision]


def test_batched_walker_wait_that_gives_up_is_reported(gpu, port):
    cs = [synth.Case(nt, ns, 0.1, 720 + i) for i, (nt, ns) in
          enumerate([(12, 600), (40, 1500), (25, 3000)])]
    want = [c.lik(lib=port).lnL() for c in cs]
    liks = [c.lik(lib=gpu, precision="fp32") for c in cs]
    for lk in liks:
        lk.prepare_plan()
    b = Batch(liks, "fp32")
    try:
        with spin_limit(gpu, 0):
            with pytest.raises(DeviceTimeout):
                b.run()
        got = b.run()
    finally:
        b.close()
    for g, w in zip(got, want):
        assert rel(g, w) <= TOL["fp32"]


def test_mc3_wait_that_gives_up_is_reported(gpu):
    from crux_gb300.mc3 import Mc3
    case = synth.Case(12, 500, 0.1, 73)
    aln = case.alignment()
    m = Mc3(case.tree(aln.taxaMap), aln, case.params["rates"],
            case.params["freqs"], alpha=0.5, ncat=4, nchains=2,
            heat_delta=0.2, seed=3, moves={"brlen": 1.0}, precision="fp32",
            graph_gens=4)
    try:
        m.run(4)
        with spin_limit(gpu, 0):
            with pytest.raises(DeviceTimeout):
                m.run(4)
    finally:
        m.close()


def test_server_wait_that_gives_up_is_reported(gpu, port):
    from crux_gb300.serve import LNL, PreparedRequest, Server
    req = PreparedRequest(synth.Case(20, 1200, 0.1, 74), LNL)
    want = req.oracle_lik(port).lnL()
    srv = Server("fp32")
    try:
        assert rel(srv.wait(srv.submit(req))[0], want) <= TOL["fp32"]
        with spin_limit(gpu, 0):
            with pytest.raises(DeviceTimeout):
                srv.wait(srv.submit(req))
        assert rel(srv.wait(srv.submit(req))[0], want) <= TOL["fp32"]
    finally:
        srv.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_cl_registry_allocation_failure(gpu, port, precision):
    """Every allocation of building a Lik and of its first two evaluations
    fails in turn; each failure raises MemoryError, leaves the registry's
    device bytes as they were once the Lik is gone, and the next call on the
    same Lik matches the oracle."""
    case = synth.Case(14, 900, 0.1, 75)
    lo = case.lik(lib=port)
    want = lo.lnL()
    lo.tree.edges[4].length *= 1.3
    want_dirty = lo.lnL()
    gc.collect()
    base = registry_bytes(gpu)
    failures = 0
    for k in range(40):
        lg = None
        failed = False
        with fail_allocs(gpu, k):
            try:
                lg = case.lik(lib=gpu, precision=precision)
                lg.lnL()
                lg.tree.edges[4].length *= 1.3
                lg.lnL()
            except MemoryError:
                failed = True
        if not failed:
            break
        failures += 1
        if lg is not None:
            # Injection is off: the same Lik recovers.
            lg.tree.edges[4].length = lo.tree.edges[4].length
            assert rel(lg.lnL(), want_dirty) <= TOL[precision]
        del lg
        gc.collect()
        assert registry_bytes(gpu) == base, k
    assert failures >= 3
    lg = case.lik(lib=gpu, precision=precision)
    assert rel(lg.lnL(), want) <= TOL[precision]
    del lg
    gc.collect()
    assert registry_bytes(gpu) == base


def test_batch_create_allocation_failure(gpu, port):
    import torch
    cs = [synth.Case(nt, ns, 0.1, 760 + i) for i, (nt, ns) in
          enumerate([(10, 400), (30, 2500)])]
    want = [c.lik(lib=port).lnL() for c in cs]
    liks = [c.lik(lib=gpu, precision="fp32") for c in cs]
    for lk in liks:
        lk.prepare_plan()
    Batch(liks, "fp32").close()          # warm: module and pools loaded
    free0 = torch.cuda.mem_get_info()[0]
    failures = 0
    for _ in range(5):
        for k in range(60):
            b = None
            with fail_allocs(gpu, k):
                try:
                    b = Batch(liks, "fp32")
                except MemoryError:
                    failures += 1
            if b is not None:
                b.close()
                break
    assert failures >= 5
    free1 = torch.cuda.mem_get_info()[0]
    assert free0 - free1 < (8 << 20), (free0, free1)
    b = Batch(liks, "fp32")
    try:
        got = b.run()
    finally:
        b.close()
    for g, w in zip(got, want):
        assert rel(g, w) <= TOL["fp32"]


def test_server_admission_allocation_failure(gpu, port):
    """A request whose device memory cannot be had fails alone with
    MemoryError, whether it carries its patterns or names a resident
    dataset; the server keeps serving the same requests afterwards."""
    from crux_gb300.serve import LNL, PreparedRequest, Server
    reqs = [PreparedRequest(synth.Case(nt, 700, 0.1, 780 + nt), LNL)
            for nt in (9, 17, 26)]
    want = [r.oracle_lik(port).lnL() for r in reqs]
    srv = Server("fp32")
    try:
        srv.add_dataset(7, reqs[1])
        resident = PreparedRequest(reqs[1].case, LNL,
                                   alignment=reqs[1].alignment, dataset=7)
        for r in (reqs[0], resident):
            with fail_allocs(gpu, 0):
                with pytest.raises(MemoryError):
                    srv.wait(srv.submit(r))
        got = [srv.wait(srv.submit(r))[0] for r in reqs + [resident]]
        st = srv.stats()
    finally:
        srv.close()
    for g, w in zip(got, want + [want[1]]):
        assert rel(g, w) <= TOL["fp32"]
    assert st["completed"] >= 6


def test_allocation_canaries_detect_an_overrun(gpu):
    """The canary check every GPU test ends with sees a byte changed past
    the end of an allocation (written by a host-side memset inside the
    allocation's canary, not by a kernel)."""
    det = ctypes.c_int()
    assert gpu.cxgDebugCanarySelfTest(ctypes.byref(det)) == 0
    assert det.value == 1
    checked, bad = ctypes.c_ulonglong(), ctypes.c_ulonglong()
    assert gpu.cxgDebugCheckCanaries(ctypes.byref(checked), ctypes.byref(bad)) == 0
    assert bad.value == 0
