"""GPU parity: the GB300 library against the FP64 oracle on the same inputs.

Bars (written into each assertion): plain FP64 path within 1e-11 relative of
the oracle's lnL, FP32-scaled path within 1e-6 relative.  Every call goes
through the C ABI of include/cxlik_gpu.h.
"""
import ctypes
import math

import numpy as np
import pytest

import kat_cases as K
from crux_gb300 import _abi, synth
from crux_gb300.lik import Lik

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-11, "fp32": 1e-6}


def rel(a, b):
    if math.isinf(a) and math.isinf(b) and (a < 0) == (b < 0):
        return 0.0
    return abs(a - b) / max(abs(b), 1e-300)


def from_scratch(case, lo):
    """lnL of `lo`'s current tree from a fresh oracle Lik that recomputes
    every CL (invalidate, Python planner): a dirty-path result checked
    against this does not depend on the planner's cache-validity rule."""
    fresh = case.lik(lib=lo.lib, alignment=lo.alignment)
    assert not fresh.native_plan
    for e, src in zip(fresh.tree.edges, lo.tree.edges):
        e.length = src.length
    fresh.lik.invalidate = True
    return fresh.lnL()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_kat_lik_b(gpu, port, precision):
    g = K.run_lik_b(gpu, precision)
    o = K.run_lik_b(port)
    for (gl, gs), (ol, os_), (el, es) in zip(g, o, K.LIK_B):
        assert rel(gl, ol) <= TOL[precision]
        assert K.close(gl, el, 5)
        for a, b in zip(gs, os_):
            assert abs(a - b) <= TOL[precision] * max(1.0, abs(b)) * 10


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_kat_lik_e_gamma(gpu, port, precision):
    for g, o in zip(K.run_lik_e(gpu, precision), K.run_lik_e(port)):
        for gg, oo in zip(g, o):
            for a, b in zip(gg, oo):
                assert rel(a, b) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_kat_missing_and_every_root(gpu, port, precision):
    for g, o in zip(K.run_lik_h(gpu, precision), K.run_lik_h(port)):
        for a, b in zip(g, o):
            assert rel(a, b) <= TOL[precision]
    g = K.run_every_root(gpu, K.THREE, "(one:0.0,two:0.0,three:1.25);",
                         precision=precision)
    o = K.run_every_root(port, K.THREE, "(one:0.0,two:0.0,three:1.25);")
    for (gl, gs), (ol, os_) in zip(g, o):
        assert rel(gl, ol) <= TOL[precision]
        assert K.close(gl, K.LIK_C[0], 4)
    for blen, elnl, _ in K.LIK_J:
        nw = "(one:0.0,two:0.0,three:%r);" % blen
        g = K.run_every_root(gpu, K.THREE, nw, (0.4, 0.3, 0.2, 0.1), precision)
        o = K.run_every_root(port, K.THREE, nw, (0.4, 0.3, 0.2, 0.1))
        for (gl, _), (ol, _) in zip(g, o):
            assert rel(gl, ol) <= TOL[precision]
            assert K.close(gl, elnl, 5)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_kat_zero_lengths_give_minus_inf(gpu, precision):
    for v in K.run_lik_g(gpu, precision):
        assert v <= -50.0


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_kat_invariant_and_mixtures(gpu, port, precision):
    gd, ge = K.run_lik_l(gpu, precision)
    od, oe = K.run_lik_l(port)
    for (gl, _), (ol, _) in zip(gd + ge, od + oe):
        assert rel(gl, ol) <= TOL[precision]
    for g, o in zip(K.run_lik_d(gpu, precision), K.run_lik_d(port)):
        for a, b in zip(g, o):
            assert rel(a, b) <= TOL[precision]
    for g, o in zip(K.run_lik_k(gpu, precision), K.run_lik_k(port)):
        for (a, _), (b, _) in zip(g, o):
            assert rel(a, b) <= TOL[precision]


def test_kat_lik_m_tightest_pin(gpu):
    render, lnl = K.run_lik_m(gpu, "fp64")
    assert render == K.LIK_M_RENDER
    assert abs(lnl - K.LIK_M) <= 5e-10


CASES = [
    # (ntaxa, nsites, mean brlen, seed, pinv, gap fraction)
    (16, 1000, 0.1, 11, 0.0, 0.0),
    (64, 10000, 0.05, 12, 0.2, 0.005),
    (37, 3000, 0.3, 13, 0.0, 0.02),
]


@pytest.mark.parametrize("shape", CASES)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_synthetic_full_then_dirty_paths(gpu, port, shape, precision):
    nt, ns, bl, seed, pinv, gap = shape
    case = synth.Case(nt, ns, bl, seed, pinv=pinv, gap_frac=gap)
    lg = case.lik(lib=gpu, precision=precision)
    lo = case.lik(lib=port)
    a, b = lg.lnL(), lo.lnL()
    assert rel(a, b) <= TOL[precision], (a, b)
    rng = np.random.default_rng(seed)
    eg, eo = lg.tree.edges, lo.tree.edges
    for _ in range(12):
        i = int(rng.integers(len(eg)))
        f = float(rng.uniform(0.5, 2.0))
        eg[i].length *= f
        eo[i].length *= f
        a, b = lg.lnL(), lo.lnL()
        assert lg.nsteps < 2 * nt - 2 or nt < 8
        assert rel(a, b) <= TOL[precision], (a, b)
        full = from_scratch(case, lo)
        assert rel(b, full) <= 1e-12, (b, full)
        assert rel(a, full) <= TOL[precision], (a, full)
    sg = np.array(lg.siteLnLs())
    so = np.array(lo.siteLnLs())
    tol = TOL[precision] * np.maximum(1.0, np.abs(so)) * 10
    assert np.all(np.abs(sg - so) <= tol)


def test_dropin_cxlikexecute_host_buffers(gpu, port):
    """CxLikExecute with Lik.pyx's host layout: leaf rows of 4 doubles,
    siteLnL and stripeLnL written back, stripe sums in pattern order."""
    ld = synth.Case(24, 2000, 0.1, 21, gap_frac=0.01)
    aln = ld.alignment()
    lik = Lik(ld.tree(aln.taxaMap), aln, ncat=4, lib=gpu, dropin=True)
    synth.apply_params(lik, 0, ld.params, ld.alpha)
    lo = ld.lik(lib=port)
    a = lik.execute_dropin()
    b = lo.lnL()
    assert rel(a, b) <= 1e-11
    assert np.allclose(lik.siteLnLBuf, lo.siteLnLBuf, rtol=1e-11, atol=1e-11)
    assert np.allclose(lik.stripeLnLBuf, lo.stripeLnLBuf, rtol=1e-11,
                       atol=1e-11)
    # Dirty path through the drop-in entry point.
    e1, e2 = lik.tree.edges, lo.tree.edges
    for i in (3, 7, 11):
        e1[i].length *= 1.7
        e2[i].length *= 1.7
        assert rel(lik.execute_dropin(), lo.lnL()) <= 1e-11


def test_qdecomp_and_pt_match_oracle(gpu, port):
    rng = np.random.default_rng(5)
    dp = _abi.dptr
    for _ in range(20):
        p = synth.gtr_params(rng)
        outs = []
        for lib in (gpu, port):
            rt = np.array(p["rates"])
            pi = np.array(p["freqs"]) * 3.0
            pn = np.zeros(4)
            cube = np.zeros(64)
            ev = np.zeros(4)
            qn = ctypes.c_double()
            assert not lib.CxLikQDecomp(4, dp(rt), dp(pi), dp(pn),
                                        ctypes.byref(qn), dp(cube), dp(ev))
            Ps = []
            for t in (0.0, 0.01, 0.3, 2.0):
                P = np.zeros(16)
                lib.CxLikPt(4, dp(P), dp(cube), dp(ev), t)
                Ps.append(P)
            outs.append((pn, qn.value, Ps))
        (pa, qa, Pa), (pb, qb, Pb) = outs
        assert np.allclose(pa, pb, rtol=1e-15, atol=0)
        assert math.isclose(qa, qb, rel_tol=1e-14)
        for x, y in zip(Pa, Pb):
            assert np.allclose(x, y, rtol=1e-12, atol=1e-14)


def test_qdecomp_rejects_bad_input(gpu):
    dp = _abi.dptr
    rt = np.ones(6)
    pi = np.array([0.25, 0.25, 0.0, 0.5])
    out = [np.zeros(4), np.zeros(64), np.zeros(4)]
    qn = ctypes.c_double()
    assert gpu.CxLikQDecomp(4, dp(rt), dp(pi), dp(out[0]), ctypes.byref(qn),
                            dp(out[1]), dp(out[2]))
    assert gpu.CxLikQDecomp(5, dp(rt), dp(pi), dp(out[0]), ctypes.byref(qn),
                            dp(out[1]), dp(out[2]))


@pytest.mark.parametrize("ncat,nmod", [(1, 1), (2, 1), (3, 2), (8, 1), (2, 4)])
def test_component_counts(gpu, port, ncat, nmod):
    case = synth.Case(12, 800, 0.2, 31)
    res = []
    for lib in (gpu, port):
        aln = case.alignment()
        lik = Lik(case.tree(aln.taxaMap), aln, nmodels=nmod, ncat=ncat, lib=lib)
        for m in range(nmod):
            synth.apply_params(lik, m, case.params, 0.7 if ncat > 1 else None)
            lik.setRmult(m, 1.0 + 0.3 * m)
        res.append(lik.lnL())
    assert rel(res[0], res[1]) <= 1e-11


def test_too_many_components_is_an_error(gpu):
    case = synth.Case(8, 200, 0.2, 3)
    aln = case.alignment()
    lik = Lik(case.tree(aln.taxaMap), aln, nmodels=3, ncat=3, lib=gpu)
    for m in range(3):
        lik.setAlpha(m, 0.5)
    with pytest.raises(RuntimeError, match="8 active"):
        lik.lnL()


def test_plan_handle_runs_and_times(gpu, port):
    case = synth.Case(32, 4000, 0.1, 41)
    lik = case.lik(lib=gpu, precision="fp32")
    a = lik.lnL()
    from crux_gb300 import plan as planmod
    lik.lik.invalidate = True
    lik._prep(None)
    pl = planmod.Plan(lik, "fp32")
    b = pl.run()
    t = pl.time(5)
    info = pl.info()
    pl.close()
    assert rel(b, a) <= 1e-12
    assert rel(t["lnL"], a) <= 1e-12
    assert info["nops"] == 31
    assert info["updates"] == 31 * lik.lik.mschars
    assert t["ms_per_run"] > 0 and t["kernel_ms"] > 0


def test_device_memory_released(gpu):
    import gc
    gc.collect()
    before = ctypes.c_size_t()
    gpu.cxgLikDeviceBytes(ctypes.byref(before))
    case = synth.Case(20, 1500, 0.1, 51)
    lik = case.lik(lib=gpu)
    lik.lnL()
    mid = ctypes.c_size_t()
    gpu.cxgLikDeviceBytes(ctypes.byref(mid))
    assert mid.value > before.value
    del lik
    gc.collect()
    after = ctypes.c_size_t()
    gpu.cxgLikDeviceBytes(ctypes.byref(after))
    assert after.value == before.value


import golden_cases as G  # noqa: E402


@pytest.mark.parametrize("path", G.fixtures())
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_golden_fixtures(gpu, path, precision):
    """Full lnL, site lnLs and dirty-path lnLs against the reference's own
    outputs stored in tests/golden."""
    fx = G.load(path)
    lik = G.build_lik(fx, gpu, precision)
    assert rel(lik.lnL(), fx["lnL"]) <= TOL[precision]
    sites = np.array(lik.siteLnLs())
    want = np.array(fx["siteLnL"])
    assert np.all(np.abs(sites - want) <=
                  TOL[precision] * np.maximum(1.0, np.abs(want)) * 10)
    edges = lik.tree.edges
    for i, f, w, scratch in fx["dirty"]:
        edges[i].length *= f
        got = lik.lnL()
        assert rel(got, w) <= TOL[precision]
        assert rel(got, scratch) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_many_dirty_paths_gtr_gamma_inv(gpu, port, precision):
    """300 dirty-path lnLs on the 64-taxon GTR+G4+I shape with 0.5 % gaps:
    each rescale sets one branch to its generated length x U(0.5, 2), and
    every lnL is checked against the oracle replaying the same rescales."""
    case = synth.Case(64, 10000, 0.05, 20261208, pinv=0.2, gap_frac=0.005)
    lg = case.lik(lib=gpu, precision=precision)
    lo = case.lik(lib=port)
    eg, eo = lg.tree.edges, lo.tree.edges
    base = [e.length for e in eg]
    rng = np.random.default_rng(8)
    assert rel(lg.lnL(), lo.lnL()) <= TOL[precision]
    for k in range(300):
        i = int(rng.integers(len(eg)))
        f = float(rng.uniform(0.5, 2.0))
        eg[i].length = eo[i].length = base[i] * f
        a, b = lg.lnL(), lo.lnL()
        assert rel(a, b) <= TOL[precision], (a, b)
        if k % 10 == 0:
            full = from_scratch(case, lo)
            assert rel(b, full) <= 1e-12, (k, b, full)
            assert rel(a, full) <= TOL[precision], (k, a, full)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_repeated_full_plans_reuse_translation(gpu, port, precision):
    """A full re-plan of an unchanged tree has the previous call's steps on
    the same buffers, so the library reuses that translation and uploads only
    the new values.  Branch lengths, alpha, rates and frequencies change
    between calls and every lnL must follow the oracle; the program upload
    of a reused call is small.  A second Lik interleaved with the first
    changes the plan on every call (no reuse) and must also follow.  The
    garbage collector stays off during the calls: a Lik of an earlier test
    collected between two calls would release its CL buffers, and a
    registry change rightly ends the reuse."""
    import gc
    gc.collect()
    gc.disable()
    try:
        _repeated_full_plans(gpu, port, precision)
    finally:
        gc.enable()


def _repeated_full_plans(gpu, port, precision):
    case = synth.Case(24, 2000, 0.1, 611)
    other = synth.Case(17, 900, 0.1, 612)
    a = case.lik(lib=gpu, precision=precision)
    ra = case.lik(lib=port)
    b = other.lik(lib=gpu, precision=precision)
    rb = other.lik(lib=port)
    rng = np.random.default_rng(3)
    h2d, d2h = ctypes.c_size_t(), ctypes.c_size_t()
    seen = []
    for it in range(12):
        kind = it % 4
        for lk in (a, ra):
            lk.lik.invalidate = True
        if kind == 0:
            f = rng.uniform(0.5, 2.0, size=len(ra.tree.edges))
            for lk in (a, ra):
                for e, x in zip(lk.tree.edges, f):
                    e.length *= float(x)
        elif kind == 1:
            alpha = float(rng.uniform(0.2, 2.0))
            for lk in (a, ra):
                lk.setAlpha(0, alpha)
        elif kind == 2:
            rates = [float(x) for x in rng.dirichlet(np.ones(6)) * 6]
            for lk in (a, ra):
                lk.setRclass(0, [0, 1, 2, 3, 4, 5], rates)
        else:
            freqs = rng.dirichlet(np.full(4, 5.0))
            for lk in (a, ra):
                for i, x in enumerate(freqs):
                    lk.setFreq(0, i, float(x))
        got, want = a.lnL(), ra.lnL()
        gpu.cxgLikLastIo(ctypes.byref(h2d), ctypes.byref(d2h))
        assert rel(got, want) <= TOL[precision], (it, got, want)
        seen.append(got)
        if it % 2 == 1:
            # The previous call was a's own (b runs after a on odd calls):
            # the translation is reused and only the values travel.
            assert h2d.value < 8192, (it, h2d.value)
        if it % 2 == 1:
            for lk in (b, rb):
                lk.lik.invalidate = True
            assert rel(b.lnL(), rb.lnL()) <= TOL[precision]
    assert len(set(seen)) == len(seen)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_pickle_round_trip_and_simulate(gpu, port, precision):
    """A pickled Lik completed by unpickle gives the same lnL bit for bit
    on the GPU (Lik.pyx:326-386, 573-585); a simulated Lik (Lik.pyx:
    662-833, P(t) from the GPU library's CxLikPt) evaluates on the GPU as
    the oracle evaluates the same simulated alignment."""
    import pickle
    import random
    case = synth.Case(20, 1500, 0.1, 95, pinv=0.2)
    lik = case.lik(lib=gpu, precision=precision)
    want = lik.lnL()
    ret = lik.unpickle(pickle.dumps(lik))
    assert ret.lnL() == want
    sim = lik.simulate(3000, rng=random.Random(7))
    got = sim.lnL()
    ref = Lik(sim.tree.dup(), sim.alignment, ncat=case.ncat, invar=True,
              lib=port)
    synth.apply_params(ref, 0, case.params, case.alpha, case.pinv)
    assert rel(got, ref.lnL()) <= TOL[precision], (got, ref.lnL())
