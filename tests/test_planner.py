"""The native step planner (cxgPlanSnapRun) against the Python restatement of
Lik._plan / _planRecurse (pkg/Crux/Tree/Lik.pyx:1427-1601).

Two Liks on identical trees take the same random sequence of operations:
branch rescales, invalidations, other roots, NNI rearrangements, model
changes, flushes, the other-polarity clone and a negative branch length.
One plans natively whenever its traversal is unchanged, and the other always
plans in Python.  After every plan the step arrays, the lnLs (CPU oracle) and
every CL's mirrors and CxtLikCL fields must be identical.  No GPU is used."""
import ctypes
import random

import numpy as np
import pytest

from crux_gb300 import _abi, lik as likmod, synth


def _addr(p):
    return ctypes.cast(p, ctypes.c_void_p).value


def _pairs(a, b):
    """(CL of a, CL of b) for every ring of the two (same-shaped) trees."""
    out = [(a.rootCL, b.rootCL)]
    if a.mate is not None:
        out.append((a.mate.rootCL, b.mate.rootCL))
    for ea, eb in zip(a.tree.edges, b.tree.edges):
        for ra, rb in ((ea.ring, eb.ring), (ea.ring.other, eb.ring.other)):
            assert (ra.aux is None) == (rb.aux is None)
            if ra.aux is not None:
                out.append((ra.aux, rb.aux))
    return out


def _check_same(a, b, la, lb):
    assert la == lb or (np.isnan(la) and np.isnan(lb))
    pairs = _pairs(a, b)
    amap = {None: None}
    for ca, cb in pairs:
        for p in (0, 1):
            amap[ca.addr[p]] = cb.addr[p]
    objmap = {id(ca): cb for ca, cb in pairs}
    sa = np.frombuffer(a._steps, dtype=_abi.STEP_DTYPE)[:a.lik.stepsLen]
    sb = np.frombuffer(b._steps, dtype=_abi.STEP_DTYPE)[:b.lik.stepsLen]
    assert len(sa) == len(sb)
    assert (sa["variant"] == sb["variant"]).all()
    assert (sa["ntrail"] == sb["ntrail"]).all()
    assert (sa["edgeLen"] == sb["edgeLen"]).all()
    assert [amap[int(x)] for x in sa["parentCL"]] == sb["parentCL"].tolist()
    assert [amap[int(x)] for x in sa["childCL"]] == sb["childCL"].tolist()
    for ca, cb in pairs:
        for p in (0, 1):
            assert ca.valid[p] == cb.valid[p]
            assert ca.cvalid[p] == cb.cvalid[p]
            assert ca.nSibs[p] == cb.nSibs[p]
            assert ca.edgeLen[p] == cb.edgeLen[p]
            assert (ca.bufs[p] is None) == (cb.bufs[p] is None)
            pa = ca.parent[p]
            assert (pa is None and cb.parent[p] is None) or \
                objmap[id(pa)] is cb.parent[p]
            sa_, sb_ = ca.c[p], cb.c[p]
            assert bool(sa_.valid) == bool(sb_.valid)
            assert sa_.nSibs == sb_.nSibs and sa_.edgeLen == sb_.edgeLen
            assert amap.get(_addr(sa_.parent)) == _addr(sb_.parent)


def _nni(tree, k, side):
    """Swap subtree x (across ring a of u) with subtree y (across ring b of
    v) over the internal edge u-v.  Each subtree keeps the ring it hangs
    from, and with it that ring's cached CL, as the sampler's NNI does."""
    inner = [e for e in tree.edges if e.ring.node.getDegree() > 1
             and e.ring.other.node.getDegree() > 1]
    e = inner[k % len(inner)]
    u, v = e.ring, e.ring.other
    a = u.next
    b = v.next if side == 0 else v.next.next
    ea, eb = a.edge, b.edge
    x, y = a.other.node, b.other.node
    un, vn = u.node, v.node
    xa = ea.ring is a.other      # edge.ring lands on attach's first node
    yb = eb.ring is b.other
    ea.detach()
    eb.detach()
    if xa:
        ea.attach(x, vn)
    else:
        ea.attach(vn, x)
    if yb:
        eb.attach(y, un)
    else:
        eb.attach(un, y)


def _lnl(lk, root):
    try:
        return lk.lnL(root)
    except ValueError as e:
        return str(e)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_native_planner_matches_python_planner(port, seed):
    assert likmod.planner_library() is not None, \
        "libcxlik_gpu.so (which holds the native planner) is not built"
    case = synth.Case(10, 300, 0.1, 40 + seed)
    a = case.lik(lib=port)
    b = case.lik(lib=port)
    a.native_plan = True
    b.native_plan = False
    rng = random.Random(seed)
    root_a = root_b = None
    native_runs = 0
    for it in range(400):
        op = rng.random()
        ea, eb = a.tree.edges, b.tree.edges
        if op < 0.45:
            i = rng.randrange(len(ea))
            f = rng.uniform(0.5, 2.0)
            ea[i].length *= f
            eb[i].length *= f
        elif op < 0.55:
            a.lik.invalidate = b.lik.invalidate = True
        elif op < 0.62:
            k = rng.randrange(len(a.tree.nodes))
            root_a, root_b = a.tree.nodes[k], b.tree.nodes[k]
            if rng.random() < 0.3:
                root_a = root_b = None
        elif op < 0.70:
            k, side = rng.randrange(100), rng.randrange(2)
            _nni(a.tree, k, side)
            _nni(b.tree, k, side)
            root_a = root_b = None
        elif op < 0.76:
            alpha = rng.uniform(0.2, 2.0)
            a.setAlpha(0, alpha)
            b.setAlpha(0, alpha)
        elif op < 0.80:
            a.flush()
            b.flush()
        elif op < 0.85:
            ma, mb = a.clone(), b.clone()
            ma.native_plan = True
            mb.native_plan = False
            for _ in range(rng.randrange(1, 4)):
                _check_same(ma, mb, _lnl(ma, root_a), _lnl(mb, root_b))
        elif op < 0.88:
            i = rng.randrange(len(ea))
            old = ea[i].length
            ea[i].length = eb[i].length = -0.25
            ra, rb = _lnl(a, root_a), _lnl(b, root_b)
            assert ra == rb
            ea[i].length = eb[i].length = old
        had = a._snap is not None
        _check_same(a, b, _lnl(a, root_a), _lnl(b, root_b))
        native_runs += had and a._snap is not None
    # Most plans after the first one on a traversal ran natively.
    assert native_runs > 100, native_runs


def test_native_planner_full_and_dirty_plans(port):
    """Full re-plans and single-branch dirty paths of a 64-taxon tree plan
    natively.  A full plan has one step per edge, 2N-3, plus the 0-length
    merge of a leaf base (Lik.pyx:1560-1575): 2N-2 here."""
    case = synth.Case(64, 200, 0.05, 11)
    a = case.lik(lib=port)
    b = case.lik(lib=port)
    a.native_plan = True
    b.native_plan = False
    # The first plans create every CL (which any traversal kept for the
    # native planner notices); from the third plan on `a` plans natively.
    for _ in range(2):
        for lk in (a, b):
            lk.lik.invalidate = True
        _check_same(a, b, a.lnL(), b.lnL())
    for lk in (a, b):
        lk.lik.invalidate = True
    _check_same(a, b, a.lnL(), b.lnL())
    assert a.tree.base.getDegree() == 1
    assert a._snap is not None and a.lik.stepsLen == 2 * 64 - 2
    rng = random.Random(5)
    for _ in range(50):
        i = rng.randrange(len(a.tree.edges))
        f = rng.uniform(0.5, 2.0)
        a.tree.edges[i].length *= f
        b.tree.edges[i].length *= f
        _check_same(a, b, a.lnL(), b.lnL())
        assert a._snap is not None


def test_native_planner_polytomies(port):
    """Multifurcating nodes (a degree-5 root, degree-4 and degree-3
    internal nodes): one Compute step and degree-2 Merge steps per dirty
    node with ntrail counting down, as the Python planner writes them, at
    every root and after rescales; and the same lnL as the Python planner
    on the oracle."""
    import kat_cases as K
    from crux_gb300.alignment import Alignment, CTMatrix
    from crux_gb300.lik import Lik
    rng = np.random.default_rng(8)
    names = ["t%d" % i for i in range(9)]
    fasta = "".join(">%s\n%s\n" % (n, "".join(rng.choice(list("ACGT"), 60)))
                    for n in names)
    newick = ("(t0:0.1,t1:0.2,(t2:0.1,t3:0.3,t4:0.05,t5:0.2):0.15,"
              "(t6:0.1,t7:0.2,t8:0.3):0.1);")
    aln = Alignment(CTMatrix(fasta))
    a = Lik(K.tree_for(newick, aln), aln, ncat=4, lib=port)
    b = Lik(K.tree_for(newick, aln), aln, ncat=4, lib=port)
    a.setAlpha(0, 0.7)
    b.setAlpha(0, 0.7)
    a.native_plan = True
    b.native_plan = False
    degrees = sorted(n.getDegree() for n in a.tree.nodes)
    assert degrees[-1] >= 4
    prng = random.Random(2)
    native = 0
    for it in range(60):
        k = prng.randrange(len(a.tree.nodes))
        if it % 3 == 0:
            i = prng.randrange(len(a.tree.edges))
            f = prng.uniform(0.5, 2.0)
            a.tree.edges[i].length *= f
            b.tree.edges[i].length *= f
        ra, rb = (a.tree.nodes[k], b.tree.nodes[k]) if it % 4 == 1 else (None, None)
        _check_same(a, b, a.lnL(ra), b.lnL(rb))
        native += a._snap is not None
    assert native > 20, native
    # Steps of a node with four children: Compute with ntrail 3, then
    # Merges with 2, 1, 0.
    a.lik.invalidate = True
    a.lnL()
    steps = a.steps()
    trails = [t for _, t, _ in steps]
    assert 3 in trails and trails[trails.index(3) + 1:trails.index(3) + 4] == [2, 1, 0]


def test_plan_snap_c_entry_point():
    """cxgPlanSnapRun through the C ABI (host code: no GPU) on a hand-made
    snapshot: a root with two leaf children.  It writes the steps and the
    CxtLikCL fields, reports which visits changed, plans nothing when
    nothing changed, replans after a length change, returns 1 for a
    negative length, and rejects a malformed snapshot or a full step
    array."""
    from crux_gb300 import _native
    lib = _native.load()   # loading makes no CUDA call
    cls = [_abi.CxtLikCL() for _ in range(3)]
    addr = [ctypes.addressof(c) for c in cls]
    u32, i32 = np.uint32, np.int32
    arrs = dict(
        cl=np.array(addr, dtype=np.uint64), up=np.array([2, 2, -1], dtype=i32),
        nsibs=np.array([2, 2, 0], dtype=u32), edge=np.array([0, 1, -1], dtype=i32),
        kid0=np.array([0, 0, 0], dtype=u32), nkids=np.array([0, 0, 2], dtype=u32),
        kid_cl=np.array(addr[:2], dtype=np.uint64),
        kid_int=np.array([0, 0], dtype=np.uint8),
        kid_edge=np.array([0, 1], dtype=i32),
        valid=np.zeros(3, dtype=np.uint8), cvalid=np.zeros(3, dtype=np.uint8),
        m_parent=np.zeros(3, dtype=np.uint64), m_nsibs=np.zeros(3, dtype=u32),
        m_elen=np.zeros(3, dtype=np.float64))
    snap = _abi.CxgPlanSnap()
    snap.nvis, snap.nkid = 3, 2
    for k, v in arrs.items():
        setattr(snap, k, v.ctypes.data)
    lens = np.array([0.1, 0.2])
    steps = (_abi.CxtLikStep * 4)()
    ns, nc = ctypes.c_uint32(), ctypes.c_uint32()
    changed = np.zeros(3, dtype=np.uint32)

    def run(inval, cap=4):
        return lib.cxgPlanSnapRun(
            ctypes.byref(snap), _abi.dptr(lens), inval, steps, cap,
            ctypes.byref(ns), changed.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
            ctypes.byref(nc))

    assert run(1) == 0 and ns.value == 2
    got = [(steps[i].variant, steps[i].ntrail, _addr(steps[i].parentCL),
            _addr(steps[i].childCL), steps[i].edgeLen) for i in range(2)]
    assert got == [(_abi.ComputeL, 1, addr[2], addr[0], 0.1),
                   (_abi.MergeL, 0, addr[2], addr[1], 0.2)]
    assert sorted(changed[:nc.value].tolist()) == [0, 1, 2]
    assert _addr(cls[0].parent) == addr[2] and cls[1].nSibs == 2
    assert cls[1].edgeLen == 0.2 and bool(cls[2].valid)
    assert run(0) == 0 and ns.value == 0 and nc.value == 0
    lens[0] = 0.3
    assert run(0) == 0 and ns.value == 2 and steps[0].edgeLen == 0.3
    assert changed[:nc.value].tolist() == [0] and cls[0].edgeLen == 0.3
    lens[1] = -1.0
    assert run(1) == 1                      # "Negative branch length"
    lens[1] = 0.2
    assert run(1, cap=1) == -1              # the step array is too small
    arrs["up"][2] = 0                       # the last visit must be the root
    assert run(1) == -1
    assert b"root" in lib.cxgLastError()
