"""Walker shapes and the autotuner: every (tile, threads per pattern,
patterns per thread, stack budget, op lanes) gives bit-identical lnLs and
site lnLs, in single plans and in batches, within the oracle tolerance of
each form; the tuner times its candidates and sets the fastest."""
import numpy as np
import pytest

from crux_gb300 import synth, tune
from crux_gb300.batch import Batch

pytestmark = pytest.mark.gpu

TOL = {"fp32": 1e-6, "fp64": 1e-11}


@pytest.fixture
def restore(gpu):
    saved = tune.get(gpu)
    yield
    tune.set_shape(gpu, *saved)


@pytest.mark.parametrize("shape", [(40, 3000, 0.0), (40, 3000, 0.2),
                                   (16, 1000, 0.0)])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_every_shape_same_bits(gpu, port, restore, precision, shape):
    """Every candidate shape, every stack budget (a budget near 48 KiB puts
    static plus dynamic shared memory across the default launch limit)."""
    ntaxa, nsites, pinv = shape
    case = synth.Case(ntaxa, nsites, 0.1, 77, pinv=pinv, gap_frac=0.01)
    want = case.lik(lib=port).lnL()
    lik = case.lik(lib=gpu, precision=precision)
    lik.lnL()  # the component weights are set by the first evaluation
    kact = tune.active_components(lik)
    assert kact == (4 if pinv == 0.0 else 5)
    shapes = tune.candidates(precision, kact)
    assert any(g > 1 for _, g, _, _, _ in shapes) == (precision == "fp32" and
                                                      kact % 2 == 0)
    assert any(p > 1 for _, _, p, _, _ in shapes) == (precision == "fp32" and
                                                      kact <= 5)
    assert any(n > 1 for _, _, _, _, n in shapes) == (precision == "fp32" and
                                                      kact <= 5)
    first = None
    for shape in shapes:
        tune.set_shape(gpu, *shape)
        lik.lik.invalidate = True
        v = lik.lnL()
        lik.lik.invalidate = True
        s = lik.siteLnLs()
        if first is None:
            first = (v, s)
            assert abs(v - want) <= TOL[precision] * abs(want), (v, want)
        else:
            assert v == first[0], shape
            assert s == first[1], shape


def test_batch_every_shape_same_bits(gpu, restore):
    rng = np.random.default_rng(5)
    cases = [synth.Case(int(rng.integers(8, 70)), int(rng.integers(300, 5000)),
                        0.1, 300 + i) for i in range(6)]
    liks = [c.lik(lib=gpu, precision="fp32") for c in cases]
    first = None
    for shape in tune.candidates("fp32", 4, budgets=(0, 24 << 10), lanes=(1,)):
        tune.set_shape(gpu, *shape)
        for lk in liks:
            lk.prepare_plan()
        b = Batch(liks, "fp32")
        out = b.run()
        b.close()
        if first is None:
            first = out
        else:
            assert np.array_equal(out, first), shape


def test_tune_plan_sets_fastest(gpu, restore):
    case = synth.Case(32, 20000, 0.1, 91)
    lik = case.lik(lib=gpu, precision="fp32")
    lik.prepare_plan()
    shapes = [(64, 1, 1, 24 << 10, 1), (64, 4, 1, 24 << 10, 1),
              (128, 2, 1, 12 << 10, 1), (128, 1, 2, 24 << 10, 1),
              (64, 1, 1, 24 << 10, 2)]
    res = tune.tune_plan(lik, "fp32", iters=5, shapes=shapes)
    assert len(res["table"]) == 5
    best = res["best"]
    assert best["ms"] == min(r["ms"] for r in res["table"])
    assert tune.get(gpu) == (best["tile"], best["tpp"], best["ppt"],
                             best["budget"], best["lanes"])


@pytest.mark.parametrize("tile", [32, 64])
def test_op_lanes_same_bits_on_dirty_paths(gpu, port, restore, tile):
    """Two op lanes against one on full plans, single-branch dirty paths
    (chains of dependent ops, so most steps have an empty lane) and other
    roots, with and without a stack budget: the same bits every time, and
    the oracle within the FP32 tolerance."""
    import random
    from crux_gb300.plan import Plan
    case = synth.Case(48, 4000, 0.1, 123, pinv=0.2, gap_frac=0.01)
    one = case.lik(lib=gpu, precision="fp32")
    two = case.lik(lib=gpu, precision="fp32")
    ref = case.lik(lib=port)
    rng = random.Random(9)
    lanes_seen = set()
    for it in range(40):
        if it % 10 == 0:
            for lk in (one, two, ref):
                lk.lik.invalidate = True
        else:
            i = rng.randrange(len(ref.tree.edges))
            f = rng.uniform(0.5, 2.0)
            for lk in (one, two, ref):
                lk.tree.edges[i].length *= f
        budget = (0, 12 << 10, 24 << 10)[it % 3]
        k = rng.randrange(len(ref.tree.nodes)) if it % 7 == 3 else None
        roots = [None if k is None else lk.tree.nodes[k]
                 for lk in (one, two, ref)]
        tune.set_shape(gpu, tile, 1, 1, budget, 1)
        a = one.lnL(roots[0])
        tune.set_shape(gpu, tile, 1, 1, budget, 2)
        two._prep(roots[1])
        plan = Plan(two, "fp32")
        lanes_seen.add(plan.shape()["lanes"])
        b = plan.run()
        plan.close()
        want = ref.lnL(roots[2])
        assert a == b, (it, a, b)
        assert abs(a - want) <= TOL["fp32"] * abs(want)
    assert 2 in lanes_seen


def test_mc3_and_server_follow_the_shape(gpu, restore):
    """MC3 chains and server requests translated under different shapes
    give the same bits."""
    from crux_gb300.mc3 import Mc3
    from crux_gb300.serve import LNL, PreparedRequest, Server
    case = synth.Case(16, 1500, 0.1, 12)
    aln = case.alignment()
    req = PreparedRequest(case, LNL)
    traces, served = [], []
    shapes = [(64, 1, 1, 24 << 10, 1), (64, 4, 1, 24 << 10, 1), (32, 2, 1, 0, 1),
              (128, 1, 2, 24 << 10, 2)]
    for shape in shapes:
        tune.set_shape(gpu, *shape)
        m = Mc3(case.tree(aln.taxaMap), aln, case.params["rates"],
                case.params["freqs"], alpha=0.5, ncat=4, nchains=2, seed=3,
                moves={"brlen": 1.0, "nni": 1.0, "rates": 0.5, "alpha": 0.5},
                precision="fp32", graph_gens=4)
        m.run(24)
        traces.append(m.trace(25))
        m.close()
        srv = Server("fp32")
        served.append(srv.wait(srv.submit(req))[0])
        srv.close()
    assert all(np.array_equal(traces[0], t) for t in traces[1:])
    assert all(s == served[0] for s in served[1:])


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_streamed_leaves_every_shape(gpu, port, restore, precision):
    """A 300-taxon tree: at tile 64 and 128 its leaf masks exceed the
    staging budget (16 KiB a tile), so each op's leaf rows travel with its
    record (streamed leaves) and the FP32 op kinds read a leaf's row by its
    rank among the op's leaf children.  Every shape gives the same bits as
    the staged tile-32 shape, within the oracle tolerance, full and after a
    dirty path; so does a batch holding the tree."""
    case = synth.Case(300, 400, 0.1, 303, gap_frac=0.01)
    lo = case.lik(lib=port)
    want = lo.lnL()
    lik = case.lik(lib=gpu, precision=precision)
    lik.lnL()
    first = None
    for shape in tune.candidates(precision, 4, budgets=(0, 24 << 10), lanes=(1,)):
        tune.set_shape(gpu, *shape)
        lik.lik.invalidate = True
        v = lik.lnL()
        if first is None:
            first = v
            assert abs(v - want) <= TOL[precision] * abs(want), (v, want)
        else:
            assert v == first, shape
    e_lo, e_g = lo.tree.edges[7], lik.tree.edges[7]
    old = e_g.length
    e_lo.length = old * 1.4
    want2 = lo.lnL()
    for shape in [(128, 1, 1, 0), (64, 1, 1, 24 << 10), (32, 1, 1, 0)]:
        tune.set_shape(gpu, *shape)
        e_g.length = old
        lik.lik.invalidate = True
        lik.lnL()
        e_g.length = old * 1.4
        v2 = lik.lnL()  # a dirty path
        assert abs(v2 - want2) <= TOL[precision] * abs(want2), (shape, v2, want2)
    if precision == "fp32":
        tune.set_shape(gpu, 128, 1, 1, 0)
        lik.prepare_plan()
        b = Batch([lik], "fp32")
        got = b.run()
        b.close()
        assert abs(got[0] - want2) <= TOL["fp32"] * abs(want2)
