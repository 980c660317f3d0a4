"""Batched persistent walker: many jobs in one launch give the same lnLs as
one plan at a time (FP64 within 1e-11 relative, FP32 within 1e-6 of the
FP64 oracle), for uneven taxon and pattern counts; the per-node comparison
path agrees too."""
import math

import numpy as np
import pytest

from crux_gb300 import synth
from crux_gb300.batch import Batch

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-11, "fp32": 1e-6}
SHAPES = [(16, 700, 0.1), (57, 2100, 0.05), (9, 333, 0.3), (130, 1500, 0.07),
          (33, 5000, 0.02)]


def cases():
    return [synth.Case(nt, ns, bl, 1000 + i) for i, (nt, ns, bl) in
            enumerate(SHAPES)]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("per_node", [False, True])
def test_batch_matches_oracle(gpu, port, precision, per_node):
    cs = cases()
    want = [c.lik(lib=port).lnL() for c in cs]
    liks = [c.lik(lib=gpu, precision=precision) for c in cs]
    for lk in liks:
        lk.prepare_plan()
    b = Batch(liks, precision, per_node=per_node)
    got = b.run()
    got2 = b.run()          # replay of the captured graph
    info = b.info()
    b.close()
    for g, g2, w in zip(got, got2, want):
        assert abs(g - w) <= TOL[precision] * abs(w), (g, w)
        assert g == g2
    assert info["items"] > len(cs)
    if per_node:
        assert info["launches_per_run"] > 100


def test_batch_after_dirty_paths(gpu, port):
    """Jobs whose plans are dirty paths (cached CLs read from HBM)."""
    cs = cases()[:3]
    lo = [c.lik(lib=port) for c in cs]
    lg = [c.lik(lib=gpu, precision="fp32") for c in cs]
    for a, b in zip(lo, lg):
        a.lnL()
        b.lnL()
        a.tree.edges[3].length *= 1.5
        b.tree.edges[3].length *= 1.5
        b.prepare_plan(full=False)
    bt = Batch(lg, "fp32")
    got = bt.run()
    bt.close()
    for g, a in zip(got, lo):
        w = a.lnL()
        assert abs(g - w) <= 1e-6 * abs(w)


def test_batch_rejects_mixed_components(gpu):
    c1, c2 = synth.Case(8, 300, 0.1, 1), synth.Case(8, 300, 0.1, 2, pinv=0.2)
    l1, l2 = c1.lik(lib=gpu), c2.lik(lib=gpu)
    l1.prepare_plan()
    l2.prepare_plan()
    with pytest.raises(RuntimeError, match="group them by K"):
        Batch([l1, l2], "fp64")


def test_batch_timing_reports(gpu):
    cs = cases()[:2]
    liks = [c.lik(lib=gpu, precision="fp32") for c in cs]
    for lk in liks:
        lk.prepare_plan()
    b = Batch(liks, "fp32")
    t = b.time(3)
    b.close()
    assert t["ms_per_run"] > 0 and t["walk_ms"] > 0
    assert math.isfinite(t["ms_per_run"])
