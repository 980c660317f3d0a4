"""Lik pickling (Lik.pyx:326-386, 573-585) and simulation (Lik.pyx:662-833)
on the CPU oracle.

* A pickled Lik carries its tree and models, not its alignment;
  ``unpickle`` on a Lik with the alignment completes it, and the result
  gives the same lnL bit for bit, with Γ, +I, two models and median
  categories.  The tree keeps its ring order through pickling.
* ``simulate`` cannot be pinned to the reference's values (it draws from
  Python 2's ``random``), so its output is checked against the model it
  simulates from: the shape and padding of the alignment, each leaf's
  base composition against the stationary frequencies, and each pair of
  leaves' fraction of identical sites against sum_i pi_i P(d)_ii, with P
  from CxLikPt at the pair's path length d, as the reference's
  _simulateChild uses it.  Seeded draws repeat.
"""
import math
import pickle
import random

import numpy as np

from crux_gb300 import synth
from crux_gb300.lik import Lik


def mixture_lik(lib):
    case = synth.Case(12, 800, 0.1, 91, pinv=0.2)
    aln = case.alignment()
    lik = Lik(case.tree(aln.taxaMap), aln, nmodels=2, ncat=4, invar=True,
              lib=lib)
    synth.apply_params(lik, 0, case.params, 0.7, 0.2)
    lik.setRclass(1, [0, 1, 0, 0, 1, 0], [1.0, 4.0])
    lik.setAlpha(1, 1.9)
    lik.setWeight(1, 0.4)
    lik.setRmult(1, 1.3)
    lik.setWVar(1, 0.9)
    lik.setWInvar(1, 0.1)
    for j, f in enumerate((0.1, 0.2, 0.3, 0.4)):
        lik.setFreq(1, j, f)
    return lik


def test_pickle_round_trip_same_lnl(port):
    lik = mixture_lik(port)
    want = lik.lnL()
    data = pickle.dumps(lik)
    ret = lik.unpickle(data)
    assert ret is not lik and ret.lib is lik.lib
    assert ret.tree.render() == lik.tree.render()
    assert ret.nmodels() == 2
    for i in range(2):
        assert ret.getRclass(i) == lik.getRclass(i)
        assert ret.getAlpha(i) == lik.getAlpha(i)
        assert ret.getWVar(i) == lik.getWVar(i)
        assert ret.getWInvar(i) == lik.getWInvar(i)
        assert ret.getRmult(i) == lik.getRmult(i)
    assert ret.lnL() == want
    assert ret.siteLnLs() == lik.siteLnLs()


def test_pickled_partial_lik_has_no_alignment(port):
    lik = mixture_lik(port)
    part = pickle.loads(pickle.dumps(lik))
    assert part.lib is None and not hasattr(part, "alignment")
    assert part.getWeight(1) == lik.getWeight(1)
    assert part.getFreq(1, 3) == lik.getFreq(1, 3)


def test_tree_pickle_keeps_ring_order():
    case = synth.Case(40, 50, 0.1, 92)
    aln = case.alignment()
    t = case.tree(aln.taxaMap)
    t2 = pickle.loads(pickle.dumps(t))
    assert t2.render() == t.render()
    assert [e.length for e in t2.edges] == [e.length for e in t.edges]
    assert t2.getBase().taxon == t.getBase().taxon


def _path_lengths(tree):
    """Leaf-to-leaf path lengths of an unrooted tree."""
    adj = {}
    for e in tree.edges:
        a, b = e.ring.node, e.ring.other.node
        adj.setdefault(id(a), []).append((b, e.length))
        adj.setdefault(id(b), []).append((a, e.length))
    leaves = [n for n in tree.nodes if n.taxon is not None]
    out = {}
    for s in leaves:
        dist = {id(s): 0.0}
        stack = [s]
        while stack:
            n = stack.pop()
            for m, ln in adj[id(n)]:
                if id(m) not in dist:
                    dist[id(m)] = dist[id(n)] + ln
                    stack.append(m)
        for t in leaves:
            out[(s.taxon, t.taxon)] = dist[id(t)]
    return out


def test_simulate_follows_the_model(port):
    case = synth.Case(6, 400, 0.3, 93)
    aln = case.alignment()
    lik = case.lik(lib=port, alignment=aln)
    nsim = 20000
    sim = lik.simulate(nsim, rng=random.Random(5))
    a = sim.alignment
    # Shape: the taxa, nsim simulated columns, stripe padding of 'N'.
    assert a.taxaMap.taxa == aln.taxaMap.taxa
    assert a.nchars - a.npad == nsim
    assert (a.rows[:, nsim:] == ord("N")).all()
    body = a.rows[:, :nsim]
    assert set(np.unique(body).tolist()) <= set(b"ACGT")
    # Seeded draws repeat.
    again = lik.simulate(nsim, rng=random.Random(5))
    assert np.array_equal(again.alignment.rows, a.rows)
    # The model: pi and P(t) = CxLikPt(cube, eigenvalues, t), as simulated.
    lik.prep()
    m = lik.lik.comps[0].model.contents
    pi = np.array([m.piDiagNorm[i] for i in range(4)])
    codes = np.frombuffer(b"ACGT", dtype=np.uint8)
    idx = np.searchsorted(codes, body)
    for r in range(a.ntaxa):
        comp = np.bincount(idx[r], minlength=4) / nsim
        se = np.sqrt(pi * (1 - pi) / nsim)
        assert np.all(np.abs(comp - pi) <= 5 * se), (r, comp, pi)
    dist = _path_lengths(lik.tree)
    P = np.zeros(16)
    from crux_gb300 import _abi
    taxa = a.taxaMap.taxa
    for i in range(a.ntaxa):
        for j in range(i + 1, a.ntaxa):
            d = dist[(taxa[i], taxa[j])]
            port.CxLikPt(4, _abi.dptr(P), m.qEigVecCube, m.qEigVals, d)
            want = float(np.sum(pi * np.diag(P.reshape(4, 4))))
            got = float(np.mean(idx[i] == idx[j]))
            se = math.sqrt(want * (1 - want) / nsim)
            assert abs(got - want) <= 5 * se, (taxa[i], taxa[j], got, want)


def test_simulated_lik_evaluates(port):
    case = synth.Case(8, 300, 0.2, 94, pinv=0.25)
    lik = case.lik(lib=port)
    sim = lik.simulate(500, rng=random.Random(1))
    assert sim.nmodels() == lik.nmodels()
    v = sim.lnL()
    assert math.isfinite(v) and v < 0
    # The simulated Lik's models are this Lik's (dup semantics).
    assert sim.getAlpha(0) == lik.getAlpha(0)
    assert sim.getWInvar(0) == lik.getWInvar(0)
