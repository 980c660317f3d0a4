"""CPU checks of the MC3 host side: tree <-> rooted-array conversion keeps
the likelihood (FP64 oracle), and the arrays describe a binary tree."""
import math

import numpy as np

from crux_gb300 import mc3, synth
from crux_gb300.tree import Tree


def test_tree_arrays_round_trip(port):
    case = synth.Case(20, 600, 0.1, 3)
    aln = case.alignment()
    t = case.tree(aln.taxaMap)
    parent, length, root = mc3.tree_arrays(t, aln.taxaMap)
    n = aln.ntaxa
    assert len(parent) == 2 * n - 2 and parent[root] == -1
    kids = np.bincount(parent[parent >= 0], minlength=2 * n - 2)
    assert (kids[:n] == 0).all()
    assert kids[root] == 3
    assert all(kids[v] == 2 for v in range(n, 2 * n - 2) if v != root)
    nw = mc3.newick_from_arrays(parent, length, aln.taxaMap.taxa)
    t2 = Tree(nw)
    t2.deroot()
    t2.canonize(aln.taxaMap)
    a = case.lik(lib=port, alignment=aln).lnL()
    from crux_gb300.lik import Lik
    lik = Lik(t2, case.alignment(), ncat=4, lib=port)
    synth.apply_params(lik, 0, case.params, case.alpha)
    b = lik.lnL()
    assert math.isclose(a, b, rel_tol=1e-12)
