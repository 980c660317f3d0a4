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


def test_invar_jump_terms_keep_the_prior():
    """The +I jump's prior and Hastings terms, as the device proposal
    computes them (cxg_mc3.cu, MV_INVARJ), with the +I weight move's terms,
    run as a Markov chain without data: +I is on half the time
    (invarJumpPrior 1) and, when on, wVar and wInvar have the weight
    move's Exp priors of rates 1 - invarPrior and invarPrior (means 2)."""
    rng = np.random.default_rng(1)
    ip, lam = 0.5, 2.0 * math.log(1.6)

    def lnw(a, b):
        return math.log(1 - ip) - (1 - ip) * a + math.log(ip) - ip * b

    on, wv, wi = True, 0.7, 0.3
    n = 400_000
    U = rng.random((n, 4))
    non = swv = swi = 0.0
    for u in U:
        if u[0] < 0.5:                      # weight move (off: nothing)
            if on:
                lnm = lam * (u[2] - 0.5)
                if u[1] < 0.5:
                    w1 = wv * math.exp(lnm)
                    if math.exp(-(1 - ip) * (w1 - wv) + lnm) >= u[3]:
                        wv = w1
                else:
                    w1 = wi * math.exp(lnm)
                    if math.exp(-ip * (w1 - wi) + lnm) >= u[3]:
                        wi = w1
        elif on:                            # jump: remove
            d = lnw(wv, wi)
            if math.exp((math.log(1.0) - d) + d) >= u[3]:
                on, wv, wi = False, 1.0, 0.0
        else:                               # jump: add
            a = -math.log(1 - u[1]) / (1 - ip)
            b = -math.log(1 - u[2]) / ip
            d = lnw(a, b)
            if math.exp((-math.log(1.0) + d) - d) >= u[3]:
                on, wv, wi = True, a, b
        if on:
            non += 1
            swv += wv
            swi += wi
    assert abs(non / n - 0.5) < 0.02, non / n
    assert abs(swv / non - 2.0) < 0.1, swv / non
    assert abs(swi / non - 2.0) < 0.1, swi / non
