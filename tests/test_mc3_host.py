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


def test_rate_jump_terms_keep_the_prior():
    """The rate-class merge/split terms, as the device proposal computes
    them (cxg_mc3.cu, MV_RATEJ), with the class-rate multiplier and the
    sum-keeping Dirichlet move, run as a Markov chain without data: each
    number of classes 1..6 about equally often (rateJumpPrior 1), every
    two-class partition visited, class rates of mean 1."""
    S6 = [0, 1, 31, 90, 65, 15, 1]
    lam, conc = 2.0 * math.log(1.6), 300.0
    rng = np.random.default_rng(3)

    def rgs(rc):
        m = {}
        return [m.setdefault(x, len(m)) for x in rc]

    def lndir(a, x):
        return (math.lgamma(sum(a)) - sum(math.lgamma(v) for v in a) +
                sum((v - 1) * math.log(y) for v, y in zip(a, x)))

    rc, rates = [0, 1, 2, 3, 4, 5], [1.0] * 6
    n = 300_000
    ks = np.zeros(7)
    parts, rsum = set(), 0.0
    for _ in range(n):
        k = max(rc) + 1
        cr = [rates[rc.index(r)] for r in range(k)]
        cnt = [rc.count(r) for r in range(k)]
        mv = rng.integers(3)
        if mv == 0:
            merge = k == 6 or (k > 1 and rng.integers(2) == 0)
            if not merge:
                sp = [r for r in range(k) if cnt[r] > 1]
                c = sp[rng.integers(len(sp))]
                n0 = cnt[c]
                z = 1 + rng.integers((1 << n0) - 2)
                mem = [i for i in range(6) if rc[i] == c]
                A = [i for j, i in enumerate(mem) if (z >> j) & 1]
                B = [i for i in mem if i not in A]
                na, nb, r0, u = len(A), len(B), cr[c], rng.random()
                ra, rb = r0 * n0 * u / na, r0 * n0 * (1 - u) / nb
                ps, pm = (1.0 if k == 1 else 0.5), (1.0 if k + 1 == 6 else 0.5)
                lp = math.log(S6[k] / S6[k + 1]) + (r0 - ra - rb)
                lh = (math.log(pm / ((k + 1) * k / 2)) -
                      math.log(ps / (len(sp) * ((1 << (n0 - 1)) - 1))) +
                      math.log(n0 * n0 * r0 / (na * nb)))
                if math.exp(lp + lh) >= rng.random():
                    nrc, nr = list(rc), list(rates)
                    for i in A:
                        nr[i] = ra
                    for i in B:
                        nrc[i], nr[i] = k, rb
                    rc, rates = rgs(nrc), nr
            else:
                x = rng.integers(k)
                y = rng.integers(k - 1)
                y += y >= x
                a, b = min(x, y), max(x, y)
                na, nb = cnt[a], cnt[b]
                n0, ra, rb = na + nb, cr[a], cr[b]
                r0 = (na * ra + nb * rb) / n0
                nrc = [a if v == b else (v - 1 if v > b else v) for v in rc]
                nr = [r0 if nrc[i] == a else rates[i] for i in range(6)]
                ns1 = sum(1 for r in range(k - 1) if nrc.count(r) > 1)
                ps, pm = (1.0 if k - 1 == 1 else 0.5), (1.0 if k == 6 else 0.5)
                lp = math.log(S6[k] / S6[k - 1]) - (r0 - ra - rb)
                lh = (math.log(ps / (ns1 * ((1 << (n0 - 1)) - 1))) -
                      math.log(pm / (k * (k - 1) / 2)) -
                      math.log(n0 * n0 * r0 / (na * nb)))
                if math.exp(lp + lh) >= rng.random():
                    rc, rates = nrc, nr
        elif mv == 1 and k >= 2:
            r = rng.integers(k)
            lnm = lam * (rng.random() - 0.5)
            c1 = cr[r] * math.exp(lnm)
            if math.exp(-(c1 - cr[r]) + lnm) >= rng.random():
                rates = [c1 if rc[i] == r else rates[i] for i in range(6)]
        elif mv == 2 and k >= 2:
            s = sum(cr)
            f0 = [v / s for v in cr]
            a0 = [conc * v for v in f0]
            g = [max(rng.gamma(v), 1e-300) for v in a0]
            f1 = [v / sum(g) for v in g]
            if math.exp(lndir([conc * v for v in f1], f0) - lndir(a0, f1)) >= rng.random():
                rates = [s * f1[rc[i]] for i in range(6)]
        k = max(rc) + 1
        ks[k] += 1
        if k == 2:
            parts.add(tuple(rc))
        rsum += rates[0]
    frac = ks[1:] / n
    assert np.all(np.abs(frac - 1.0 / 6.0) < 0.05), frac
    assert len(parts) == 31
    assert abs(rsum / n - 1.0) < 0.1, rsum / n
