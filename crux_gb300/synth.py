"""Seeded synthetic workloads with the shapes the benchmarks name.

* ``yule_newick(n, mean, rng)``: a pure-birth (Yule) topology grown from a
  2-leaf root by splitting a uniformly chosen leaf lineage until n leaves,
  every branch length drawn Exp(mean); taxa are named T0..T(n-1).
* ``gtr_params(rng)``: exchangeabilities ~ Dirichlet(1 x 6) scaled to mean
  rate 1, base frequencies ~ Dirichlet(5, 5, 5, 5).
* ``simulate(newick, nsites, params, rng)``: sequences simulated down the
  tree under GTR (+Gamma categories, +I), with an optional fraction of cells
  replaced by gaps; returns FASTA text.
* ``build_case(...)``: tree + compressed alignment + a configured ``Lik``.

The simulator is this package's own (the reference's Lik.simulate uses the
Python-2 ``random`` module); only the model and the shapes are shared.
"""
import math

import numpy as np

from .alignment import Alignment, CTMatrix
from .cxmath import gamma_rates
from .tree import Tree

STATES = np.frombuffer(b"ACGT", dtype=np.uint8)


def yule_newick(ntaxa, mean_brlen, rng):
    """Newick text of a rooted Yule tree with Exp(mean) branch lengths."""
    assert ntaxa >= 2
    children = {0: []}
    leaves = [0]
    nxt = 1
    while len(leaves) < ntaxa:
        i = int(rng.integers(len(leaves)))
        node = leaves[i]
        a, b = nxt, nxt + 1
        nxt += 2
        children[node] = [a, b]
        children[a] = []
        children[b] = []
        leaves[i] = a
        leaves.append(b)
    names = {leaf: "T%d" % k for k, leaf in enumerate(sorted(leaves))}

    def rec(node):
        if not children[node]:
            return names[node]
        parts = []
        for c in children[node]:
            parts.append("%s:%r" % (rec(c), float(rng.exponential(mean_brlen))))
        return "(" + ",".join(parts) + ")"

    import sys
    old = sys.getrecursionlimit()
    sys.setrecursionlimit(max(old, 10 * ntaxa + 100))
    try:
        return rec(0) + ";"
    finally:
        sys.setrecursionlimit(old)


def gtr_params(rng):
    rates = rng.dirichlet(np.ones(6)) * 6.0
    freqs = rng.dirichlet(np.full(4, 5.0))
    return {"rates": [float(x) for x in rates],
            "freqs": [float(x) for x in freqs]}


def _eigensystem(rates, freqs):
    """Q normalised to one expected substitution per unit length."""
    pi = np.asarray(freqs, dtype=np.float64)
    pi = pi / pi.sum()
    R = np.zeros((4, 4))
    iu = np.triu_indices(4, 1)
    R[iu] = rates
    R = R + R.T
    Q = R * pi[None, :]
    np.fill_diagonal(Q, -Q.sum(1))
    Q /= -(pi * np.diag(Q)).sum()
    sq = np.sqrt(pi)
    S = sq[:, None] * Q / sq[None, :]
    S = 0.5 * (S + S.T)
    lam, U = np.linalg.eigh(S)
    V = U / sq[:, None]
    Vi = U.T * sq[None, :]
    return lam, V, Vi, pi


def _pmat(lam, V, Vi, t):
    P = (V * np.exp(lam * t)[None, :]) @ Vi
    P = np.clip(P, 0.0, None)
    return P / P.sum(1, keepdims=True)


def simulate(newick, nsites, params, rng, alpha=None, ncat=4, pinv=0.0,
             gap_frac=0.0):
    """FASTA text of nsites sites simulated on the (rooted) Newick tree."""
    tree = Tree(newick)
    lam, V, Vi, pi = _eigensystem(params["rates"], params["freqs"])
    if alpha is not None:
        cat_rates = np.asarray(gamma_rates(alpha, ncat), dtype=np.float64)
        cat = rng.integers(ncat, size=nsites)
        site_rate = cat_rates[cat]
    else:
        site_rate = np.ones(nsites)
    if pinv > 0.0:
        inv = rng.random(nsites) < pinv
        site_rate = np.where(inv, 0.0, site_rate / (1.0 - pinv))
    # Distinct rates get one P matrix per edge.
    uniq, rate_idx = np.unique(site_rate, return_inverse=True)
    seqs = {}
    root = tree.base
    start = rng.choice(4, size=nsites, p=pi)
    stack = [(root.ring.other, start)] if root.ring is not None else []
    if root.taxon is not None:
        seqs[root.taxon] = start
    while stack:
        ring, parent_states = stack.pop()
        t = ring.edge.length
        cdfs = np.stack([np.cumsum(_pmat(lam, V, Vi, r * t), 1) for r in uniq])
        u = rng.random(nsites)
        row = cdfs[rate_idx, parent_states]          # [nsites, 4]
        child = np.minimum((u[:, None] > row).sum(1), 3)
        node = ring.node
        if node.taxon is not None:
            seqs[node.taxon] = child
        for s in ring.siblings():
            stack.append((s.other, child))
    names = sorted(seqs, key=lambda x: int(x[1:]) if x[1:].isdigit() else x)
    lines = []
    for nm in names:
        chars = STATES[seqs[nm]].copy()
        if gap_frac > 0.0:
            gaps = rng.random(nsites) < gap_frac
            chars[gaps] = ord("-")
        lines.append(">" + nm)
        lines.append(chars.tobytes().decode("ascii"))
    return "\n".join(lines) + "\n"


class Case:
    """A seeded workload: unrooted canonized tree, compressed alignment."""

    def __init__(self, ntaxa, nsites, mean_brlen, seed, alpha=0.5, ncat=4,
                 pinv=0.0, gap_frac=0.0, params=None):
        rng = np.random.default_rng(seed)
        self.newick = yule_newick(ntaxa, mean_brlen, rng)
        self.params = params or gtr_params(rng)
        self.alpha, self.ncat, self.pinv = alpha, ncat, pinv
        fasta = simulate(self.newick, nsites, self.params, rng, alpha=alpha,
                         ncat=ncat, pinv=pinv, gap_frac=gap_frac)
        self.fasta = fasta
        self.nsites = nsites
        self.ntaxa = ntaxa

    def alignment(self):
        aln = Alignment(CTMatrix(self.fasta))
        aln.compact()
        return aln

    def tree(self, taxaMap):
        t = Tree(self.newick)
        t.deroot()
        t.canonize(taxaMap)
        return t

    def lik(self, lib=None, precision="fp64", alignment=None, dropin=False):
        from .lik import Lik
        aln = alignment if alignment is not None else self.alignment()
        t = self.tree(aln.taxaMap)
        invar = self.pinv > 0.0
        ncat = self.ncat if self.alpha is not None else 1
        lik = Lik(t, aln, ncat=ncat, invar=invar, lib=lib, precision=precision,
                  dropin=dropin)
        apply_params(lik, 0, self.params, self.alpha, self.pinv)
        return lik


def apply_params(lik, model, params, alpha=None, pinv=0.0):
    """Set GTR rates/frequencies, Gamma alpha and +I weights on a model."""
    lik.setRclass(model, [0, 1, 2, 3, 4, 5], [float(r) for r in params["rates"]])
    for i, f in enumerate(params["freqs"]):
        lik.setFreq(model, i, float(f))
    if alpha is not None and lik.getNcat(model) > 1:
        lik.setAlpha(model, float(alpha))
    if pinv > 0.0:
        lik.setWVar(model, 1.0 - pinv)
        lik.setWInvar(model, pinv)


def nnodes_updates(lik):
    """Pattern-node updates of the current plan: #Compute steps x patterns."""
    n = sum(1 for v, _, _ in lik.steps() if v in (0, 1))
    return n * lik.lik.mschars


def log_uniform_int(rng, lo, hi):
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
