"""On-device MC3: Python front end of cxgMc3* (include/cxlik_gpu.h).

``Mc3(case_or_lik_inputs, ...)`` builds the chains on the GPU from an
unrooted tree and a compressed alignment, ``run(ngen)`` advances them, and
``chain_state(i)`` / ``chain_lik(i, lib)`` read a chain back -- the latter as
a ``Lik`` on any library, which is how tests check the device lnL against
the FP64 oracle.

Defaults follow the reference's Mc3 (pkg/Crux/Mc3/__init__.pyx:237-290):
multiplier tuning 2 ln 1.6, branch-length prior Exp(10), prior Exp(1) on
1/alpha, heats 1/(1 + i heatDelta).
"""
import ctypes
import math

import numpy as np

from . import _native
from .alignment import Alignment, TaxaMap
from .tree import Tree

LAMBDA = 2.0 * math.log(1.6)
MOVES = ("brlen", "nni", "rates", "alpha", "freqs", "spr", "etbr", "invar",
         "gammajump", "freqjump", "invarjump", "ratejump", "rate", "weight",
         "rmult", "mixturejump", "polytomyjump")
MAX_MODELS = 4


class Mc3Config(ctypes.Structure):
    _fields_ = [
        ("ntaxa", ctypes.c_uint),
        ("npat", ctypes.c_uint),
        ("masks", ctypes.POINTER(ctypes.c_uint8)),
        ("freqs_pattern", ctypes.POINTER(ctypes.c_uint32)),
        ("parent", ctypes.POINTER(ctypes.c_int32)),
        ("len", ctypes.POINTER(ctypes.c_double)),
        ("root", ctypes.c_uint),
        ("rates", ctypes.c_double * 6),
        ("freqs", ctypes.c_double * 4),
        ("alpha", ctypes.c_double),
        ("ncat", ctypes.c_uint),
        ("nchains", ctypes.c_uint),
        ("heat_delta", ctypes.c_double),
        ("swap_stride", ctypes.c_uint),
        ("seed", ctypes.c_ulonglong),
        ("move_weight", ctypes.c_double * 17),
        ("brlen_lambda", ctypes.c_double),
        ("brlen_prior", ctypes.c_double),
        ("rate_conc", ctypes.c_double),
        ("freq_conc", ctypes.c_double),
        ("etbr_pext", ctypes.c_double),
        ("alpha_lambda", ctypes.c_double),
        ("alpha_prior", ctypes.c_double),
        ("pinv", ctypes.c_double),
        ("invar_lambda", ctypes.c_double),
        ("invar_prior", ctypes.c_double),
        ("gamma_jump_prior", ctypes.c_double),
        ("freq_jump_prior", ctypes.c_double),
        ("precision", ctypes.c_int),
        ("graph_gens", ctypes.c_uint),
        ("trace_cap", ctypes.c_ulonglong),
        ("invar_jump_prior", ctypes.c_double),
        ("rclass", ctypes.c_int * 6),
        ("rate_jump_prior", ctypes.c_double),
        ("rate_lambda", ctypes.c_double),
        ("max_models", ctypes.c_uint),
        ("mixture_jump_prior", ctypes.c_double),
        ("weight_lambda", ctypes.c_double),
        ("rmult_lambda", ctypes.c_double),
        ("polytomy_jump_prior", ctypes.c_double),
    ]


class Mc3ModelState(ctypes.Structure):
    _fields_ = [
        ("rates", ctypes.c_double * 6),
        ("freqs", ctypes.c_double * 4),
        ("alpha", ctypes.c_double),
        ("wvar", ctypes.c_double),
        ("winvar", ctypes.c_double),
        ("weight", ctypes.c_double),
        ("rmult", ctypes.c_double),
        ("rclass", ctypes.c_int * 6),
        ("nrates", ctypes.c_int),
        ("freqs_est", ctypes.c_int),
    ]


def declare(lib):
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    lib.cxgMc3Create.argtypes = [P(Mc3Config), P(vp)]
    lib.cxgMc3Create.restype = ctypes.c_int
    lib.cxgMc3Run.argtypes = [vp, ctypes.c_ulonglong, P(ctypes.c_double)]
    lib.cxgMc3Run.restype = ctypes.c_int
    lib.cxgMc3Chain.argtypes = [vp, ctypes.c_uint, P(ctypes.c_double),
                                P(ctypes.c_double), P(ctypes.c_int32),
                                P(ctypes.c_double), P(ctypes.c_double),
                                P(ctypes.c_double), P(ctypes.c_double)]
    lib.cxgMc3Chain.restype = ctypes.c_int
    lib.cxgMc3ChainWeights.argtypes = [vp, ctypes.c_uint, P(ctypes.c_double),
                                       P(ctypes.c_double)]
    lib.cxgMc3ChainWeights.restype = ctypes.c_int
    lib.cxgMc3ChainModel.argtypes = [vp, ctypes.c_uint, ctypes.c_uint,
                                     P(ctypes.c_uint), P(Mc3ModelState)]
    lib.cxgMc3ChainModel.restype = ctypes.c_int
    lib.cxgMc3SetChain.argtypes = [vp, ctypes.c_uint, P(ctypes.c_int32),
                                   P(ctypes.c_double), P(ctypes.c_uint8),
                                   ctypes.c_double, ctypes.c_uint,
                                   P(Mc3ModelState)]
    lib.cxgMc3ChainCollapsed.argtypes = [vp, ctypes.c_uint, P(ctypes.c_uint8)]
    lib.cxgMc3ChainCollapsed.restype = ctypes.c_int
    lib.cxgMc3SetChain.restype = ctypes.c_int
    lib.cxgMc3SetCounts.argtypes = [vp, P(ctypes.c_uint), P(ctypes.c_uint),
                                    P(ctypes.c_uint)]
    lib.cxgMc3SetCounts.restype = ctypes.c_int
    lib.cxgMc3Resume.argtypes = [vp, ctypes.c_ulonglong]
    lib.cxgMc3Resume.restype = ctypes.c_int
    lib.cxgMc3Stats.argtypes = [vp, P(ctypes.c_uint), P(ctypes.c_uint),
                                P(ctypes.c_uint), P(ctypes.c_ulonglong)]
    lib.cxgMc3Stats.restype = ctypes.c_int
    lib.cxgMc3Trace.argtypes = [vp, P(ctypes.c_double), ctypes.c_ulonglong]
    lib.cxgMc3Trace.restype = ctypes.c_int
    lib.cxgMc3Destroy.argtypes = [vp]
    lib.cxgMc3Destroy.restype = ctypes.c_int


def tree_arrays(tree, taxaMap):
    """Rooted arrays of an unrooted binary tree: leaves are nodes
    0..ntaxa-1 in taxaMap order, internal nodes follow; the root is the
    neighbour of the tree's base leaf."""
    n = taxaMap.ntaxa
    nn = 2 * n - 2
    parent = np.full(nn, -1, dtype=np.int32)
    length = np.zeros(nn, dtype=np.float64)
    base = tree.base
    start = base.ring.other.node if base.taxon is not None else base
    if start.degree_calc() != 3:
        raise ValueError("MC3 needs a binary tree (root of degree 3)")
    ids = {}
    nxt = [n]

    def ident(node):
        if node.taxon is not None:
            return taxaMap.indGet(node.taxon)
        if id(node) not in ids:
            ids[id(node)] = nxt[0]
            nxt[0] += 1
        return ids[id(node)]

    root = ident(start)
    stack = [(start, None)]
    while stack:
        node, via = stack.pop()
        me = ident(node)
        for r in node.ring:
            if via is not None and r.edge is via:
                continue
            ch = r.other.node
            cid = ident(ch)
            parent[cid] = me
            length[cid] = r.edge.length
            if ch.degree_calc() > 1:
                if ch.degree_calc() != 3:
                    raise ValueError("MC3 needs a binary tree")
                stack.append((ch, r.edge))
    if nxt[0] != nn:
        raise ValueError("tree has %d nodes, expected %d" % (nxt[0], nn))
    return parent, length, root


def newick_from_arrays(parent, length, taxa):
    """Unrooted Newick text of rooted arrays (full-precision lengths)."""
    nn = len(parent)
    kids = [[] for _ in range(nn)]
    root = -1
    for v in range(nn):
        if parent[v] < 0:
            root = v
        else:
            kids[parent[v]].append(v)

    def rec(v):
        if not kids[v]:
            return taxa[v]
        return "(" + ",".join("%s:%r" % (rec(u), float(length[u]))
                              for u in kids[v]) + ")"

    return rec(root) + ";"


class Mc3:
    def __init__(self, tree, alignment, rates, freqs, alpha=None, ncat=4,
                 nchains=4, heat_delta=0.05, swap_stride=1, seed=1,
                 moves=None, precision="fp32", brlen_lambda=LAMBDA,
                 brlen_prior=10.0, rate_conc=300.0, freq_conc=300.0,
                 etbr_pext=0.8, pinv=0.0, invar_lambda=LAMBDA, invar_prior=0.5,
                 gamma_jump_prior=1.0, freq_jump_prior=1.0, invar_jump_prior=1.0,
                 rclass=(0, 1, 2, 3, 4, 5), rate_jump_prior=1.0, rate_lambda=LAMBDA,
                 max_models=1, mixture_jump_prior=1.0 / 3.0,
                 weight_lambda=LAMBDA, rmult_lambda=LAMBDA,
                 polytomy_jump_prior=1.0,
                 alpha_lambda=LAMBDA,
                 alpha_prior=1.0, graph_gens=16, trace_cap=1 << 20, lib=None):
        self.lib = lib or _native.load()
        declare(self.lib)
        self.alignment = alignment
        self.taxa = alignment.taxaMap.taxa
        parent, length, root = tree_arrays(tree, alignment.taxaMap)
        ch = alignment.charType.get()
        vals = ch.val_table[alignment.rows]
        if (vals < 0).any():
            raise ValueError("alignment holds undefined state codes")
        self._masks = np.ascontiguousarray(vals, dtype=np.uint8)
        self._freqs = np.ascontiguousarray(alignment.freqs, dtype=np.uint32)
        self._parent = parent
        self._len = length
        c = Mc3Config()
        c.ntaxa = len(self.taxa)
        c.npat = alignment.nchars
        c.masks = self._masks.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
        c.freqs_pattern = self._freqs.ctypes.data_as(
            ctypes.POINTER(ctypes.c_uint32))
        c.parent = parent.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        c.len = length.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        c.root = root
        for i in range(6):
            c.rates[i] = float(rates[i])
        for i in range(4):
            c.freqs[i] = float(freqs[i])
        c.alpha = float(alpha) if alpha is not None else 1.0
        c.ncat = ncat if alpha is not None else 1
        c.nchains = nchains
        c.heat_delta = heat_delta
        c.swap_stride = swap_stride
        c.seed = seed
        mv = moves or {"brlen": 1.0, "nni": 1.0}
        for i, name in enumerate(MOVES):
            c.move_weight[i] = float(mv.get(name, 0.0))
        c.brlen_lambda = brlen_lambda
        c.brlen_prior = brlen_prior
        c.rate_conc = rate_conc
        c.freq_conc = freq_conc
        c.etbr_pext = etbr_pext
        c.pinv = pinv
        c.invar_lambda = invar_lambda
        c.invar_prior = invar_prior
        c.gamma_jump_prior = gamma_jump_prior
        c.freq_jump_prior = freq_jump_prior
        c.invar_jump_prior = invar_jump_prior
        for i in range(6):
            c.rclass[i] = int(rclass[i])
        c.rate_jump_prior = rate_jump_prior
        c.rate_lambda = rate_lambda
        c.max_models = max_models
        c.mixture_jump_prior = mixture_jump_prior
        c.weight_lambda = weight_lambda
        c.rmult_lambda = rmult_lambda
        c.polytomy_jump_prior = polytomy_jump_prior
        c.alpha_lambda = alpha_lambda
        c.alpha_prior = alpha_prior
        c.precision = 1 if precision == "fp32" else 0
        c.graph_gens = graph_gens
        c.trace_cap = trace_cap
        self.cfg = c
        self.nchains = nchains
        self.ncat = c.ncat
        self.invar = pinv > 0.0
        self.h = ctypes.c_void_p()
        rc = self.lib.cxgMc3Create(ctypes.byref(c), ctypes.byref(self.h))
        if rc != 0:
            raise _native.error(self.lib, rc, "cxgMc3Create")

    def _check(self, rc, what):
        if rc != 0:
            raise _native.error(self.lib, rc, what)

    def run(self, ngen):
        secs = ctypes.c_double()
        self._check(self.lib.cxgMc3Run(self.h, ngen, ctypes.byref(secs)),
                    "cxgMc3Run")
        return secs.value

    def chain_state(self, i):
        nn = len(self._parent)
        lnl, heat, alpha = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        par = np.zeros(nn, dtype=np.int32)
        ln = np.zeros(nn)
        rates = np.zeros(6)
        freqs = np.zeros(4)
        dp = ctypes.POINTER(ctypes.c_double)
        self._check(self.lib.cxgMc3Chain(
            self.h, i, ctypes.byref(lnl), ctypes.byref(heat),
            par.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
            ln.ctypes.data_as(dp), rates.ctypes.data_as(dp),
            freqs.ctypes.data_as(dp), ctypes.byref(alpha)), "cxgMc3Chain")
        wv, wi = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.cxgMc3ChainWeights(self.h, i, ctypes.byref(wv),
                                                ctypes.byref(wi)),
                    "cxgMc3ChainWeights")
        # Rate classes: exchangeabilities of one class hold one value.
        seen = {}
        rclass = [seen.setdefault(float(x), len(seen)) for x in rates]
        coll = np.zeros(nn, dtype=np.uint8)
        self._check(self.lib.cxgMc3ChainCollapsed(
            self.h, i, coll.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))),
            "cxgMc3ChainCollapsed")
        return {"lnL": lnl.value, "heat": heat.value, "parent": par,
                "len": ln, "rates": rates, "rclass": rclass, "freqs": freqs,
                "alpha": alpha.value, "wvar": wv.value, "winvar": wi.value,
                "models": self.chain_models(i), "collapsed": coll}

    def chain_models(self, i):
        """Chain i's mixture members: one dict of parameters each."""
        n = ctypes.c_uint()
        self._check(self.lib.cxgMc3ChainModel(self.h, i, 0, ctypes.byref(n),
                                              None), "cxgMc3ChainModel")
        out = []
        for m in range(n.value):
            st = Mc3ModelState()
            self._check(self.lib.cxgMc3ChainModel(self.h, i, m, None,
                                                  ctypes.byref(st)),
                        "cxgMc3ChainModel")
            out.append({"rates": [st.rates[j] for j in range(6)],
                        "rclass": [st.rclass[j] for j in range(6)],
                        "nrates": st.nrates,
                        "freqs": [st.freqs[j] for j in range(4)],
                        "freqs_est": bool(st.freqs_est),
                        "alpha": st.alpha, "wvar": st.wvar,
                        "winvar": st.winvar, "weight": st.weight,
                        "rmult": st.rmult})
        return out

    def checkpoint(self):
        """The run's state as plain data: the generation count, each
        chain's tree, heat and mixture members, and the move and swap
        counts.  CLs are not saved; ``restore`` recomputes them."""
        st = self.stats()
        chains = []
        for i in range(self.nchains):
            cs = self.chain_state(i)
            chains.append({"parent": cs["parent"].tolist(),
                           "len": cs["len"].tolist(), "heat": cs["heat"],
                           "collapsed": cs["collapsed"].tolist(),
                           "lnL": cs["lnL"], "models": cs["models"]})
        return {"generation": int(st["generation"]), "chains": chains,
                "accepts": st["accepts"].tolist(),
                "rejects": st["rejects"].tolist(),
                "swaps": st["swaps"].tolist()}

    def restore(self, ckpt):
        """Continue a checkpointed run in this one (built with the same
        configuration and seed): every chain takes its saved state, the
        CLs are recomputed, and the next generation draws what the
        uninterrupted run draws there."""
        if len(ckpt["chains"]) != self.nchains:
            raise ValueError("checkpoint has %d chains, this run %d"
                             % (len(ckpt["chains"]), self.nchains))
        for i, ch in enumerate(ckpt["chains"]):
            par = np.ascontiguousarray(ch["parent"], dtype=np.int32)
            ln = np.ascontiguousarray(ch["len"], dtype=np.float64)
            co = np.ascontiguousarray(ch.get("collapsed", np.zeros(len(par))),
                                      dtype=np.uint8)
            ms = (Mc3ModelState * len(ch["models"]))()
            for k, q in enumerate(ch["models"]):
                for j in range(6):
                    ms[k].rates[j] = q["rates"][j]
                    ms[k].rclass[j] = q["rclass"][j]
                for j in range(4):
                    ms[k].freqs[j] = q["freqs"][j]
                ms[k].alpha = q["alpha"]
                ms[k].wvar = q["wvar"]
                ms[k].winvar = q["winvar"]
                ms[k].weight = q["weight"]
                ms[k].rmult = q["rmult"]
                ms[k].nrates = q["nrates"]
                ms[k].freqs_est = int(q["freqs_est"])
            self._check(self.lib.cxgMc3SetChain(
                self.h, i, par.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                ln.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                co.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                float(ch["heat"]), len(ch["models"]), ms), "cxgMc3SetChain")
        n = self.nchains * len(MOVES)
        acc = (ctypes.c_uint * n)(*np.ravel(ckpt["accepts"]).tolist())
        rej = (ctypes.c_uint * n)(*np.ravel(ckpt["rejects"]).tolist())
        sw = (ctypes.c_uint * self.nchains)(*ckpt["swaps"])
        self._check(self.lib.cxgMc3SetCounts(self.h, acc, rej, sw),
                    "cxgMc3SetCounts")
        self._check(self.lib.cxgMc3Resume(self.h, int(ckpt["generation"])),
                    "cxgMc3Resume")

    def stats(self):
        n = self.nchains * len(MOVES)
        acc = (ctypes.c_uint * n)()
        rej = (ctypes.c_uint * n)()
        sw = (ctypes.c_uint * self.nchains)()
        gen = ctypes.c_ulonglong()
        self._check(self.lib.cxgMc3Stats(self.h, acc, rej, sw,
                                         ctypes.byref(gen)), "cxgMc3Stats")
        a = np.array(acc).reshape(self.nchains, len(MOVES))
        r = np.array(rej).reshape(self.nchains, len(MOVES))
        return {"accepts": a, "rejects": r, "swaps": np.array(sw),
                "generation": gen.value}

    def trace(self, n):
        out = np.zeros(n)
        self._check(self.lib.cxgMc3Trace(
            self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n),
            "cxgMc3Trace")
        return out

    def chain_lik(self, i, lib, precision="fp64"):
        """A Lik holding chain i's tree and model, on library `lib`."""
        from .lik import Lik
        st = self.chain_state(i)
        nw = newick_from_arrays(st["parent"], st["len"], self.taxa)
        rows = self.alignment.rows.copy()
        aln = Alignment(taxaMap=TaxaMap(self.taxa), rows=rows)
        aln.freqs = self.alignment.freqs.copy()
        t = Tree(nw)
        t.deroot()
        t.canonize(aln.taxaMap)
        models = st["models"]
        lik = Lik(t, aln, nmodels=len(models), ncat=self.ncat,
                  invar=self.invar, lib=lib, precision=precision)
        for m, q in enumerate(models):
            lik.setRclass(m, [0, 1, 2, 3, 4, 5],
                          [float(x) for x in q["rates"]])
            for j in range(4):
                lik.setFreq(m, j, float(q["freqs"][j]))
            if self.ncat > 1:
                lik.setAlpha(m, float(q["alpha"]))
            if self.invar:
                lik.setWVar(m, q["wvar"])
                lik.setWInvar(m, q["winvar"])
            if len(models) > 1:
                lik.setWeight(m, q["weight"])
                lik.setRmult(m, q["rmult"])
        return lik, st

    def close(self):
        if self.h:
            self.lib.cxgMc3Destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
