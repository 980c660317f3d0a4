"""Known-answer cases of the reference's likelihood tests.

Inputs and printed answers of canonware/crux test/Lik_*.cx and their .exp
files.  Each runner builds the trees exactly as those scripts do
(``Tree(newick)``, ``deroot()``, ``canonize(alignment taxa map)``) and
returns the values the scripts print, so a test can compare them with the
.exp text at the printed precision and, more tightly, across backends.
"""
import math

from crux_gb300.alignment import Alignment, CTMatrix
from crux_gb300.lik import Lik
from crux_gb300.tree import Tree

FIVE = """>A
    ata
>B
    cta
>C
    cat
>D
    gat
>E
    gtr
"""

THREE = """>one
ACGT
>two
ACGT
>three
AAAA
"""

FIVE_TREES = [
    "(A:0.1,B:0.1,(C:0.25,(D:0.2,E:0.3):0.1):0.4):0.0;",
    "(A:3.3333331e-01,B:2.9802322e-08,((C:2.9166669e-01,D:4.1666865e-02)"
    ":9.3981469e-01,E:3.5648149e-01):4.3981487e-01);",
    "(A:1,B:0,(C:0,(D:0,E:2):1):2);",
    "(A:0,B:1,((C:1,D:0):2,E:0):1);",
]

# test/Lik_b.cx.exp: lnL (5 dp) and site lnLs (6 dp) per tree.
LIK_B = [
    (-20.98087, [-8.591872, -6.490368, -5.898628]),
    (-17.64423, [-9.186881, -4.375946, -4.081402]),
    (-18.29198, [-7.164750, -5.910187, -5.217040]),
    (-17.82664, [-7.660067, -5.255514, -4.911062]),
]

# test/Lik_e.cx.exp: +G4, alpha in (0.5, 1, 5, 300); means then medians.
ALPHAS = (0.5, 1.0, 5.0, 300.0)
LIK_E = [
    ([-21.91979, -21.52568, -21.11582, -20.98329],
     [-21.78182, -21.44264, -21.09430, -20.98288]),
    ([-18.29427, -17.90326, -17.64944, -17.64395],
     [-18.29490, -17.89324, -17.64738, -17.64400]),
    ([-19.60181, -18.93819, -18.29005, -18.29059],
     [-19.58217, -18.91875, -18.28400, -18.29082]),
    ([-17.76422, -17.36831, -17.51841, -17.81987],
     [-17.83552, -17.38507, -17.55429, -17.82103]),
]

# test/Lik_h.cx: gaps and N as missing data; both alignments, same answers.
GAPPY = [""">A
    at-
>B
    c--
>C
    cat
>D
    -a-
>E
    -tr
""", """>A
    atn
>B
    cnn
>C
    cat
>D
    nan
>E
    ntr
"""]
LIK_H = [-14.10650, -11.35155, -11.42647, -11.01951]

# test/Lik_c.cx.exp (every node as root).
LIK_C = (-11.2694, [-2.323664, -2.981923, -2.981923, -2.981923])

# test/Lik_j.cx.exp: freqs (0.4, 0.3, 0.2, 0.1); three:{0.25 .. 1.25}.
LIK_J = [
    (0.25, -12.58849, [-1.114981, -3.323145, -3.728611, -4.421758]),
    (0.5, -11.16418, [-1.281970, -2.792710, -3.198175, -3.891322]),
    (0.75, -10.54086, [-1.417973, -2.539603, -2.945068, -3.638215]),
    (1.0, -10.21228, [-1.525482, -2.394241, -2.799706, -3.492854]),
    (1.25, -10.02370, [-1.608226, -2.303799, -2.709264, -3.402411]),
]

# test/Lik_l.cx.exp: +I direct and emulated, pinvar in (0, .25, .5, .75).
LIK_L = [
    (0.0, -11.26943, [-2.323664, -2.981923, -2.981923, -2.981923]),
    (0.25, -11.60745, [-2.082532, -3.174973, -3.174973, -3.174973]),
    (0.5, -12.34130, [-1.835119, -3.502062, -3.502062, -3.502062]),
    (0.75, -14.07411, [-1.593640, -4.160157, -4.160157, -4.160157]),
]

# test/Lik_m.cx.exp, first value (12 significant digits).
LIK_M_FASTA = ">A1\nACGT\n>A2\nACGT\n>B\nAAAA\n>C\nGGGG\n>D\nCCCC\n"
LIK_M_TREE = "(((A1:0.0,A2:0.0):0.05,B:0.15):0.75,(C:0.05,D:0.05));"
LIK_M = -34.190306481
LIK_M_RENDER = ("(A1:0.0000000e+00,A2:0.0000000e+00,(B:1.5000000e-01,"
                "(C:5.0000000e-02,D:5.0000000e-02):7.5000000e-01)"
                ":5.0000000e-02);")

# test/Lik_d.cx / Lik_k.cx trees as printed (they are built by RNJ there).
LIK_D_TREES = [("one:1.2500e+00", ">one\nACGT\n>two\nAAAA\n",
                "(one:1.25,two:0.0);", -11.2694),
               ("five", FIVE,
                "(A:3.3333e-01,B:2.9802e-08,((C:2.9167e-01,D:4.1667e-02)"
                ":1.1713e+00,E:1.2500e-01):2.0833e-01);", -17.5466)]
LIK_K = [(">one\nACGT\n>two\nAAAA\n", "(one:1.25,two:0.0);", -11.435,
          [-1.231, -2.969, -3.290, -3.945]),
         (FIVE, "(A:3.3333e-01,B:2.9802e-08,((C:2.9167e-01,D:4.1667e-02)"
          ":1.1713e+00,E:1.2500e-01):2.0833e-01);", -20.642,
          [-8.597, -6.459, -5.586])]


def tree_for(newick, aln):
    t = Tree(newick)
    t.deroot()
    t.canonize(aln.taxaMap)
    return t


def run_lik_b(lib, precision="fp64"):
    out = []
    for nw in FIVE_TREES:
        aln = Alignment(CTMatrix(FIVE))
        lik = Lik(tree_for(nw, aln), aln, lib=lib, precision=precision)
        out.append((lik.lnL(), lik.siteLnLs()))
    return out


def run_lik_e(lib, precision="fp64"):
    out = []
    for nw in FIVE_TREES:
        aln = Alignment(CTMatrix(FIVE))
        t = tree_for(nw, aln)
        per = []
        for med in (False, True):
            lik = Lik(t, aln, ncat=4, catMedian=med, lib=lib,
                      precision=precision)
            vals = []
            for a in ALPHAS:
                lik.setAlpha(0, a)
                vals.append(lik.lnL())
            per.append(vals)
        out.append(tuple(per))
    return out


def run_lik_h(lib, precision="fp64"):
    out = []
    for fasta in GAPPY:
        row = []
        for nw in FIVE_TREES:
            aln = Alignment(CTMatrix(fasta))
            lik = Lik(tree_for(nw, aln), aln, lib=lib, precision=precision)
            row.append(lik.lnL())
        out.append(row)
    return out


def run_every_root(lib, fasta, newick, freqs=None, precision="fp64"):
    """Lik_c / Lik_j: lnL and site lnLs with every node as root."""
    aln = Alignment(CTMatrix(fasta))
    t = tree_for(newick, aln)
    lik = Lik(t, aln, lib=lib, precision=precision)
    if freqs:
        for i, f in enumerate(freqs):
            lik.setFreq(0, i, f)
    return [(lik.lnL(n), lik.siteLnLs(n)) for n in t.nodes]


def run_lik_g(lib, precision="fp64"):
    aln = Alignment(CTMatrix(THREE))
    t = tree_for("(one:0.0,two:0.0,three:0.0);", aln)
    lik = Lik(t, aln, lib=lib, precision=precision)
    return [lik.lnL(n) for n in t.nodes]


def run_lik_l(lib, precision="fp64"):
    aln = Alignment(CTMatrix(THREE))
    t = tree_for("(one:0.0,two:0.0,three:1.25);", aln)
    lik = Lik(t, aln, invar=True, lib=lib, precision=precision)
    direct = []
    for pinv, _, _ in LIK_L:
        lik.setWVar(0, 1.0 - pinv)
        lik.setWInvar(0, pinv)
        direct.append((lik.lnL(), lik.siteLnLs()))
    lik.setWInvar(0, 0.0)
    lik.addModel(1.0)
    lik.setRate(1, 0, 0.0)
    emulated = []
    for pinv, _, _ in LIK_L:
        lik.setWeight(0, 1.0 - pinv)
        lik.setWeight(1, pinv)
        emulated.append((lik.lnL(), lik.siteLnLs()))
    return direct, emulated


def run_lik_m(lib, precision="fp64"):
    aln = Alignment(CTMatrix(LIK_M_FASTA))
    t = tree_for(LIK_M_TREE, aln)
    lik = Lik(t, aln, lib=lib, precision=precision)
    return t.render(), lik.lnL()


def run_lik_d(lib, precision="fp64"):
    """Normalisation invariance and mixtures (test/Lik_d.cx)."""
    out = []
    for _, fasta, nw, _ in LIK_D_TREES:
        aln = Alignment(CTMatrix(fasta))
        t = Tree(nw)
        t.deroot()
        t.canonize(aln.taxaMap)
        lik = Lik(t, aln, lib=lib, precision=precision)
        vals = [lik.lnL()]
        lik.setRate(0, 0, 0.75)
        for i in range(4):
            lik.setFreq(0, i, 0.20)
        vals.append(lik.lnL())
        lik.setRate(0, 0, 1.0)
        lik.addModel(0.0)
        vals.append(lik.lnL())
        lik.setWeight(0, 0.5)
        lik.setWeight(1, 0.5)
        vals.append(lik.lnL())
        lik.setWeight(0, 0.0)
        lik.setWeight(1, 0.3)
        lik.addModel(0.7)
        vals.append(lik.lnL())
        lik.setWeight(0, 1.0)
        lik.setWeight(1, 1.0)
        lik.setWeight(2, 1.0)
        vals.append(lik.lnL())
        lik.delModel(1)
        vals.append(lik.lnL())
        lik.delModel(1)
        vals.append(lik.lnL())
        out.append(vals)
    return out


def run_lik_k(lib, precision="fp64"):
    """+G2 equals a two-model mixture (test/Lik_k.cx)."""
    out = []
    for fasta, nw, _, _ in LIK_K:
        res = []
        for ncat, nmod in ((2, 1), (1, 2)):
            aln = Alignment(CTMatrix(fasta))
            t = Tree(nw)
            t.deroot()
            t.canonize(aln.taxaMap)
            lik = Lik(t, aln, nmodels=nmod, ncat=ncat, lib=lib,
                      precision=precision)
            for i in range(nmod):
                for j, f in enumerate((0.40, 0.30, 0.20, 0.10)):
                    lik.setFreq(i, j, f)
                lik.setRclass(i, [0, 1, 2, 3, 4, 5],
                              [0.1, 0.2, 0.3, 0.4, 0.5, 0.6])
            if ncat == 2:
                lik.setAlpha(0, 0.179062)
            else:
                lik.setRmult(0, 0.011437)
                lik.setRmult(1, 1.988563)
            res.append((lik.lnL(), lik.siteLnLs()))
        out.append(res)
    return out


def close(a, b, places):
    """True when a rounds to the printed value b at `places` decimals."""
    return abs(a - b) <= 0.5 * 10.0 ** (-places) + 1e-12 * abs(b) \
        or (math.isinf(a) and math.isinf(b))
