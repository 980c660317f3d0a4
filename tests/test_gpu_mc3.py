"""On-device MC3: after generations of branch-length, NNI, SPR, eTBR, rate,
frequency and alpha moves, every chain's device lnL equals the FP64
oracle's lnL of that chain's tree and model (1e-11 relative for the plain FP64 chains, 1e-6 for
FP32 chains); moves are accepted and heats are swapped."""
import numpy as np
import pytest

from crux_gb300 import synth
from crux_gb300.mc3 import Mc3

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-11, "fp32": 1e-6}
MOVES = {"brlen": 2.0, "nni": 1.0, "spr": 1.0, "rates": 0.5, "alpha": 0.5,
         "freqs": 0.5, "etbr": 1.0}


def build(precision, nchains=4, seed=9, moves=MOVES, ntaxa=16, nsites=1000):
    case = synth.Case(ntaxa, nsites, 0.1, 5)
    aln = case.alignment()
    t = case.tree(aln.taxaMap)
    return Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=0.5,
               ncat=4, nchains=nchains, heat_delta=0.2, seed=seed,
               moves=moves, precision=precision, graph_gens=8)


def check_chains(m, port, tol):
    for i in range(m.nchains):
        lik, st = m.chain_lik(i, port)
        want = lik.lnL()
        assert abs(st["lnL"] - want) <= tol * abs(want), (i, st["lnL"], want)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_mc3_chains_match_oracle(gpu, port, precision):
    m = build(precision)
    check_chains(m, port, TOL[precision])       # generation 0
    m.run(157)                                  # graphs of 8 + remainder
    check_chains(m, port, TOL[precision])
    st = m.stats()
    assert st["generation"] == 158
    acc = st["accepts"].sum(axis=0)
    rej = st["rejects"].sum(axis=0)
    assert (acc + rej)[:7].min() > 0            # every move but +I drawn
    assert acc[7] + rej[7] == 0                 # no +I component here
    assert (acc + rej)[8:].max() == 0           # no jump moves asked for
    assert acc[0] > 0 and acc[1] > 0            # brlen and NNI accepted
    assert acc[5] > 0                           # SPR accepted
    assert acc[6] > 0                           # eTBR accepted
    assert st["swaps"].sum() > 0
    heats = sorted(m.chain_state(i)["heat"] for i in range(m.nchains))
    assert np.allclose(heats, sorted(1.0 / (1.0 + 0.2 * i) for i in range(4)))
    tr = m.trace(158)
    assert np.isfinite(tr).all()
    m.close()


def test_mc3_same_seed_fp32_follows_fp64(gpu):
    """Same seed: the FP32 chains draw the same moves as the FP64 chains, so
    the cold-chain traces agree until an acceptance decision falls within
    the FP32 error of its threshold."""
    a, b = build("fp64", seed=21), build("fp32", seed=21)
    a.run(40)
    b.run(40)
    ta, tb = a.trace(41), b.trace(41)
    rel = np.abs(ta - tb) / np.abs(ta)
    assert rel[0] <= 1e-6
    assert (rel[:20] <= 1e-6).all()
    a.close()
    b.close()


def test_mc3_brlen_only_single_category(gpu, port):
    case = synth.Case(10, 500, 0.1, 11, alpha=None)
    aln = case.alignment()
    t = case.tree(aln.taxaMap)
    m = Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=None,
            nchains=2, heat_delta=0.1, seed=4, moves={"brlen": 1.0},
            precision="fp64", graph_gens=4)
    m.run(50)
    for i in range(2):
        lik, st = m.chain_lik(i, port)
        want = lik.lnL()
        assert abs(st["lnL"] - want) <= 1e-11 * abs(want)
    m.close()


def test_mc3_samples_the_prior_without_data(gpu):
    """With all-gap columns the likelihood is 1, so the chain samples the
    prior: iid Exp(10) branch lengths, whatever the topology moves do.  A
    wrong Hastings ratio in the branch-length, NNI or SPR move biases the
    tree length away from (2N - 3) x 0.1."""
    from crux_gb300.alignment import Alignment, TaxaMap
    case = synth.Case(8, 50, 0.1, 17)
    aln0 = case.alignment()
    rows = np.full((aln0.ntaxa, 4), ord("-"), dtype=np.uint8)
    aln = Alignment(taxaMap=TaxaMap(aln0.taxaMap.taxa), rows=rows)
    t = case.tree(aln.taxaMap)
    m = Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=None,
            nchains=1, seed=123, precision="fp64", graph_gens=32,
            moves={"brlen": 1.0, "nni": 1.0, "spr": 1.0})
    tl = []
    m.run(2000)
    for _ in range(1500):
        m.run(64)
        st = m.chain_state(0)
        assert abs(st["lnL"]) < 1e-9
        tl.append(st["len"].sum())
    m.close()
    nedge = 2 * 8 - 3
    assert abs(np.mean(tl) - nedge * 0.1) < 0.08 * nedge * 0.1, np.mean(tl)
    # Exp(10) lengths: the tree length has variance nedge / 100.
    assert abs(np.var(tl) - nedge / 100.0) < 0.3 * nedge / 100.0, np.var(tl)


def _empty_alignment(ntaxa, seed):
    from crux_gb300.alignment import Alignment, TaxaMap
    case = synth.Case(ntaxa, 50, 0.1, seed)
    aln0 = case.alignment()
    rows = np.full((aln0.ntaxa, 4), ord("-"), dtype=np.uint8)
    aln = Alignment(taxaMap=TaxaMap(aln0.taxaMap.taxa), rows=rows)
    return case, aln


def _is_three_cherries(parent, ntaxa):
    """A 6-taxon unrooted binary tree is either a caterpillar or three
    cherries; it is three cherries when every internal edge splits off a
    pair of leaves."""
    nn = len(parent)
    below = [0] * nn
    for leaf in range(ntaxa):
        v = leaf
        while v >= 0:
            below[v] |= 1 << leaf
            v = parent[v]
    for v in range(ntaxa, nn):
        if parent[v] < 0:
            continue
        k = bin(below[v]).count("1")
        if min(k, ntaxa - k) != 2:
            return False
    return True


@pytest.mark.parametrize("moves", [{"etbr": 1.0}, {"etbr": 1.0, "brlen": 1.0}])
def test_mc3_etbr_samples_uniform_topologies(gpu, moves):
    """Without data the chains sample the prior: every 6-taxon topology is
    equally likely, so 15 of 105 (1/7) are three cherries, and the Exp(10)
    branch lengths sum to 0.9 on average.  A wrong eTBR Hastings ratio
    moves the shape frequency (the extension terms) or the tree length
    (the multipliers)."""
    case, aln = _empty_alignment(6, 29)
    t = case.tree(aln.taxaMap)
    m = Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=None,
            nchains=4, heat_delta=0.0, seed=77, precision="fp64",
            graph_gens=32, moves=moves)
    m.run(3000)
    cherries, tl, n = 0, [], 0
    for _ in range(1000):
        m.run(64)
        for i in range(4):
            st = m.chain_state(i)
            assert abs(st["lnL"]) < 1e-9
            cherries += _is_three_cherries(list(st["parent"]), 6)
            tl.append(st["len"].sum())
            n += 1
    acc = m.stats()["accepts"].sum(axis=0)
    m.close()
    assert acc[6] > 0
    frac = cherries / n
    # 4000 thinned samples: standard error about 0.0055.
    assert abs(frac - 1.0 / 7.0) < 0.025, frac
    assert abs(np.mean(tl) - 0.9) < 0.05, np.mean(tl)


def test_mc3_etbr_chains_match_oracle(gpu, port):
    """eTBR alone re-roots the tree buffer on every accepted move; the
    cached CLs of the nodes it leaves alone must still be right."""
    m = build("fp64", nchains=3, seed=31, moves={"etbr": 1.0, "brlen": 0.2},
              ntaxa=24)
    m.run(200)
    check_chains(m, port, TOL["fp64"])
    acc = m.stats()["accepts"].sum(axis=0)
    assert acc[6] > 0
    m.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_mc3_invar_chains_match_oracle(gpu, port, precision):
    """GTR+G4+I chains (five components) with +I weight, alpha, rate,
    NNI and eTBR moves: each chain's lnL is the oracle's for its tree,
    model and weights."""
    case = synth.Case(16, 1000, 0.1, 41, pinv=0.2)
    aln = case.alignment()
    t = case.tree(aln.taxaMap)
    m = Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=0.5,
            ncat=4, pinv=0.2, nchains=3, heat_delta=0.2, seed=8,
            moves={"brlen": 1.0, "invar": 2.0, "alpha": 0.5, "rates": 0.5,
                   "nni": 0.5, "etbr": 0.5},
            precision=precision, graph_gens=8)
    check_chains(m, port, TOL[precision])
    m.run(120)
    check_chains(m, port, TOL[precision])
    st = m.stats()
    acc = st["accepts"].sum(axis=0)
    assert acc[7] > 0                           # +I weight moves accepted
    w = [m.chain_state(i) for i in range(3)]
    assert any(s["winvar"] != 0.2 for s in w)
    m.close()


def test_mc3_invar_weights_sample_their_prior(gpu):
    """Without data the +I weight moves sample the reference's priors:
    wVar ~ Exp(1 - invarPrior) and wInvar ~ Exp(invarPrior), both of mean
    2 at invarPrior 0.5.  A wrong Hastings ratio or prior term moves the
    means."""
    case, aln = _empty_alignment(6, 31)
    t = case.tree(aln.taxaMap)
    m = Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=None,
            pinv=0.3, nchains=4, heat_delta=0.0, seed=5, precision="fp64",
            graph_gens=32, moves={"invar": 1.0})
    m.run(2000)
    wv, wi = [], []
    for _ in range(1000):
        m.run(32)
        for i in range(4):
            st = m.chain_state(i)
            assert abs(st["lnL"]) < 1e-9
            wv.append(st["wvar"])
            wi.append(st["winvar"])
    m.close()
    assert abs(np.mean(wv) - 2.0) < 0.25, np.mean(wv)
    assert abs(np.mean(wi) - 2.0) < 0.25, np.mean(wi)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_mc3_jump_chains_match_oracle(gpu, port, precision):
    """Gamma on/off and equal/estimated frequency jumps with the moves
    inside each state: each chain's lnL is the oracle's for its tree and
    model, Gamma switched off reading as alpha = INFINITY."""
    import math
    # Few sites and hot chains (heats down to 0.1), so that jumps are
    # accepted now and then.
    case = synth.Case(16, 100, 0.1, 43, pinv=0.15)
    aln = case.alignment()
    t = case.tree(aln.taxaMap)
    m = Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=0.5,
            ncat=4, pinv=0.15, nchains=4, heat_delta=3.0, seed=12,
            moves={"brlen": 1.0, "gammajump": 2.0, "freqjump": 2.0,
                   "alpha": 0.5, "freqs": 0.5, "invar": 0.5},
            precision=precision, graph_gens=8)
    m.run(160)
    check_chains(m, port, TOL[precision])
    st = m.stats()
    acc = st["accepts"].sum(axis=0)
    rej = st["rejects"].sum(axis=0)
    assert acc[8] + rej[8] > 0 and acc[9] + rej[9] > 0
    assert acc[8] + acc[9] > 0
    m.close()


def test_mc3_jumps_sample_their_prior(gpu):
    """On empty data the jumps sample the model prior: with prior odds 3 of
    Gamma off (and of equal frequencies), a quarter of the samples have
    Gamma on (estimated frequencies), and 1/alpha follows its Exp(1) prior
    while Gamma is on."""
    import math
    case, aln = _empty_alignment(6, 33)
    t = case.tree(aln.taxaMap)
    m = Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=0.7,
            ncat=4, nchains=4, heat_delta=0.0, seed=19, precision="fp64",
            graph_gens=32, gamma_jump_prior=3.0, freq_jump_prior=3.0,
            moves={"gammajump": 1.0, "freqjump": 1.0, "alpha": 1.0})
    m.run(2000)
    on, est, rsi, n = 0, 0, [], 0
    for _ in range(800):
        m.run(32)
        for i in range(4):
            st = m.chain_state(i)
            assert abs(st["lnL"]) < 1e-9
            n += 1
            if math.isfinite(st["alpha"]):
                on += 1
                rsi.append(1.0 / st["alpha"])
            f = st["freqs"]
            est += not (f[0] == f[1] == f[2] == f[3])
    m.close()
    assert abs(on / n - 0.25) < 0.04, on / n
    assert abs(est / n - 0.25) < 0.04, est / n
    assert abs(np.mean(rsi) - 1.0) < 0.15, np.mean(rsi)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_mc3_invar_jump_chains_match_oracle(gpu, port, precision):
    """The +I off/on jump (invarJumpPropose, Chain.pyx:1449-1546) beside
    the +I weight, alpha and branch moves: every chain's lnL is the
    oracle's for its tree, model and weights, +I off reading as wInvar = 0
    with wVar = 1; hot chains switch +I both ways."""
    case = synth.Case(16, 100, 0.1, 47, pinv=0.2)
    aln = case.alignment()
    t = case.tree(aln.taxaMap)
    m = Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=0.5,
            ncat=4, pinv=0.2, nchains=4, heat_delta=3.0, seed=14,
            moves={"brlen": 1.0, "invar": 1.0, "invarjump": 2.0, "alpha": 0.5},
            precision=precision, graph_gens=8)
    seen_off = seen_on_again = False
    for _ in range(10):
        m.run(24)
        check_chains(m, port, TOL[precision])
        for i in range(4):
            st = m.chain_state(i)
            if st["winvar"] == 0.0:
                assert st["wvar"] == 1.0
                seen_off = True
            elif seen_off:
                seen_on_again = True
    st = m.stats()
    assert st["accepts"].sum(axis=0)[10] > 0
    assert seen_off and seen_on_again
    m.close()


def test_mc3_invar_jump_samples_its_prior(gpu):
    """Without data the +I jump and weight moves sample the prior: +I on
    and off equally often (invarJumpPrior 1), and when on, wVar and wInvar
    of the weight move's priors, Exp of rates 1 - invarPrior and
    invarPrior (means 2 at invarPrior 0.5).  A wrong Hastings ratio or
    prior term moves the fraction or the means."""
    case, aln = _empty_alignment(6, 33)
    t = case.tree(aln.taxaMap)
    m = Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=None,
            pinv=0.3, nchains=4, heat_delta=0.0, seed=6, precision="fp64",
            graph_gens=32, moves={"invar": 1.0, "invarjump": 1.0})
    m.run(2000)
    on, wv, wi = [], [], []
    for _ in range(1200):
        m.run(32)
        for i in range(4):
            st = m.chain_state(i)
            assert abs(st["lnL"]) < 1e-9
            on.append(st["winvar"] != 0.0)
            if st["winvar"] != 0.0:
                wv.append(st["wvar"])
                wi.append(st["winvar"])
    m.close()
    assert abs(np.mean(on) - 0.5) < 0.06, np.mean(on)
    assert abs(np.mean(wv) - 2.0) < 0.3, np.mean(wv)
    assert abs(np.mean(wi) - 2.0) < 0.3, np.mean(wi)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_mc3_rate_jump_chains_match_oracle(gpu, port, precision):
    """Rate classes merged and split (rateJumpPropose, Chain.pyx:821-1075)
    beside the class-rate multiplier (ratePropose, :267-319) and the
    Dirichlet move over class rates: every chain's lnL is the oracle's for
    its tree and exchangeabilities, and hot chains visit fewer classes."""
    case = synth.Case(16, 100, 0.1, 48)
    aln = case.alignment()
    t = case.tree(aln.taxaMap)
    m = Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=0.5,
            ncat=4, nchains=4, heat_delta=3.0, seed=15,
            moves={"brlen": 1.0, "ratejump": 2.0, "rate": 1.0, "rates": 0.5},
            precision=precision, graph_gens=8)
    ks = set()
    for _ in range(10):
        m.run(24)
        check_chains(m, port, TOL[precision])
        for i in range(4):
            ks.add(max(m.chain_state(i)["rclass"]) + 1)
    st = m.stats()
    acc = st["accepts"].sum(axis=0)
    assert acc[11] > 0 and acc[12] > 0
    assert min(ks) < 6
    m.close()


def test_mc3_rate_jump_samples_its_prior(gpu):
    """Without data the rate moves sample the prior the reference's
    randomLik draws from (rateJumpPrior 1): every number of rate classes
    1..6 equally often, every partition with two classes seen, and class
    rates of mean 1 (Exp(1)).  A wrong Hastings ratio or prior term moves
    the class counts."""
    case, aln = _empty_alignment(6, 34)
    t = case.tree(aln.taxaMap)
    m = Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=None,
            nchains=8, heat_delta=0.0, seed=7, precision="fp64", graph_gens=32,
            moves={"ratejump": 1.0, "rate": 1.0, "rates": 1.0})
    m.run(2000)
    ks, parts, r0 = [], set(), []
    for _ in range(1500):
        m.run(32)
        for i in range(8):
            st = m.chain_state(i)
            assert abs(st["lnL"]) < 1e-9
            k = max(st["rclass"]) + 1
            ks.append(k)
            if k == 2:
                parts.add(tuple(st["rclass"]))
            r0.append(st["rates"][0])
    m.close()
    frac = np.bincount(ks, minlength=7)[1:] / len(ks)
    assert np.all(np.abs(frac - 1.0 / 6.0) < 0.05), frac
    assert len(parts) == 31
    assert abs(np.mean(r0) - 1.0) < 0.15, np.mean(r0)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_mc3_mixture_chains_match_oracle(gpu, port, precision):
    """Mixture members added and removed (mixtureJumpPropose,
    Chain.pyx:1633-1814), their weights and rate multipliers moved
    (weightPropose, rmultPropose, :72-141, 200-266) beside per-member
    model moves: every chain's lnL is the oracle's for a Lik holding the
    chain's members (nmodels, setWeight, setRmult and each member's
    parameters)."""
    case = synth.Case(14, 150, 0.1, 61)
    aln = case.alignment()
    t = case.tree(aln.taxaMap)
    m = Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=0.5,
            ncat=4, nchains=4, heat_delta=0.5, seed=21,
            moves={"brlen": 1.0, "mixturejump": 2.0, "weight": 1.0,
                   "rmult": 1.0, "alpha": 0.5, "rates": 0.5, "freqs": 0.5,
                   "freqjump": 0.5, "gammajump": 0.5},
            max_models=2, mixture_jump_prior=0.2, precision=precision,
            graph_gens=8)
    seen = set()
    for _ in range(12):
        m.run(24)
        check_chains(m, port, TOL[precision])
        for i in range(4):
            seen.add(len(m.chain_models(i)))
    st = m.stats()
    acc = st["accepts"].sum(axis=0)
    assert acc[15] > 0, acc
    assert acc[13] > 0 and acc[14] > 0, acc
    assert seen == {1, 2}, seen
    m.close()


def test_mc3_mixture_jump_samples_its_prior(gpu):
    """Without data the mixture moves sample their prior: k members with
    probability proportional to (1 - mixtureJumpPrior)^(k-1) for k <= 4,
    member weights and rate multipliers of mean 1 (Exp(1)), estimated base
    frequencies in half the members (freqJumpPrior 1) and class rates of
    mean 1.  A wrong Hastings ratio or member density moves the counts."""
    case, aln = _empty_alignment(6, 35)
    t = case.tree(aln.taxaMap)
    mjp = 1.0 / 3.0
    m = Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=None,
            nchains=8, heat_delta=0.0, seed=8, precision="fp64", graph_gens=32,
            moves={"mixturejump": 2.0, "weight": 1.0, "rmult": 1.0,
                   "rates": 0.5, "freqs": 0.5, "freqjump": 1.0},
            max_models=4, mixture_jump_prior=mjp)
    m.run(2000)
    ks, w, rm, est, r0 = [], [], [], [], []
    for _ in range(1200):
        m.run(32)
        for i in range(8):
            ms = m.chain_models(i)
            ks.append(len(ms))
            for q in ms:
                w.append(q["weight"])
                rm.append(q["rmult"])
                est.append(q["freqs_est"])
                r0.append(q["rates"][0])
        assert abs(m.chain_state(0)["lnL"]) < 1e-9
    m.close()
    want = np.array([(1.0 - mjp) ** (k - 1) for k in range(1, 5)])
    want /= want.sum()
    frac = np.bincount(ks, minlength=5)[1:] / len(ks)
    assert np.all(np.abs(frac - want) < 0.04), (frac, want)
    assert abs(np.mean(w) - 1.0) < 0.12, np.mean(w)
    assert abs(np.mean(rm) - 1.0) < 0.12, np.mean(rm)
    assert abs(np.mean(est) - 0.5) < 0.06, np.mean(est)
    assert abs(np.mean(r0) - 1.0) < 0.15, np.mean(r0)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_mc3_checkpoint_resume_continues_bit_exact(gpu, precision):
    """A run checkpointed after 96 generations (trees, heats, mixture members,
    move and swap counts; plain data, through JSON) and resumed in a new
    run of the same configuration recomputes every chain's lnL bit for bit
    and then follows the uninterrupted run exactly: the same cold-chain
    trace, chain states and counts after 64 more generations."""
    import json
    moves = {"brlen": 1.0, "nni": 0.5, "spr": 0.5, "etbr": 0.5, "rates": 0.5,
             "alpha": 0.5, "freqs": 0.5, "gammajump": 0.3, "ratejump": 0.3,
             "mixturejump": 0.5, "weight": 0.3, "rmult": 0.3,
             "polytomyjump": 0.5}

    def make():
        case = synth.Case(12, 300, 0.1, 71)
        aln = case.alignment()
        t = case.tree(aln.taxaMap)
        return Mc3(t, aln, case.params["rates"], case.params["freqs"],
                   alpha=0.5, ncat=4, nchains=3, heat_delta=0.3, seed=33,
                   moves=moves, max_models=2, precision=precision,
                   graph_gens=8)

    a = make()
    a.run(96)
    ck = json.loads(json.dumps(a.checkpoint()))
    a.run(64)
    b = make()
    b.restore(ck)
    for i in range(3):
        assert b.chain_state(i)["lnL"] == ck["chains"][i]["lnL"], i
    b.run(64)
    # Generation g writes trace[g]; the checkpoint was taken before g = 97.
    assert np.array_equal(a.trace(161)[97:], b.trace(161)[97:])
    for i in range(3):
        sa, sb = a.chain_state(i), b.chain_state(i)
        assert sa["lnL"] == sb["lnL"] and sa["heat"] == sb["heat"]
        assert np.array_equal(sa["parent"], sb["parent"])
        assert np.array_equal(sa["len"], sb["len"])
        assert sa["models"] == sb["models"]
    ta, tb = a.stats(), b.stats()
    assert np.array_equal(ta["accepts"], tb["accepts"])
    assert np.array_equal(ta["rejects"], tb["rejects"])
    assert np.array_equal(ta["swaps"], tb["swaps"])
    assert ta["generation"] == tb["generation"] == 161
    a.close()
    b.close()


def _splits(parent, collapsed, ntaxa):
    """The multifurcating tree a chain stands for: the leaf sets below its
    internal edges that are not contracted, each as the side without leaf
    0."""
    nn = len(parent)
    below = [0] * nn
    for leaf in range(ntaxa):
        v = leaf
        while v >= 0:
            below[v] |= 1 << leaf
            v = parent[v]
    full = (1 << ntaxa) - 1
    out = set()
    for v in range(ntaxa, nn):
        if parent[v] < 0 or collapsed[v]:
            continue
        s = below[v]
        out.add(s if not (s & 1) else full ^ s)
    return frozenset(out)


def test_mc3_polytomy_jumps_sample_their_prior(gpu):
    """Without data, polytomy jumps with NNI, SPR, eTBR and branch moves
    sample the reference's prior over multifurcating trees (polytomyJumpPrior
    1: every one of the 26 five-taxon trees equally often: 15 resolved, 10
    with one polytomy, the star) with Exp(10) lengths on the edges that are
    not contracted.  A missing resolution-count term in the topology moves,
    or a wrong Hastings ratio in the jump, moves these frequencies."""
    case, aln = _empty_alignment(5, 36)
    t = case.tree(aln.taxaMap)
    m = Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=None,
            nchains=8, heat_delta=0.0, seed=10, precision="fp64", graph_gens=32,
            moves={"polytomyjump": 2.0, "nni": 1.0, "spr": 0.5, "etbr": 0.5,
                   "brlen": 1.0})
    m.run(2000)
    seen, lens = {}, []
    for _ in range(1500):
        m.run(16)
        for i in range(8):
            st = m.chain_state(i)
            assert abs(st["lnL"]) < 1e-9
            sp = _splits(st["parent"], st["collapsed"], 5)
            seen[sp] = seen.get(sp, 0) + 1
            for v in range(5, len(st["parent"])):
                if st["parent"][v] >= 0:
                    if st["collapsed"][v]:
                        assert st["len"][v] == 0.0
                    else:
                        lens.append(st["len"][v])
    m.close()
    total = sum(seen.values())
    assert len(seen) == 26, len(seen)
    by_edges = {0: 0, 1: 0, 2: 0}
    for sp, n in seen.items():
        by_edges[len(sp)] += n
        assert abs(n / total - 1.0 / 26.0) < 0.012, (sorted(sp), n / total)
    assert abs(by_edges[2] / total - 15.0 / 26.0) < 0.03, by_edges
    assert abs(np.mean(lens) - 0.1) < 0.01, np.mean(lens)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_mc3_polytomy_chains_match_oracle(gpu, port, precision):
    """Chains whose trees gain and lose polytomies (contracted edges of
    length 0): every chain's lnL is the oracle's for its tree."""
    case = synth.Case(14, 200, 0.1, 62)
    aln = case.alignment()
    t = case.tree(aln.taxaMap)
    m = Mc3(t, aln, case.params["rates"], case.params["freqs"], alpha=0.5,
            ncat=4, nchains=4, heat_delta=0.5, seed=23,
            moves={"brlen": 1.0, "polytomyjump": 2.0, "nni": 0.5, "etbr": 0.5,
                   "spr": 0.5}, precision=precision, graph_gens=8)
    ncoll = set()
    for _ in range(10):
        m.run(24)
        check_chains(m, port, TOL[precision])
        for i in range(4):
            ncoll.add(int(m.chain_state(i)["collapsed"].sum()))
    acc = m.stats()["accepts"].sum(axis=0)
    assert acc[16] > 0, acc
    assert max(ncoll) > 0, ncoll
    m.close()
