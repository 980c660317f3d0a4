"""Generate tests/golden/*.json with the reference's own CxLik.c core.

Run where the reference tree is available (it builds oracle/_ref first):
    python tests/golden/make_golden.py
Each fixture stores its inputs -- rooted Newick, the compressed alignment
(rows of pattern characters and their frequencies), the GTR/Gamma/+I
parameters and the host-core count that fixed the stripe padding -- and the
reference's outputs: lnL, site lnLs, and the lnL after each of a sequence of
single-branch rescales (dirty-path recomputes), each beside the lnL of the
same tree evaluated from scratch by a second reference Lik (every CL
recomputed), so that a dirty-path result is pinned independently of the
planner's cache-validity rule.  The planner here is the Python restatement
of Lik._plan alone.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from crux_gb300 import synth  # noqa: E402
from crux_gb300.lik import Config  # noqa: E402
from oracle import oracle  # noqa: E402

CASES = {
    # name: (ntaxa, nsites, mean brlen, seed, pinv, gap fraction)
    "yule16_gtr_g4": (16, 1000, 0.1, 101, 0.0, 0.0),
    "yule64_gtr_g4_inv_gaps": (64, 3000, 0.05, 102, 0.2, 0.005),
    "yule40_long_branches": (40, 1500, 0.6, 103, 0.0, 0.01),
}
NCPUS = 8


def main():
    oracle.build(os.environ.get("CRUX_REF", "/root/reference/crux"))
    ref = oracle.load_ref()
    assert ref is not None, "reference core not built"
    Config.ncpus = NCPUS
    for name, (nt, ns, bl, seed, pinv, gap) in CASES.items():
        case = synth.Case(nt, ns, bl, seed, pinv=pinv, gap_frac=gap)
        aln = case.alignment()
        rows = [aln.getSeq(i) for i in range(aln.ntaxa)]
        freqs = [int(x) for x in aln.freqs]
        lik = case.lik(lib=ref, alignment=aln)
        scratch = case.lik(lib=ref, alignment=aln)
        assert not lik.native_plan and not scratch.native_plan
        lnl = lik.lnL()
        sites = lik.siteLnLs()
        rng = np.random.default_rng(seed)
        edges = lik.tree.edges
        dirty = []
        for _ in range(10):
            i = int(rng.integers(len(edges)))
            f = float(rng.uniform(0.5, 2.0))
            edges[i].length *= f
            se = scratch.tree.edges
            se[i].length *= f
            assert se[i].length == edges[i].length
            scratch.lik.invalidate = True
            full = scratch.lnL()
            got = lik.lnL()
            assert abs(got - full) <= 1e-12 * abs(full), (got, full)
            dirty.append([i, f, got, full])
        fx = {"name": name, "newick": case.newick, "taxa": aln.taxaMap.taxa,
              "rows": rows, "freqs": freqs, "params": case.params,
              "alpha": case.alpha, "ncat": case.ncat, "pinv": pinv,
              "ncpus": NCPUS, "lnL": lnl, "siteLnL": sites, "dirty": dirty,
              "generator": "reference lib/Crux/Tree/CxLik.c via oracle/_ref"}
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(fx, f)
        print(name, "patterns", len(freqs), "lnL", lnl)


if __name__ == "__main__":
    main()
