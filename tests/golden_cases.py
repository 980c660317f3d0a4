"""Load tests/golden/*.json fixtures into Lik objects."""
import glob
import json
import os

import numpy as np

from crux_gb300 import synth
from crux_gb300.alignment import Alignment, TaxaMap
from crux_gb300.lik import Config
from crux_gb300.tree import Tree

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fixtures():
    """Likelihood fixtures (the compaction known answers are not one)."""
    return sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.json"))
                  if not os.path.basename(p).startswith("compaction"))


def load(path):
    return json.load(open(path))


def build_lik(fx, lib, precision="fp64"):
    """The fixture's Lik with the stripe padding it was generated with."""
    old = Config.ncpus
    Config.ncpus = fx["ncpus"]
    try:
        rows = np.frombuffer("".join(fx["rows"]).encode("ascii"),
                             dtype=np.uint8).reshape(len(fx["rows"]), -1)
        aln = Alignment(taxaMap=TaxaMap(fx["taxa"]), rows=rows)
        aln.freqs = np.asarray(fx["freqs"], dtype=np.uint32)
        t = Tree(fx["newick"])
        t.deroot()
        t.canonize(aln.taxaMap)
        from crux_gb300.lik import Lik
        lik = Lik(t, aln, ncat=fx["ncat"], invar=fx["pinv"] > 0.0, lib=lib,
                  precision=precision)
        synth.apply_params(lik, 0, fx["params"], fx["alpha"], fx["pinv"])
        return lik
    finally:
        Config.ncpus = old
