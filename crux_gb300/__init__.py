"""crux_gb300: GB300-native Felsenstein pruning likelihood.

A from-scratch sm_103a implementation of the likelihood core of Crux
(``Crux.Tree.Lik`` and the C entry points it wraps).  Host-side model and
planning code lives in this package; every likelihood is computed by
crux_gb300/_lib/libcxlik_gpu.so on the GPU.
"""
from .alignment import Alignment, CTMatrix, Dna, Protein, TaxaMap  # noqa: F401
from .lik import Config, Lik  # noqa: F401
from .tree import Edge, Node, Ring, Tree  # noqa: F401

__all__ = ["Alignment", "CTMatrix", "Config", "Dna", "Edge", "Lik", "Node",
           "Protein", "Ring", "TaxaMap", "Tree"]
