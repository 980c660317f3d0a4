"""ORACLE TEST INFRASTRUCTURE -- not part of the product.

CPU checkers for the GB300 pruning likelihood.  Only tests/,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline legs may import
this package; the product (``crux_gb300``) never does.
"""
