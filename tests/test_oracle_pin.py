"""Pin the CPU oracle port against outputs of the reference's own C core
(tests/golden/*.json, written by tests/golden/make_golden.py)."""
import math

import numpy as np
import pytest

import golden_cases as G


@pytest.mark.parametrize("path", G.fixtures())
def test_port_matches_reference_fixture(port, path):
    fx = G.load(path)
    lik = G.build_lik(fx, port)
    assert math.isclose(lik.lnL(), fx["lnL"], rel_tol=1e-12)
    sites = np.array(lik.siteLnLs())
    assert np.allclose(sites, fx["siteLnL"], rtol=1e-12, atol=1e-12)
    edges = lik.tree.edges
    for i, f, want, scratch in fx["dirty"]:
        edges[i].length *= f
        got = lik.lnL()
        assert math.isclose(got, want, rel_tol=1e-12)
        # The same tree from scratch (every CL recomputed).
        assert math.isclose(got, scratch, rel_tol=1e-12)


def test_fixtures_present():
    assert len(G.fixtures()) >= 3
