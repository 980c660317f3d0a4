"""The reference's likelihood known-answer tests (test/Lik_*.cx.exp) through
the host restatement (planner, model prep, Gamma discretisation) driving the
CPU oracles: the reference's own CxLik.c build and this repository's port."""
import math

import kat_cases as K


def test_lik_b(oracle_lib):
    for (lnl, sites), (elnl, esites) in zip(K.run_lik_b(oracle_lib), K.LIK_B):
        assert K.close(lnl, elnl, 5)
        assert all(K.close(a, b, 6) for a, b in zip(sites, esites))


def test_lik_e_gamma(oracle_lib):
    for got, exp in zip(K.run_lik_e(oracle_lib), K.LIK_E):
        for g, e in zip(got, exp):
            assert all(K.close(a, b, 5) for a, b in zip(g, e))


def test_lik_h_missing(oracle_lib):
    for row in K.run_lik_h(oracle_lib):
        assert all(K.close(a, b, 5) for a, b in zip(row, K.LIK_H))


def test_lik_c_every_root(oracle_lib):
    res = K.run_every_root(oracle_lib, K.THREE, "(one:0.0,two:0.0,three:1.25);")
    assert len(res) == 4
    for lnl, sites in res:
        assert K.close(lnl, K.LIK_C[0], 4)
        assert all(K.close(a, b, 6) for a, b in zip(sites, K.LIK_C[1]))


def test_lik_j_freqs_every_root(oracle_lib):
    for blen, elnl, esites in K.LIK_J:
        res = K.run_every_root(oracle_lib, K.THREE,
                               "(one:0.0,two:0.0,three:%r);" % blen,
                               freqs=(0.4, 0.3, 0.2, 0.1))
        for lnl, sites in res:
            assert K.close(lnl, elnl, 5)
            assert all(K.close(a, b, 6) for a, b in zip(sites, esites))


def test_lik_g_zero_lengths(oracle_lib):
    for v in K.run_lik_g(oracle_lib):
        assert v <= -50.0


def test_lik_l_invariant(oracle_lib):
    direct, emulated = K.run_lik_l(oracle_lib)
    for (lnl, sites), (_, elnl, esites) in zip(direct, K.LIK_L):
        assert K.close(lnl, elnl, 5)
        assert all(K.close(a, b, 6) for a, b in zip(sites, esites))
    for (lnl, sites), (_, elnl, esites) in zip(emulated, K.LIK_L):
        assert K.close(lnl, elnl, 5)
        assert all(K.close(a, b, 6) for a, b in zip(sites, esites))


def test_lik_m_first_value(oracle_lib):
    render, lnl = K.run_lik_m(oracle_lib)
    assert render == K.LIK_M_RENDER
    assert abs(lnl - K.LIK_M) <= 5e-10


def test_lik_d_normalisation_and_mixtures(oracle_lib):
    for vals, (_, _, _, printed) in zip(K.run_lik_d(oracle_lib), K.LIK_D_TREES):
        for v in vals:
            assert abs(v - vals[0]) <= 1e-9 * abs(vals[0])
        assert abs(vals[0] - printed) < 2e-3


def test_lik_k_gamma2_equals_mixture(oracle_lib):
    for (cat, mod), (_, _, elnl, esites) in zip(K.run_lik_k(oracle_lib), K.LIK_K):
        assert K.close(cat[0], elnl, 3) or abs(cat[0] - elnl) < 2e-3
        assert abs(cat[0] - mod[0]) < 1e-3
        for a, b in zip(cat[1], mod[1]):
            assert abs(a - b) < 1e-3


def test_ref_port_agree(ref, port):
    """Port and reference agree far below the printed precision."""
    a = K.run_lik_e(ref)
    b = K.run_lik_e(port)
    for x, y in zip(a, b):
        for u, v in zip(x, y):
            for p, q in zip(u, v):
                assert math.isclose(p, q, rel_tol=1e-12)


def test_tune_candidates_follow_walker_shapes():
    """The autotuner offers only shapes the library has a walker for."""
    from crux_gb300 import tune
    c4 = tune.candidates("fp32", 4)
    assert (64, 4, 1, 24 << 10, 1) in c4 and (128, 2, 1, 0, 1) in c4
    assert all(t * g * n <= 256 for t, g, _, _, n in c4)
    assert (128, 4, 1, 0, 1) not in c4
    # Two patterns per thread: FP32, one thread per pattern, <= 5
    # components, and a tile that keeps at least one warp.
    assert (128, 1, 2, 0, 1) in c4 and (64, 1, 2, 0, 1) in c4
    assert (32, 1, 2, 0, 1) not in c4 and (64, 2, 2, 0, 1) not in c4
    # Two op lanes: FP32, one thread and one pattern per thread, <= 5
    # components, tile <= 64.
    assert (64, 1, 1, 0, 2) in c4 and (32, 1, 1, 24 << 10, 2) in c4
    assert (128, 1, 1, 0, 2) not in c4 and (64, 2, 1, 0, 2) not in c4
    assert (64, 1, 2, 0, 2) not in c4
    assert all(n == 1 for *_, n in tune.candidates("fp32", 4, lanes=(1,)))
    assert {n for *_, n in tune.candidates("fp32", 5)} == {1, 2}
    assert all(n == 1 for *_, n in tune.candidates("fp32", 6))
    assert all(n == 1 for *_, n in tune.candidates("fp64", 4))
    assert all(g == 1 for _, g, _, _, _ in tune.candidates("fp32", 5))
    assert {p for _, _, p, _, _ in tune.candidates("fp32", 5)} == {1, 2}
    assert all(g == 1 for _, g, _, _, _ in tune.candidates("fp64", 4))
    assert all(p == 1 for _, _, p, _, _ in tune.candidates("fp64", 4))
    assert all(p == 1 for _, _, p, _, _ in tune.candidates("fp32", 6))
    assert {g for _, g, _, _, _ in tune.candidates("fp32", 6)} == {1, 2}
    assert {g for _, g, _, _, _ in tune.candidates("fp32", 8)} == {1, 2, 4}
