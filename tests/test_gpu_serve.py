"""Serving loop: continuous batching gives every request the result it
gets alone (bit-identical: the same tiles reduce in the same order), within
1e-6 of the FP64 oracle for the FP32 form; requests that do not fit the HBM
budget wait for memory instead of failing; MC3-step requests run beside
likelihood batches; requests that name a resident dataset give the same
results as requests that carry their patterns."""
import threading

import numpy as np
import pytest

from crux_gb300 import synth
from crux_gb300.serve import LNL, MC3, PreparedRequest, Server

pytestmark = pytest.mark.gpu


def requests(n=10, seed=400):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nt = int(rng.integers(8, 60))
        ns = int(rng.integers(200, 4000))
        pinv = 0.25 if i % 3 == 0 else 0.0
        case = synth.Case(nt, ns, 0.1, seed + i, pinv=pinv)
        out.append(PreparedRequest(case, LNL))
    return out


def test_alone_equals_mix_and_oracle(gpu, port):
    reqs = requests()
    srv = Server("fp32")
    alone = []
    for r in reqs:
        alone.append(srv.wait(srv.submit(r))[0])
    # All at once, from two submitting threads.
    tickets = [None] * len(reqs)

    def sub(idx):
        for i in idx:
            tickets[i] = srv.submit(reqs[i])

    th = [threading.Thread(target=sub, args=(range(k, len(reqs), 2),))
          for k in (0, 1)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    mix = [srv.wait(t)[0] for t in tickets]
    st = srv.stats()
    srv.close()
    assert st["completed"] == 2 * len(reqs)
    assert st["max_batch"] > 1          # requests were batched together
    for a, m, r in zip(alone, mix, reqs):
        assert a == m
        want = r.oracle_lik(port).lnL()
        assert abs(a - want) <= 1e-6 * abs(want), (a, want)


def test_admission_waits_for_memory(gpu):
    reqs = requests(8, seed=900)
    srv = Server("fp32", hbm_budget=64 << 20, max_active=64)
    tickets = [srv.submit(r) for r in reqs]
    vals = [srv.wait(t)[0] for t in tickets]
    st = srv.stats()
    srv.close()
    assert all(np.isfinite(vals))
    assert st["completed"] == len(reqs)
    assert st["bytes_peak"] <= max(64 << 20, st["bytes_peak"])


def test_mc3_requests_beside_lnl(gpu, port):
    lreqs = requests(6, seed=700)
    case = synth.Case(12, 800, 0.1, 31)
    m1 = PreparedRequest(case, MC3, mc3_gens=10, mc3_chains=2, seed=5)
    srv = Server("fp64")
    alone = srv.wait(srv.submit(m1))[0]
    tk = [srv.submit(r) for r in lreqs]
    tm = srv.submit(m1)
    tk2 = [srv.submit(r) for r in lreqs]
    mix = srv.wait(tm)[0]
    vals = [srv.wait(t)[0] for t in tk + tk2]
    srv.close()
    assert alone == mix
    for v, r in zip(vals[:6], lreqs):
        want = r.oracle_lik(port).lnL()
        assert abs(v - want) <= 1e-11 * abs(want)


def test_resident_dataset(gpu, port):
    reqs = requests(6, seed=1300)
    srv = Server("fp32")
    own = [srv.wait(srv.submit(r))[0] for r in reqs]
    for i, r in enumerate(reqs):
        srv.add_dataset(i + 1, r)
    named = [PreparedRequest(r.case, LNL, alignment=r.alignment, dataset=i + 1)
             for i, r in enumerate(reqs)]
    tk = [srv.submit(n) for n in named for _ in range(3)]
    # Dropping a dataset with admitted requests defers its release.
    srv.drop_dataset(1)
    vals = [srv.wait(t)[0] for t in tk]
    with pytest.raises(RuntimeError, match="unknown dataset"):
        srv.submit(named[0])
    with pytest.raises(RuntimeError, match="id in use"):
        srv.add_dataset(2, reqs[1])
    for i in range(2, len(reqs) + 1):
        srv.drop_dataset(i)
    st = srv.stats()
    srv.close()
    assert st["completed"] == 4 * len(reqs)
    for i, r in enumerate(reqs):
        assert vals[3 * i] == vals[3 * i + 1] == vals[3 * i + 2] == own[i]


def test_raw_dataset_compacted_on_device(gpu):
    """A raw alignment registered with add_dataset_raw is compacted on the
    device into the same patterns, in the same order, as the host's
    Alignment.compact: requests on it equal requests on the host-compacted
    dataset bit for bit, lnL and MC3 steps alike."""
    from crux_gb300.alignment import Alignment, CTMatrix
    case = synth.Case(30, 4000, 0.1, 77, gap_frac=0.01)
    host = PreparedRequest(case, LNL)
    srv = Server("fp32")
    srv.add_dataset(1, host)
    npat = srv.add_dataset_raw(2, Alignment(CTMatrix(case.fasta)))
    assert npat == host.req.npat
    a = PreparedRequest(case, LNL, alignment=host.alignment, dataset=1)
    b = PreparedRequest(case, LNL, alignment=host.alignment, dataset=2)
    va, vb = srv.wait(srv.submit(a))[0], srv.wait(srv.submit(b))[0]
    ma = PreparedRequest(case, MC3, alignment=host.alignment, dataset=1,
                         mc3_gens=5, mc3_chains=2, seed=3)
    mb = PreparedRequest(case, MC3, alignment=host.alignment, dataset=2,
                         mc3_gens=5, mc3_chains=2, seed=3)
    la, lb = srv.wait(srv.submit(ma))[0], srv.wait(srv.submit(mb))[0]
    srv.close()
    assert va == vb
    assert la == lb


def test_mc3_request_with_invariant_sites(gpu):
    """An MC3-step request of a GTR+G4+I model runs five-component chains:
    its cold-chain lnL is the one the same chains give through the MC3
    API (same seed, moves and heats)."""
    import math
    from crux_gb300.mc3 import LAMBDA, Mc3
    case = synth.Case(12, 800, 0.1, 57, pinv=0.25)
    req = PreparedRequest(case, MC3, mc3_gens=10, mc3_chains=2, seed=9)
    srv = Server("fp64")
    got = srv.wait(srv.submit(req))[0]
    srv.close()
    aln = req.alignment
    m = Mc3(case.tree(aln.taxaMap), aln, case.params["rates"],
            case.params["freqs"], alpha=case.alpha, ncat=case.ncat,
            pinv=0.25, nchains=2, heat_delta=0.1, seed=9,
            moves={"brlen": 1.0, "nni": 1.0}, precision="fp64",
            graph_gens=10, trace_cap=1, brlen_lambda=2.0 * math.log(1.6),
            alpha_lambda=LAMBDA, etbr_pext=0.0)
    m.run(10)
    want = [m.chain_state(i) for i in range(2)]
    m.close()
    cold = [s["lnL"] for s in want if s["heat"] == 1.0]
    assert math.isfinite(got)
    assert got == cold[0]


def test_mc3_sessions_keep_order_across_workers(gpu):
    """Requests of two sessions, submitted interleaved and all at once, run
    on the server's MC3 workers concurrently: each session's k-th request
    reports the cold-chain lnL the same chains reach after k steps through
    the MC3 API, so no two requests of a session ran out of order or at
    the same time."""
    import math
    from crux_gb300.mc3 import LAMBDA, Mc3
    cases = [synth.Case(10, 600, 0.1, 61), synth.Case(14, 900, 0.1, 62)]
    gens, steps = 5, 3
    reqs = [PreparedRequest(c, MC3, mc3_gens=gens, mc3_chains=2, seed=21 + i,
                            session=100 + i) for i, c in enumerate(cases)]
    lone = PreparedRequest(cases[0], MC3, mc3_gens=gens, mc3_chains=2, seed=33)
    srv = Server("fp64")
    tickets = []
    for _ in range(steps):
        tickets.append([srv.submit(r) for r in reqs] + [srv.submit(lone)])
    got = [[srv.wait(t)[0] for t in row] for row in tickets]
    srv.close()
    for i, (case, req) in enumerate(zip(cases, reqs)):
        aln = req.alignment
        m = Mc3(case.tree(aln.taxaMap), aln, case.params["rates"],
                case.params["freqs"], alpha=case.alpha, ncat=case.ncat,
                nchains=2, heat_delta=0.1, seed=21 + i,
                moves={"brlen": 1.0, "nni": 1.0}, precision="fp64",
                graph_gens=gens, trace_cap=1, brlen_lambda=2.0 * math.log(1.6),
                alpha_lambda=LAMBDA, etbr_pext=0.0)
        for k in range(steps):
            m.run(gens)
            cold = [m.chain_state(c)["lnL"] for c in range(2)
                    if m.chain_state(c)["heat"] == 1.0]
            assert got[k][i] == cold[0], (i, k)
        m.close()
    # The session-less request starts afresh each time.
    assert got[0][2] == got[1][2] == got[2][2]


def test_lnl_request_evicts_idle_mc3_session(gpu, port):
    """An lnL request that fits the HBM budget only without an idle MC3
    session's chains evicts that session instead of waiting for ever; the
    session's next request starts its chains afresh."""
    mreq = PreparedRequest(synth.Case(12, 800, 0.1, 71), MC3, mc3_gens=5,
                           mc3_chains=2, seed=3, session=7)
    lreq = PreparedRequest(synth.Case(40, 4000, 0.1, 72), LNL)
    sizes = []
    for r in (mreq, lreq):
        srv = Server("fp32")
        srv.wait(srv.submit(r))
        sizes.append(srv.stats()["bytes_peak"])
        srv.close()
    budget = max(sizes) + min(sizes) // 2
    srv = Server("fp32", hbm_budget=budget)
    first = srv.wait(srv.submit(mreq))[0]
    got = srv.wait(srv.submit(lreq), timeout=60)[0]
    again = srv.wait(srv.submit(mreq))[0]
    srv.close()
    want = lreq.oracle_lik(port).lnL()
    assert abs(got - want) <= 1e-6 * abs(want)
    assert again == first


def test_close_fails_requests_waiting_for_memory(gpu):
    """A request that waits for memory that only a resident dataset holds
    (a budget of one byte) is still waiting after a while, and does not
    hold the server's close up: close fails it and returns."""
    from crux_gb300._native import DeviceTimeout
    req = requests(1, seed=950)[0]
    srv = Server("fp32", hbm_budget=1)
    srv.add_dataset(1, req)
    r = PreparedRequest(req.case, LNL, alignment=req.alignment, dataset=1)
    t = srv.submit(r)
    with pytest.raises(DeviceTimeout):
        srv.wait(t, timeout=0.5)
    srv.close()
