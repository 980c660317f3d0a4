"""Replica ranks on CPU (gloo, world size 2): the bench's barrier and
max-over-ranks reduction give every rank the slowest rank's time, and the
reference arm's non-zero ranks leave without work or output.

The path does not shard across GPUs beyond independent replicas (patterns
are independent until one scalar sum, and every box has one GPU), so the
only cross-rank steps are the barrier around the timed region and the max
of the per-rank times; these run here as two CPU processes."""
import json
import os
import socket
import subprocess
import sys
import textwrap

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = textwrap.dedent("""
    import json, sys
    sys.path.insert(0, %r)
    import bench
    d = bench.Dist()
    d.barrier()
    mine = 1.0 + 2.5 * d.rank        # rank 1 is the slower replica
    got = d.max(mine)
    d.barrier()
    print(json.dumps({"rank": d.rank, "ws": d.ws, "mine": mine, "max": got}))
    d.close()
""") % REPO


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_barrier_and_max_over_two_ranks():
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                                      text=True))
    outs = []
    try:
        for p in procs:
            out, err = p.communicate(timeout=120)
            assert p.returncode == 0, err
            outs.append(json.loads(out.strip().splitlines()[-1]))
    finally:
        for p in procs:  # a rank that failed must not leave its peer waiting
            if p.poll() is None:
                p.kill()
                p.wait()
    assert sorted(o["rank"] for o in outs) == [0, 1]
    for o in outs:
        assert o["ws"] == 2
        assert o["max"] == 3.5


def test_single_rank_needs_no_process_group(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.delenv("RANK", raising=False)
    sys.path.insert(0, REPO)
    import bench
    d = bench.Dist()
    assert (d.ws, d.rank) == (1, 0)
    d.barrier()
    assert d.max(2.25) == 2.25
    d.close()


def test_reference_arm_other_ranks_do_no_work(capsys):
    """Under torchrun only rank 0 times the reference's CPU path and prints
    its line; another rank closes its process group and returns."""
    sys.path.insert(0, REPO)
    import bench

    class Rank1:
        rank, ws = 1, 2
        closed = False

        def close(self):
            self.closed = True

    d = Rank1()
    bench.run_reference(None, d)
    assert d.closed
    assert capsys.readouterr().out == ""
