"""bench.py's multi-process timing plumbing on CPU (gloo, world size 2).

Slices are independent, so ranks share no data; the only collectives are
the barrier around the timed region and the max over ranks of the elapsed
time. Each rank builds different slices (its own seeds).
"""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    try:
        d.barrier()
        worst = d.max(1.5 + rank)
        seeds = bench.slice_seeds(rank, 4)
        d.barrier()
        q.put((rank, d.rank, d.world, worst, seeds))
    finally:
        d.close()


def test_two_ranks_barrier_max_and_disjoint_slices():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[1] for o in out] == [0, 1] and all(o[2] == 2 for o in out)
    assert all(o[3] == 2.5 for o in out)            # max over ranks, seen by every rank
    s0, s1 = set(out[0][4]), set(out[1][4])
    assert len(s0) == 4 and len(s1) == 4 and not (s0 & s1)


def test_single_process_dist_is_a_no_op(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    assert d.world == 1 and d.max(3.25) == 3.25
    d.barrier()
    d.close()
