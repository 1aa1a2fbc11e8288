"""The N > 1 path of bench.py on CPU: two gloo ranks (no GPU).

bench.py runs one independent solve per GPU ("replicas"); the only
cross-rank steps are the barrier around the timed region and the max of the
per-rank times.  These run here as two spawned processes over gloo.
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


def _rank_main(rank, ws, port, q):
    os.environ.update(WORLD_SIZE=str(ws), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    try:
        got_ws, got_rank, local, pg = bench.dist_init()
        bench.barrier(pg)
        # each rank reports its own time; the line carries the slowest rank
        t = bench.max_over_ranks(pg, 10.0 + 5.0 * rank)
        bench.barrier(pg)
        q.put((rank, got_ws, got_rank, local, t))
        pg.destroy_process_group()
    except Exception as e:  # reported to the parent, which fails the test
        q.put((rank, "error", repr(e)))


@pytest.mark.timeout(120)
def test_two_gloo_ranks_barrier_and_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=100) for _ in procs)
    for p in procs:
        p.join(timeout=30)
    assert all(p.exitcode == 0 for p in procs)
    assert [o[0] for o in out] == [0, 1]
    for rank, ws, got_rank, local, t in out:
        assert ws == 2 and got_rank == rank and local == rank
        assert t == 15.0  # max over ranks, seen by both


def test_single_rank_needs_no_process_group(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    sys.path.insert(0, ROOT)
    import bench
    ws, rank, local, pg = bench.dist_init()
    assert (ws, rank, local, pg) == (1, 0, 0, None)
    bench.barrier(pg)
    assert bench.max_over_ranks(pg, 3.25) == 3.25


def test_reference_arm_runs_on_rank_zero_only():
    # rank 1 of the reference arm returns at once, without building anything
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        steps, warmup = 1, 0
    assert bench.run_reference(Args(), 2, 1, None) is None
