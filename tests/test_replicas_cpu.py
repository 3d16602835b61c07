"""Replica plumbing of bench.py (N > 1 GPUs run independent replicas): two gloo
ranks on CPU agree on the max-over-ranks time and the whole-job value."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, ws: int, port: int, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), QGB_DIST_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    r, w, local = bench.dist_init()
    seconds = [2.0, 3.0][r]  # rank 1 is the slower replica
    bench.dist_barrier(w)
    t = bench.dist_max(seconds, w)
    out.put((r, w, local, t, bench.replica_value(160.0, t, w)))
    dist.destroy_process_group()


def test_two_gloo_replicas_max_over_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [x[0] for x in res] == [0, 1] and all(x[1] == 2 for x in res)
    assert all(x[3] == pytest.approx(3.0) for x in res)  # both ranks see the slowest time
    assert all(x[4] == pytest.approx(160.0 * 2 / 3.0) for x in res)
