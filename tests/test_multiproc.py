"""Multi-process host logic on CPU (gloo, world size 2).

bench.py runs N independent replicas (the search path does not shard): each
rank enumerates the same puzzle on its own GPU, the timed region is bracketed
by barriers, the time is the maximum over ranks and the work is summed.  This
checks that aggregation with two CPU ranks."""
import os
import socket
import sys

import pytest

from conftest import REPO

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(REPO))
    import bench

    d = bench.Dist(world)
    d.barrier()
    t = d.max(1.0 + rank)          # per-rank timed-region seconds
    w = d.sum(100.0 * (rank + 1))  # per-rank states processed
    d.barrier()
    d.close()
    q.put((rank, t, w))


def test_replica_aggregation_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [2.0, 2.0]      # max over ranks
    assert [r[2] for r in res] == [300.0, 300.0]  # summed work
