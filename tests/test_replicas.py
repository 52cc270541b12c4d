"""Multi-GPU runs are replicas (no collective on the data path): bench.py under
torchrun joins a gloo group only for its barrier and the max-over-ranks timing
and sum-over-ranks work counts.  Two CPU ranks exercise that host logic."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": "0",
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench

    class A:
        pass

    r, w, local, pg = bench.dist_init(A())
    bench.barrier(pg)
    ms = bench.max_over_ranks(pg, 10.0 + rank)  # slowest rank's time
    units = bench.sum_over_ranks(pg, 1000.0 * (rank + 1))  # work of all replicas
    pg.destroy_process_group()
    q.put((r, w, ms, units))


def test_two_replica_ranks_over_gloo():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, *_ in res] == [0, 1]
    for r, w, ms, units in res:
        assert w == 2 and ms == 11.0 and units == 3000.0
