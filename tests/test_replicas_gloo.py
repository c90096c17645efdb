"""Replicas-only multi-GPU form of bench.py: each rank runs the same workload,
the timed region is the maximum over ranks and throughput is the sum of the
ranks' pairs.  Exercised here with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    w, r, local, pg = bench.dist_setup()
    bench.barrier(pg)
    t = bench.reduce_max(pg, 1.0 + rank)       # rank 1 is the slower replica
    q.put((r, w, local, t))
    pg.destroy_process_group()


def test_two_rank_replica_reduction():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    assert all(o[3] == pytest.approx(2.0) for o in out)   # max over ranks
