"""The multi-GPU form of the bench is replicas (independent spectrum-slice
solves, no data-path collective): world_size-2 gloo ranks on the CPU check
the host-side aggregation -- slowest rank's time, eigenpairs summed."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, ws, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        t_solve = [10.0, 12.5][rank]
        t_e2e = [11.0, 14.0][rank]
        nev = [1232, 1230][rank]
        bench.barrier(ws)
        q.put((rank, bench.aggregate(t_solve, t_e2e, nev, ws)))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        value, e2e, t, te = out[r]
        assert t == 12.5 and te == 14.0
        assert value == pytest.approx(2462 / 12.5)
        assert e2e == pytest.approx(2462 / 14.0)


def test_single_rank_aggregation_is_local():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate(2.0, 4.0, 10, 1) == (5.0, 2.5, 2.0, 4.0)
