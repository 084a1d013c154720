"""The N-GPU benchmark runs independent replicas; its whole-job figure is
the cell-updates of all ranks over the slowest rank's time.  Checked with
two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 1000.0 * (rank + 1)          # rank 1 is the slower replica
    cus = 1_000_000 * (rank + 2)      # replicas may update different counts
    value, tmax = bench.replica_aggregate(ms, cus, world, "cpu")
    out[rank] = (value, tmax)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregate_two_gloo_ranks():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
            assert p.exitcode == 0
        for r in range(world):
            value, tmax = out[r]
            assert tmax == 2000.0
            assert value == pytest.approx((2_000_000 + 3_000_000) / 2.0)


def test_replica_aggregate_single():
    import bench
    assert bench.replica_aggregate(500.0, 1_000_000, 1, "cpu") == (2_000_000.0, 500.0)
