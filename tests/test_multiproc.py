"""The N > 1 bench path on CPU: two gloo ranks, each timing its own replica,
agree on the max-over-ranks time and the whole-job value (replicas only, no
data-path collective)."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, ms_local, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    value, ms = bench.replica_value(ms_local[rank], 1000, world)
    out[rank] = (value, ms)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_gloo():
    import torch.multiprocessing as mp
    world = 2
    ms_local = [2.0, 5.0]
    mgr = mp.Manager()
    out = mgr.dict()
    port = _free_port()
    mp.spawn(_worker, args=(world, port, ms_local, out), nprocs=world, join=True)
    for r in range(world):
        value, ms = out[r]
        assert ms == 5.0
        assert value == pytest.approx(world * 1000 / 5e-3)


def test_single_rank_value():
    import bench
    v, ms = bench.replica_value(4.0, 2000, 1)
    assert ms == 4.0 and v == pytest.approx(2000 / 4e-3)
