"""The multi-GPU mode is replicas only (one independent solve per rank, no
data exchange).  Its host logic — the max over ranks of the step time and
the whole-job DOF/s — runs here on CPU with world_size 2 over gloo."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 100.0 + 50.0 * rank  # rank 1 is the slower replica
    slow = bench.replica_max(torch, dist, ms, world, torch.device("cpu"))
    out[rank] = (slow, bench.replica_value(1000, world, slow))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_max_and_value_world2():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1] == (150.0, 2 * 1000 / 0.150)


def test_replica_single_rank_is_identity():
    import bench
    assert bench.replica_max(torch, dist, 123.0, 1, torch.device("cpu")) == 123.0
    assert bench.replica_value(10, 1, 1000.0) == pytest.approx(10.0)
