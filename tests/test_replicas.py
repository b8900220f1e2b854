"""Replica timing reduction of bench.py over gloo (world size 2, CPU).

The path does not shard: ``bench.py --gpus N`` runs N independent replicas and
only reduces the timed region's clocks (max over ranks) with a collective.
"""
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
    dev_s, e2e_s = bench.replica_max(dist, 1.0 + rank, 10.0 - rank)
    out[rank] = (dev_s, e2e_s)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_max_over_gloo():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == (2.0, 10.0)
    assert res[1] == (2.0, 10.0)


def test_replica_max_single_process():
    import bench
    assert bench.replica_max(None, 3.0, 4.0) == (3.0, 4.0)
