"""Multi-GPU path (replicas only): timing aggregation across ranks, run as two
gloo processes on the CPU."""
from __future__ import annotations

import os
import socket

import pytest


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(__file__)),
                                    "cylinder-flow_gb300"))
    from cflbm.replicas import aggregate_mlups
    # rank r took (r + 1) seconds for 10 steps of 1e6 cells
    v, t = aggregate_mlups(float(rank + 1), 1_000_000, 10, world)
    out[rank] = (v, t)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_aggregation_uses_slowest_rank():
    import torch.multiprocessing as mp
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        v, t = out[r]
        assert t == pytest.approx(2.0)
        assert v == pytest.approx(2 * 1_000_000 * 10 / 2.0 / 1e6)


def test_single_rank_is_local():
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(__file__)),
                                    "cylinder-flow_gb300"))
    from cflbm.replicas import aggregate_mlups
    v, t = aggregate_mlups(0.5, 100, 4, 1)
    assert t == 0.5 and v == pytest.approx(100 * 4 / 0.5 / 1e6)
