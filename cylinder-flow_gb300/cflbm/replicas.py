"""Replica aggregation for multi-GPU runs.

The solver does not shard: on N GPUs, N independent replicas run (one process
per GPU).  The only cross-rank traffic is the timing all-reduce used to report
whole-job throughput: the slowest rank's time bounds the job.
"""
from __future__ import annotations


def max_over_ranks(x: float, world: int) -> float:
    """Maximum of a scalar over all ranks of the default process group."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_mlups(local_seconds: float, cells: int, steps: int, world: int) -> tuple[float, float]:
    """(whole-job MLUPS, max seconds): every rank updates `cells` cells `steps`
    times; the job takes as long as its slowest rank."""
    t = max_over_ranks(local_seconds, world)
    return world * cells * steps / t / 1e6, t
