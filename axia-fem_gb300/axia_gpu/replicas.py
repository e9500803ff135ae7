"""Replica bookkeeping for runs on several GPUs of one node.

The linear-static path does not shard without a halo exchange and two
all-reduces per CG iteration, so several GPUs run independent replicas (one
process per GPU, each solving its own copy of the workload, nothing exchanged
on the data path).  The only collective is the timing reduction here: the job
time is the slowest replica's time and the job throughput is all replicas'
units over it.
"""
from __future__ import annotations

import os


def world():
    """(rank, local_rank, world_size) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """The maximum of a per-rank float over the process group (identity without one)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, seconds: float, dist=None, device=None):
    """(throughput, job_seconds): every rank processed units_per_rank in its own
    `seconds`; the job took the slowest rank's time."""
    job_s = max_over_ranks(seconds, dist, device)
    n = dist.get_world_size() if dist is not None and dist.is_initialized() else 1
    return units_per_rank * n / job_s, job_s
