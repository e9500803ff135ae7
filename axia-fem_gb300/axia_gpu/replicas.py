"""Replica bookkeeping and independent work units for runs on several GPUs of one node.

The linear-static path does not shard without a halo exchange and two
all-reduces per CG iteration, so several GPUs run independent replicas (one
process per GPU, each solving its own copy of the workload, nothing exchanged
on the data path).  A family of independent meshes is the natural unit to
spread instead: `partition_meshes` gives every rank a disjoint subset,
balanced by a work estimate.  The only collective is the timing reduction
here: the job time is the slowest rank's time and the job throughput is all
ranks' units over it.
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


def mesh_work(n_nodes: int, n_blocks: int) -> float:
    """Work estimate of one mesh's solve: its node blocks (one SpMV) times the
    cube root of its nodes (the iteration count grows with the mesh's extent);
    the estimate the multi-mesh solve uses to size its CTA groups."""
    return float(n_blocks) * float(n_nodes) ** (1.0 / 3.0)


def partition_meshes(work, world_size: int):
    """Disjoint subsets of mesh indices, one per rank, each mesh in exactly one:
    meshes in decreasing work (ties by index) go to the rank with the least work
    so far (ties by rank), and every subset is returned in ascending mesh order.
    Deterministic, so every rank computes the same split without communicating."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = sorted(range(len(work)), key=lambda k: (-float(work[k]), k))
    load = [0.0] * world_size
    parts = [[] for _ in range(world_size)]
    for k in order:
        r = min(range(world_size), key=lambda q: (load[q], q))
        parts[r].append(k)
        load[r] += float(work[k])
    return [sorted(p) for p in parts]
