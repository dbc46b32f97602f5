"""Several GPUs: independent registrations, one process per GPU.

Registrations do not exchange data, so a multi-GPU run is replicas: the cohort is split
by pairs, each rank registers its pairs on its own GPU, and the only collectives are on
the host side -- the max over ranks of the timed region and the gather of per-pair
statistics.  Splitting one volume across GPUs would need a z-slab halo exchange per pass
and is not done.
"""
from __future__ import annotations

from typing import Sequence


def shard_pairs(sizes: Sequence[int], world_size: int) -> list[list[int]]:
    """Pair indices per rank, balanced by work: largest pair first onto the rank with the
    least voxels so far (ties to the lower rank).  `sizes` are voxel counts."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    load = [0] * world_size
    shards: list[list[int]] = [[] for _ in range(world_size)]
    for k in sorted(range(len(sizes)), key=lambda k: (-int(sizes[k]), k)):
        r = min(range(world_size), key=lambda r: (load[r], r))
        shards[r].append(k)
        load[r] += int(sizes[k])
    for s in shards:
        s.sort()
    return shards


def max_over_ranks(value: float, group=None) -> float:
    """The largest `value` over the ranks of the default process group (the whole job's
    time is the slowest rank's); the value itself without a process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def gather_to_rank0(obj, group=None):
    """Every rank's `obj` on rank 0 (a list in rank order), None on the other ranks."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return [obj]
    out = [None] * dist.get_world_size(group) if dist.get_rank(group) == 0 else None
    dist.gather_object(obj, out, dst=0, group=group)
    return out
