"""The multi-GPU host logic (replicas of independent registrations) on CPU: two gloo
ranks split a cohort by pairs, take the max of their timings and gather per-pair
statistics on rank 0 -- the collectives bench.py uses with NCCL, one GPU per rank."""
import os
import socket

import pytest

from fastreg_gb300.replicas import shard_pairs


def test_shard_pairs_balanced_and_complete():
    sizes = [96 * 112 * 96, 192 * 224 * 192, 128 * 160 * 128, 160 * 112 * 96, 192 * 160 * 192, 96 * 224 * 128,
             128 * 112 * 192]
    for ws in (1, 2, 3, 8):
        shards = shard_pairs(sizes, ws)
        assert sorted(k for s in shards for k in s) == list(range(len(sizes)))
        loads = [sum(sizes[k] for k in s) for s in shards]
        # greedy largest-first: no rank exceeds the mean by more than the largest pair
        assert max(loads) - sum(sizes) / ws <= max(sizes)
    assert shard_pairs([5, 5, 5, 5], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        shard_pairs([1], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, sizes, q):
    import torch.distributed as dist
    from fastreg_gb300.replicas import gather_to_rank0, max_over_ranks, shard_pairs
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        mine = shard_pairs(sizes, ws)[rank]
        t = max_over_ranks(10.0 + rank)  # each rank's "time"
        stats = gather_to_rank0({k: float(sizes[k]) for k in mine})
        if rank == 0:
            q.put((t, stats))
        else:
            q.put((t, None))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_and_gather():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    sizes = [1000, 3000, 2000, 500, 2500]
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(t == 11.0 for t, _ in out)  # the max over ranks
    gathered = [s for _, s in out if s is not None]
    assert len(gathered) == 1
    merged = {}
    for d in gathered[0]:
        merged.update(d)
    assert sorted(merged) == list(range(len(sizes)))  # every pair once, from both ranks
