"""Sharding a batch of independent alignment jobs across ranks (one process per GPU).

Every job is a pure function of its own inputs (crates/bwa-neon/src/batched.rs:41-45), so the
path shards with no device collective: each rank takes a contiguous range of the batch, runs it on
its own GPU, and the results come back in job order.  Timing takes the maximum over ranks.  These
helpers hold the host-side logic (ranges, reduction, result assembly); they work with any
torch.distributed backend (gloo on CPU for the tests, nccl between GPUs).
"""
from __future__ import annotations

import numpy as np


def shard_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """[start, stop) of rank's contiguous share of n jobs; shares differ by at most one job."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError("bad shard arguments")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(x: float, device=None) -> float:
    """The maximum of x over all ranks (the slowest rank sets a step's time)."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_results(part: np.ndarray, n: int) -> np.ndarray | None:
    """Every rank's result slice (a structured array, in job order within the slice) assembled in
    job order on rank 0; None on the other ranks."""
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return part
    world, rank = dist.get_world_size(), dist.get_rank()
    parts = [None] * world if rank == 0 else None
    dist.gather_object(part, parts, dst=0)
    if rank != 0:
        return None
    out = np.concatenate(parts) if parts else part[:0]
    if len(out) != n:
        raise RuntimeError(f"gathered {len(out)} results for {n} jobs")
    return out
