"""Replica sharding of trajectories across processes (one per GPU) and the
deterministic merge of their FP64 moment blocks.

Trajectories are independent, so N processes run disjoint contiguous ranges
of trajectory ids (seeds and Philox keys derive from the id, so any
partitioning produces the same trajectories). Each process reduces its range
into its own moment blocks; the merge concatenates the blocks in rank order.
With T divisible by the total block count B and B divisible by the world
size W, the merged blocks are exactly the blocks a single process would
produce (same trajectories in the same order per block), so the merge is
bit-identical. No collective is needed in the data path; torch.distributed
(gloo or NCCL) is used only to gather the blocks at the end.
"""
from __future__ import annotations

import numpy as np


def shard_range(rank: int, world: int, ntraj: int) -> tuple:
    """[start, stop) trajectory indices of one rank (contiguous, balanced)."""
    return (rank * ntraj) // world, ((rank + 1) * ntraj) // world


def shard_blocks(rank: int, world: int, nblocks: int) -> int:
    if nblocks % world:
        raise ValueError("the block count must be a multiple of the world size")
    return nblocks // world


def merge_blocks(per_rank: list) -> np.ndarray:
    """Concatenate per-rank blocks (..., B_r, N, 3) along the block axis, in rank order."""
    return np.concatenate([np.asarray(b) for b in per_rank], axis=-3)


def gather_blocks(local: np.ndarray, group=None) -> np.ndarray:
    """all_gather of equal-shaped per-rank blocks through torch.distributed, merged in rank order."""
    import torch
    import torch.distributed as dist

    t = torch.from_numpy(np.ascontiguousarray(local))
    out = [torch.empty_like(t) for _ in range(dist.get_world_size(group))]
    dist.all_gather(out, t, group=group)
    return merge_blocks([o.numpy() for o in out])
