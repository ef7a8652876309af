"""Sharding one MRG8 stream over several GPUs by jump-ahead.

The path has no data exchange: rank r of a world of size W generates the
outputs [r * n_per_rank, (r + 1) * n_per_rank) of one stream, starting from
the stream state jumped ahead by r * n_per_rank on the host (the block split
of knl/mrg8.h:445-470 and cuda/mrg8_cuda.cu:205-234, one block per GPU).  The
shards concatenate to the sequential stream.  Only timing needs a collective
(a barrier and a max over ranks).
"""
from __future__ import annotations

import numpy as np


def shard_range(n_per_rank: int, rank: int) -> tuple[int, int]:
    """(first output, count) of this rank's shard."""
    if n_per_rank < 0 or rank < 0:
        raise ValueError("n_per_rank and rank must be non-negative")
    return rank * n_per_rank, n_per_rank


def shard_state(seed: int, offset: int) -> np.ndarray:
    """State of the stream seeded from `seed`, `offset` outputs in."""
    from .api import MRG8
    g = MRG8(seed)
    st = np.zeros(8, dtype=np.uint32)
    g.jump_ahead(offset, st)
    g.close()
    return st


def max_over_ranks(value: float, dist=None) -> float:
    """Max of a per-rank measurement (torch.distributed, any backend)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
