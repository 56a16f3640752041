"""Shot sharding across ranks (one process per GPU).

Shots are independent (the reference migrates them one after another,
kernel.cu:791), so a multi-GPU run gives each rank a contiguous block of shots
and combines the per-rank stacks once at the end: the only exchange is a sum
of two interior grids (image and illumination sums), done in float64 so that
the combination adds no rounding beyond each rank's compensated sum.
"""
from __future__ import annotations

import numpy as np


def shard_shots(nshot: int, rank: int, world: int) -> range:
    """Contiguous, balanced block of shot indices for `rank`."""
    if not (0 <= rank < world) or nshot < 0:
        raise ValueError("bad rank/world")
    base, extra = divmod(nshot, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def combine_stacks(up_sum: np.ndarray, down_sum: np.ndarray, nrec: int, inorm: bool, group=None):
    """Image and illumination from per-rank sums of the per-shot images
    (kernel.cu:1042-1059: divide by nrec, then by the illumination).  With a
    torch.distributed group the sums are all-reduced first."""
    s1 = np.asarray(up_sum, np.float64)
    s2 = np.asarray(down_sum, np.float64)
    if group is not None:
        import torch
        import torch.distributed as dist
        t = torch.from_numpy(np.stack([s1, s2]))
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        s1, s2 = t[0].numpy(), t[1].numpy()
    img = (s1 / nrec).astype(np.float32)
    ill = (s2 / nrec).astype(np.float32)
    if inorm:
        img = img / ill
    return img, ill
