"""Multi-rank helpers: one process per GPU, no data-path collective.

Independent systems shard by contiguous system ranges (balanced by body
count); a single large system runs as replicas.  Timing is reduced with a MAX
over ranks.  Works with any torch.distributed backend (NCCL on GPUs, gloo in
the CPU tests).
"""
from __future__ import annotations

import numpy as np


def shard_systems(offsets, rank: int, world: int):
    """Contiguous range [s0, s1) of systems for `rank`, balanced by bodies.

    Returns (s0, s1, local_offsets) with local_offsets rebased to 0."""
    off = np.asarray(offsets, dtype=np.int64)
    nsys = len(off) - 1
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    total = off[-1]
    # system s goes to the rank whose body-count quantile holds its midpoint
    mid = (off[:-1] + off[1:]) / 2.0
    owner = np.minimum((mid * world / max(total, 1)).astype(np.int64), world - 1)
    idx = np.nonzero(owner == rank)[0]
    if idx.size == 0:
        return 0, 0, np.zeros(1, np.int64)
    s0, s1 = int(idx[0]), int(idx[-1]) + 1
    return s0, s1, off[s0:s1 + 1] - off[s0]


def max_over_ranks(value: float, device=None) -> float:
    """MAX of a scalar over the ranks of the default process group."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
