"""Multi-rank paths: one process per GPU.

* Independent systems of a batch shard by contiguous system ranges, balanced by
  body count, with no data-path collective (``shard_systems``).
* One large system splits its force walk over the ranks by space-filling-curve
  key ranges, the decomposition of the reference's parallel code
  (MolecularDynamics/BarnesHutParallel/SpaceFillingCurves/src/Tree.cpp:165-317:
  ``createRanges``, ``newLoadDistribution``, ``updateRange``, ``key2proc``).
  Here every rank holds the whole system and builds the same tree from it (the
  build is deterministic); a rank's share is a contiguous range of walk groups,
  i.e. a range of keys of the sorted order, balanced by the work each group did
  in the last walk (its interaction-list length) instead of by body count.
  Each rank zeroes the accelerations, walks its groups (``nbx_forces_groups``)
  and the ranks sum the accelerations: every body is walked by exactly one rank,
  so the sum equals a single-GPU walk.  Every rank then integrates all bodies.
* Timing reduces with a MAX over ranks.

The collectives are torch.distributed calls (NCCL on GPUs, gloo in the CPU
tests); the reductions are injectable so the host logic is tested without one.
"""
from __future__ import annotations

import numpy as np

KEY_MAX = np.uint64((1 << 63) - 1) + np.uint64(1)  # above every 63-bit key (the reference's KEY_MAX)


def shard_systems(offsets, rank: int, world: int):
    """Contiguous range [s0, s1) of systems for `rank`, balanced by bodies.

    Returns (s0, s1, local_offsets) with local_offsets rebased to 0."""
    off = np.asarray(offsets, dtype=np.int64)
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


def split_groups(costs, nranks: int, valid=None) -> np.ndarray:
    """Contiguous ranges of walk groups, one per rank, with balanced total cost:
    bounds[0] = 0 <= bounds[1] <= ... <= bounds[nranks] = ngroups, rank r walks
    groups [bounds[r], bounds[r+1]).  Inner bounds sit where the cumulative cost
    first reaches r/nranks of the total (``newLoadDistribution`` balances
    particle counts the same way, Tree.cpp:202-261; equal costs give its
    ``createRanges``).  ``valid`` (bool per group) restricts inner bounds to
    allowed group starts; a bound moves forward to the next allowed one."""
    c = np.asarray(costs, np.float64)
    ng = len(c)
    if nranks < 1:
        raise ValueError("nranks must be positive")
    cum = np.concatenate([[0.0], np.cumsum(c)])
    targets = cum[-1] * np.arange(1, nranks) / nranks
    inner = np.searchsorted(cum, targets, side="left")
    if valid is not None:
        ok = np.flatnonzero(np.asarray(valid, bool))  # allowed first groups of a rank
        pos = np.searchsorted(ok, inner, side="left")
        inner = np.array([ok[q] if q < len(ok) else ng for q in pos], np.int64)
    bounds = np.concatenate([[0], inner, [ng]]).astype(np.int64)
    return np.minimum(np.maximum.accumulate(bounds), ng)


def key_decomposition(sorted_keys, group_starts, costs, nranks: int):
    """Key ranges of one system for `nranks` ranks: (bounds, ranges).

    ``bounds`` as split_groups; ``ranges`` are the reference's s->range:
    ranges[0] = 0, ranges[nranks] = KEY_MAX, ranges[r] = the key of the first
    body of rank r (Tree.cpp:171-193).  A boundary is placed only where the key
    strictly increases, so that key2proc and the group ranges agree on every
    body (bodies with equal 21-level keys stay on one rank)."""
    keys = np.asarray(sorted_keys, np.uint64)
    gs = np.asarray(group_starts, np.int64)
    valid = np.ones(len(gs), bool)
    inner = gs[1:]
    valid[1:] = keys[inner] > keys[inner - 1]
    bounds = split_groups(costs, nranks, valid)
    ranges = np.empty(nranks + 1, np.uint64)
    ranges[0] = np.uint64(0)
    ranges[nranks] = KEY_MAX
    for r in range(1, nranks):
        ranges[r] = keys[gs[bounds[r]]] if bounds[r] < len(gs) else KEY_MAX
    return bounds, ranges


def key2proc(keys, ranges) -> np.ndarray:
    """Rank owning each key: r with ranges[r] <= k < ranges[r+1] (Tree.cpp:300-314)."""
    r = np.searchsorted(np.asarray(ranges, np.uint64), np.asarray(keys, np.uint64), side="right") - 1
    return np.clip(r, 0, len(ranges) - 2)


def _allreduce_sum(tensors):
    import torch.distributed as dist
    for t in tensors:
        dist.all_reduce(t, op=dist.ReduceOp.SUM)


class SplitSystem:
    """One system stepped by `world` ranks, each walking a key range of it.

    ``ctx``/``state``: this rank's context and its full copy of the system.  Per
    step: build (same tree on every rank), zero the accelerations, walk this
    rank's groups, sum the accelerations over the ranks, integrate every body,
    and rebalance the ranges by the groups' list lengths of this walk (summed
    over the ranks; each rank knows only its own groups').  ``allreduce`` sums a
    list of tensors in place over the ranks (torch.distributed by default)."""

    def __init__(self, ctx, state, rank: int, world: int, allreduce=None):
        self.ctx, self.s, self.rank, self.world = ctx, state, rank, world
        self.allreduce = allreduce or _allreduce_sum
        self.bounds = None

    def my_groups(self):
        b = self.bounds
        return int(b[self.rank]), int(b[self.rank + 1] - b[self.rank])

    def forces(self, build: bool = True):
        """One force evaluation; build=False when the caller has just built the
        tree of the current positions itself (to time the phases apart)."""
        import torch
        ctx, s = self.ctx, self.s
        if build:
            ctx.build(s)
        if self.bounds is None:
            self.bounds = split_groups(np.ones(ctx.group_count()), self.world)
        for t in (s.ax, s.ay, s.az):
            t.zero_()
        first, count = self.my_groups()
        ctx.forces_groups(s, first, count)
        self.allreduce([s.ax, s.ay, s.az])
        # work of this walk per group: this rank's groups, zero elsewhere, summed over the ranks
        ln, _ = ctx.group_stats()
        cost = torch.zeros(len(ln), dtype=torch.float64, device=ln.device)
        cost[first:first + count] = ln[first:first + count].to(torch.float64)
        self.allreduce([cost])
        self.bounds = split_groups(cost.cpu().numpy() + 1.0, self.world)

    def step(self, nsteps: int = 1):
        for _ in range(nsteps):
            self.forces()
            self.ctx.integrate(self.s)


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
