"""Autotuner for the launch parameters of the force walk and the key sort.

In the parity mode the interaction lists are fixed by the reference's
semantics (group of 32, one body per leaf), so the tunable knobs are the ones
that leave the lists unchanged (the buffer size and the stack depth regroup
the candidates into rounds, which can change the last bits of the FP32 force
sums; the launch shape and the digit width change nothing):
  * warps per block of the walk (4, 8, 16) -- occupancy vs. shared memory,
  * candidate buffer size of the walk (64, 96 or 128 slots per warp),
  * walk stack entries per warp (a deeper stack keeps more rounds wide, a
    shallower one leaves shared memory for more blocks),
  * sort digit width (8 bits in 8 passes or 9 bits in 7 passes; a stable LSD
    sort gives the same order for any width).
Outside the parity mode the caller may also offer leaf bucket sizes
(``leaf_sizes``, nbx_params.leaf_size 1..8): they change the tree and the
lists (and the error), so the default offers only one body per leaf.
Candidates are timed with CUDA events on the caller's workload after one
build, in that order, each stage with the winners of the stages before it
(leaf sizes first, over whole build + walk steps); the winner is applied to
the context and cached per (device, n, systems, modes) in
``~/.cache/nbx_autotune.json`` (override with NBX_AUTOTUNE_CACHE).
"""
from __future__ import annotations

import json
import os

import torch

from ._lib import NbxError

CANDIDATES = ((8, 3), (16, 3), (4, 3), (8, 0), (16, 0), (8, 1), (4, 1))
STACK_DEPTHS = (512, 384, 768)
RADIX_BITS = (8, 9)


def _cache_path():
    return os.environ.get("NBX_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "nbx_autotune.json"))


def _key(ctx, n):
    name = torch.cuda.get_device_name(ctx.device)
    nsys = 1 if ctx.offsets is None else len(ctx.offsets) - 1
    return "%s|n=%d|sys=%d|comp=%d|order=%d|moments=%d|multipole=%d" % (
        name, n, nsys, int(ctx.params.compensated), int(ctx.params.key_order), int(ctx.params.moments_mode),
        int(getattr(ctx.params, "multipole", 0)))


def _time(fn, reps):
    """Mean CUDA-event milliseconds of fn() after one untimed call."""
    fn()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(reps):
        fn()
    ev1.record()
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) / reps


def tune_walk(ctx, state, reps: int = 2, candidates=CANDIDATES, use_cache: bool = True,
              stack_depths=STACK_DEPTHS, radix_bits=RADIX_BITS, timer=None, leaf_sizes=None) -> dict:
    """Times the candidate configurations and applies the fastest.  ``timer(fn,
    reps)`` returns milliseconds per call (CUDA events by default).
    ``leaf_sizes`` (None: keep the context's) are leaf bucket sizes to try."""
    timer = timer or _time
    n = int(ctx.offsets[-1])
    key = _key(ctx, n)
    if leaf_sizes is not None:
        key += "|leaves=" + ",".join(str(int(k)) for k in leaf_sizes)
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            cache = json.load(open(path))
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache and "stack_depth" in cache[key]:
        best = cache[key]
        if "leaf_size" in best:
            ctx.set_leaf_size(best["leaf_size"])
        ctx.set_walk(best["warps"], best["variant"])
        ctx.set_tuning(best["radix_bits"], best["stack_depth"])
        return dict(best, cached=True)
    bits0 = int(ctx.params.radix_bits)
    depth0 = int(ctx.params.stack_depth)
    # 0. leaf bucket size (outside the parity mode only), over build + walk
    ltimes = {}
    if leaf_sizes:
        for k in leaf_sizes:
            ctx.set_leaf_size(int(k))

            def step():
                ctx.build(state)
                ctx.forces(state)
            ltimes[str(int(k))] = timer(step, reps)
        ctx.sync()
        ctx.set_leaf_size(int(min(ltimes, key=ltimes.get)))
    ctx.build(state)
    ctx.sync()
    # 1. walk launch shape
    times = {}
    for warps, variant in candidates:
        ctx.set_walk(warps, variant)
        times["%d/%d" % (warps, variant)] = timer(lambda: ctx.forces(state), reps)
    ctx.sync()
    wbest = min(times, key=times.get)
    warps, variant = (int(v) for v in wbest.split("/"))
    ctx.set_walk(warps, variant)
    # 2. stack depth with that shape (a depth whose stacks do not fit the
    #    shape's shared memory is skipped)
    stimes = {}
    for depth in stack_depths:
        ctx.set_tuning(bits0, depth)
        try:
            stimes[str(depth)] = timer(lambda: ctx.forces(state), reps)
        except NbxError:
            continue
    ctx.sync()
    depth = int(min(stimes, key=stimes.get)) if stimes else depth0
    # 3. sort digit width, timed over whole builds
    btimes = {}
    for bits in radix_bits:
        ctx.set_tuning(bits, depth)
        btimes[str(bits)] = timer(lambda: ctx.build(state), reps)
    ctx.sync()
    bits = int(min(btimes, key=btimes.get))
    ctx.set_tuning(bits, depth)
    ctx.build(state)
    best = {"warps": warps, "variant": variant, "stack_depth": depth, "radix_bits": bits,
            "ms": times, "ms_stack": stimes, "ms_build": btimes}
    if leaf_sizes:
        best["leaf_size"] = int(ctx.params.leaf_size)
        best["ms_leaf"] = ltimes
    if use_cache:
        cache[key] = best
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            json.dump(cache, open(path, "w"), indent=1)
        except OSError:
            pass
    return dict(best, cached=False)
