"""Host logic of the tuning knobs, on the CPU (no GPU calls).

* The autotuner's stages against a fake context and a fake timer: the walk
  shape is chosen first, then the stack depth with that shape (a depth the
  context rejects is skipped), then the sort digit width over builds; the
  winner is applied and cached, and a cached entry is applied without timing.
* An LSD radix sort gives the same stable order with 8-bit digits (8 passes)
  and 9-bit digits (7 passes) over 63-bit keys with many duplicates: the
  property that makes the digit width a speed-only knob.
"""
import json

import numpy as np
import pytest

from nns_gb300 import autotune
from nns_gb300._lib import NbxError


class FakeParams:
    compensated = 0
    radix_bits = 8
    stack_depth = 512
    leaf_size = 1


class FakeCtx:
    """Records the configuration each call runs with."""

    def __init__(self, reject_depth=None):
        self.offsets = np.array([0, 4096])
        self.params = FakeParams()
        self.warps, self.variant = 8, 3
        self.reject_depth = reject_depth
        self.calls = []

    def set_walk(self, warps, variant):
        self.warps, self.variant = warps, variant

    def set_tuning(self, bits, depth):
        self.params.radix_bits, self.params.stack_depth = bits, depth

    def set_leaf_size(self, k):
        self.params.leaf_size = k

    def build(self, state):
        self.calls.append(("build", self.params.radix_bits))

    def forces(self, state):
        if self.params.stack_depth == self.reject_depth:
            raise NbxError(1, "nbx_forces", "walk: stack_depth too large")
        self.calls.append(("forces", self.warps, self.variant, self.params.stack_depth))

    def sync(self):
        pass


def fake_timer(ctx, table):
    """Milliseconds from the configuration the timed call ran with."""

    def timer(fn, reps):
        n0 = len(ctx.calls)
        fn()
        call = ctx.calls[n0]
        return table[call]
    return timer


def _table():
    t = {}
    for w, v in autotune.CANDIDATES:
        for d in autotune.STACK_DEPTHS:
            t[("forces", w, v, d)] = 10.0 + (0 if (w, v) == (4, 1) else 1) + (0 if d == 768 else 0.5)
    t[("build", 8)] = 2.0
    t[("build", 9)] = 1.5
    return t


def test_stages_pick_and_apply_the_fastest(tmp_path, monkeypatch):
    monkeypatch.setenv("NBX_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "_key", lambda ctx, n: "fake|n=%d" % n)
    ctx = FakeCtx()
    r = autotune.tune_walk(ctx, None, timer=fake_timer(ctx, _table()))
    assert (r["warps"], r["variant"], r["stack_depth"], r["radix_bits"]) == (4, 1, 768, 9)
    assert (ctx.warps, ctx.variant, ctx.params.stack_depth, ctx.params.radix_bits) == (4, 1, 768, 9)
    # the stack depths were timed with the chosen shape only
    assert {c[1:3] for c in ctx.calls if c[0] == "forces" and c[3] != 512} == {(4, 1)}
    assert not r["cached"]
    cached = json.load(open(tmp_path / "tune.json"))["fake|n=4096"]
    assert cached["stack_depth"] == 768 and cached["radix_bits"] == 9
    ctx2 = FakeCtx()
    r2 = autotune.tune_walk(ctx2, None, timer=lambda fn, reps: pytest.fail("timed a cached entry"))
    assert r2["cached"] and (ctx2.warps, ctx2.variant, ctx2.params.stack_depth, ctx2.params.radix_bits) == (4, 1, 768, 9)


def test_a_rejected_stack_depth_is_skipped(tmp_path, monkeypatch):
    monkeypatch.setattr(autotune, "_key", lambda ctx, n: "fake|n=%d" % n)
    ctx = FakeCtx(reject_depth=768)
    r = autotune.tune_walk(ctx, None, use_cache=False, timer=fake_timer(ctx, _table()))
    assert "768" not in r["ms_stack"] and r["stack_depth"] in (384, 512)
    assert ctx.params.stack_depth == r["stack_depth"]


def _lsd_order(keys, bits):
    """Stable LSD radix sort of 63-bit keys by digits of the given width."""
    order = np.arange(len(keys))
    mask = (1 << bits) - 1
    for shift in range(0, 63, bits):
        d = (keys[order] >> np.uint64(shift)) & np.uint64(mask)
        order = order[np.argsort(d, kind="stable")]
    return order


def test_digit_width_gives_the_same_stable_order():
    rng = np.random.default_rng(7)
    keys = rng.integers(0, 1 << 63, size=20000, dtype=np.uint64)
    keys[::3] = keys[1::3][: len(keys[::3])]  # many equal keys: stability decides their order
    keys[-500:] &= np.uint64((1 << 20) - 1)   # short keys: empty high digits
    want = np.argsort(keys, kind="stable")
    assert np.array_equal(_lsd_order(keys, 8), want)
    assert np.array_equal(_lsd_order(keys, 9), want)


def test_cache_key_separates_orders_and_moment_passes(monkeypatch):
    """Hilbert and Lebesgue order, the centre-of-mass pass and the multipole order
    change the tree or the walk's cost, so a tuning result for one is never
    reused for another."""
    from types import SimpleNamespace

    from nns_gb300 import autotune
    monkeypatch.setattr(autotune.torch.cuda, "get_device_name", lambda dev: "fake")
    keys = set()
    for order in (0, 1):
        for moments in (0, 1, 2):
            for comp in (0, 1):
                for mp in (0, 1):
                    p = SimpleNamespace(compensated=comp, key_order=order, moments_mode=moments, multipole=mp)
                    keys.add(autotune._key(SimpleNamespace(device=0, offsets=[0, 100], params=p), 100))
    assert len(keys) == 24


def test_leaf_sizes_are_offered_only_on_request(tmp_path, monkeypatch):
    """The leaf bucket stage runs only when the caller offers leaf sizes (outside
    the parity mode); it times build + walk steps, applies the fastest size
    before the other stages and caches it under its own key."""
    monkeypatch.setenv("NBX_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "_key", lambda ctx, n: "fake|n=%d" % n)
    step_ms = {1: 9.0, 4: 6.0, 8: 7.0}

    def timer_for(ctx):
        def timer(fn, reps):
            n0 = len(ctx.calls)
            fn()
            kinds = [c[0] for c in ctx.calls[n0:]]
            if kinds == ["build", "forces"]:
                return step_ms[ctx.params.leaf_size]
            return 1.0
        return timer

    ctx = FakeCtx()
    r = autotune.tune_walk(ctx, None, timer=timer_for(ctx))
    assert "leaf_size" not in r and ctx.params.leaf_size == 1
    ctx = FakeCtx()
    r = autotune.tune_walk(ctx, None, timer=timer_for(ctx), leaf_sizes=(1, 4, 8))
    assert r["leaf_size"] == 4 and ctx.params.leaf_size == 4 and r["ms_leaf"] == {"1": 9.0, "4": 6.0, "8": 7.0}
    ctx2 = FakeCtx()
    r2 = autotune.tune_walk(ctx2, None, timer=lambda fn, reps: pytest.fail("timed a cached entry"),
                            leaf_sizes=(1, 4, 8))
    assert r2["cached"] and ctx2.params.leaf_size == 4
