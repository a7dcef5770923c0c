"""Adjoint (trajectory gradients) on the GPU.

* dL/d(x0, v0, m) from the hand-written adjoint kernels (FP32, FP64 source
  accumulation) against FP64 central finite differences of the same
  trajectory replayed in FP64 with the recorded interaction lists (h = 1e-6),
  along random unit directions: error <= 1e-4 of the gradient norm.
* The forward steps with the recording walk, so the recompute is bit-exact;
  the checkpoint interval does not change the gradients (only the order of
  FP64 atomic additions may differ).
* The torch.autograd.Function wrapper returns the same gradients.
"""
import numpy as np
import pytest

from nns_gb300 import ic

pytestmark = pytest.mark.gpu


def _setup(n=2048, T=20, C=5, tape=None, seed=3):
    import torch
    from nns_gb300.adjoint import Adjoint
    from nns_gb300.barnes_hut import Context, State
    b = ic.plummer(n, seed=ic.SEED0 + seed)
    ctx = Context(max_bodies=n, theta=0.5, eps=0.01, dt=1e-3)
    ctx.set_systems([0, n])
    s = State.from_bodies(b)
    ctx.step(s, T)
    ctx.sync()
    rng = np.random.default_rng(seed)
    xt = np.stack([s.x.cpu().numpy(), s.y.cpu().numpy(), s.z.cpu().numpy()])
    target = torch.as_tensor((xt + 0.01 * rng.standard_normal(xt.shape)).astype(np.float32), device="cuda")
    adj = Adjoint(ctx, T, C, 8192, tape or C)
    return b, ctx, adj, target


def _grads(b, adj, target):
    from nns_gb300.barnes_hut import State
    s = State.from_bodies(b)
    loss = adj.forward(s, target)
    gx, gv, gm = adj.backward(s)
    g = np.concatenate([gx.cpu().numpy(), gv.cpu().numpy(), gm.cpu().numpy()[None]]).astype(np.float64)
    return loss, g


def test_adjoint_matches_fp64_finite_differences(cuda):
    import torch
    from nns_gb300.adjoint import random_directions
    from nns_gb300.barnes_hut import State
    n, T = 2048, 20
    b, ctx, adj, target = _setup(n, T, 5, tape=T)
    loss32, g = _grads(b, adj, target)
    adj.record(State.from_bodies(b))
    base = np.stack([b.x, b.y, b.z, b.vx, b.vy, b.vz, b.m]).astype(np.float64)
    dev = lambda a: torch.as_tensor(a, device="cuda")  # noqa: E731
    loss64 = adj.replay_fp64(dev(base))
    assert abs(loss64 - loss32) / loss32 < 1e-4, (loss64, loss32)
    h = 1e-6
    gnorm = np.linalg.norm(g)
    errs = []
    for u in random_directions(n, 6):
        lp = adj.replay_fp64(dev(base + h * u))
        lm = adj.replay_fp64(dev(base - h * u))
        fd = (lp - lm) / (2 * h)
        ad = float((g * u).sum())
        errs.append(abs(fd - ad) / gnorm)
    assert max(errs) <= 1e-4, errs


def test_forward_steps_with_the_recording_walk(cuda):
    """The adjoint's forward (the 96-slot walk, recording on its last segment)
    ends bit for bit where T ordinary steps with the 96-slot walk end: recording
    changes no force, so the reverse pass recomputes exactly the forward."""
    from nns_gb300.barnes_hut import Context, State
    n, T = 2048, 12
    b, ctx, adj, target = _setup(n, T, 5)  # segments of 5, 5, 2 steps
    s = State.from_bodies(b)
    adj.forward(s, target)
    ref = Context(max_bodies=n, theta=0.5, eps=0.01, dt=1e-3)
    ref.set_systems([0, n])
    ref.set_walk(8, 3)
    s2 = State.from_bodies(b)
    ref.step(s2, T)
    ref.sync()
    for got, want in zip(s.host(), s2.host()):
        assert np.array_equal(got, want)


def test_step_graphs_follow_context_changes(cuda):
    """The adjoint replays captured step graphs; after the context's constants
    change it recaptures them, so its forward ends where a fresh adjoint's does
    (the forward's end state is deterministic: compared bit for bit)."""
    from nns_gb300.adjoint import Adjoint
    from nns_gb300.barnes_hut import State
    b, ctx, adj, target = _setup(1024, 6, 3)

    def end_state(a):
        s = State.from_bodies(b)
        a.forward(s, target)
        return s.host()

    p1 = end_state(adj)
    assert all(np.array_equal(u, v) for u, v in zip(end_state(adj), p1))  # replayed graphs
    t, e2 = ctx.constants()
    ctx.set_constants(t, 4 * e2, 0)
    p2 = end_state(adj)
    assert not np.array_equal(p2[3], p1[3])
    p3 = end_state(Adjoint(ctx, 6, 3, 8192, 3))
    assert all(np.array_equal(u, v) for u, v in zip(p2, p3))


def test_checkpoint_interval_does_not_change_gradients(cuda):
    b, ctx, adj5, target = _setup(1024, 12, 4)
    _, g4 = _grads(b, adj5, target)
    from nns_gb300.adjoint import Adjoint
    adj12 = Adjoint(ctx, 12, 12, 8192, 12)
    _, g12 = _grads(b, adj12, target)
    # recompute is bit-exact; only the order of FP64 atomic additions differs
    assert np.allclose(g4, g12, rtol=1e-5, atol=1e-7 * np.abs(g4).max())


def test_radix_width_does_not_change_the_adjoint(cuda):
    """With 9-bit sort digits (7 passes) the adjoint's builds write the sort
    permutation into its taped arrays as with 8-bit digits: the forward ends at
    the same state bit for bit and the gradients agree (up to the order of the
    FP64 atomic additions)."""
    from nns_gb300.barnes_hut import State
    b, ctx, adj, target = _setup(1024, 8, 4)
    s8 = State.from_bodies(b)
    adj.forward(s8, target)
    _, g8 = _grads(b, adj, target)
    ctx.set_tuning(9, 512)
    s9 = State.from_bodies(b)
    adj.forward(s9, target)
    for u, v in zip(s8.host(), s9.host()):
        assert np.array_equal(u, v)
    _, g9 = _grads(b, adj, target)
    assert np.allclose(g8, g9, rtol=1e-5, atol=1e-7 * np.abs(g8).max())


def test_autograd_function(cuda):
    import torch
    from nns_gb300.adjoint import TrajectoryLoss
    b, ctx, adj, target = _setup(1024, 10, 5)
    x0 = torch.tensor(np.stack([b.x, b.y, b.z]), device="cuda", requires_grad=True)
    v0 = torch.tensor(np.stack([b.vx, b.vy, b.vz]), device="cuda", requires_grad=True)
    m = torch.tensor(b.m, device="cuda", requires_grad=True)
    loss = TrajectoryLoss.apply(x0, v0, m, target, adj)
    loss.backward()
    _, g = _grads(b, adj, target)
    tol = 1e-6 * np.abs(g).max()
    assert np.allclose(x0.grad.cpu().numpy(), g[0:3], rtol=1e-5, atol=tol)
    assert np.allclose(m.grad.cpu().numpy(), g[6], rtol=1e-5, atol=tol)


def test_adjoint_against_fp64_direct_sum_adjoint(cuda):
    """4096-body run: the Barnes-Hut adjoint against the exact gradient of the
    FP64 direct-sum trajectory (they differ by the tree approximation only)."""
    from oracle import oracle as O
    n, T = 4096, 20
    b, ctx, adj, target = _setup(n, T, 10)
    _, g = _grads(b, adj, target)
    x0 = np.stack([b.x, b.y, b.z]).astype(np.float64)
    v0 = np.stack([b.vx, b.vy, b.vz]).astype(np.float64)
    _, gx, gv, gm = O.direct_adjoint_fp64(x0, v0, b.m, target.cpu().numpy(), 1e-4, 1e-3, T)
    want = np.concatenate([gx, gv, gm[None]])
    rel = np.linalg.norm(g - want) / np.linalg.norm(want)
    assert rel < 2e-2, rel
    for k, (a, w) in enumerate(((g[0:3], gx), (g[3:6], gv), (g[6], gm))):
        r = np.linalg.norm(a - w) / np.linalg.norm(w)
        assert r < 5e-2, (k, r)


def test_adjoint_with_a_tiny_softening(cuda):
    """eps = 1e-9: each body's own list entry has d = 0 and r = eps, where
    r^-5 alone would overflow FP32 (0 * inf in the force VJP).  The VJP is
    evaluated in the unit vector d / r: the gradients are finite and agree with
    FP64 central finite differences of the FP64 replay within 1e-4 of the
    gradient norm."""
    import torch
    from nns_gb300.adjoint import Adjoint, random_directions
    from nns_gb300.barnes_hut import Context, State
    n, T = 2048, 4
    b = ic.plummer(n, seed=ic.SEED0 + 5)
    ctx = Context(max_bodies=n, theta=0.5, eps=1e-9, dt=1e-3)
    ctx.set_systems([0, n])
    s = State.from_bodies(b)
    ctx.step(s, T)
    ctx.sync()
    xt = np.stack([s.x.cpu().numpy(), s.y.cpu().numpy(), s.z.cpu().numpy()])
    rng = np.random.default_rng(5)
    target = torch.as_tensor((xt + 0.01 * rng.standard_normal(xt.shape)).astype(np.float32), device="cuda")
    adj = Adjoint(ctx, T, 2, 8192, T)
    loss32, g = _grads(b, adj, target)
    assert np.isfinite(g).all()
    adj.record(State.from_bodies(b))
    base = np.stack([b.x, b.y, b.z, b.vx, b.vy, b.vz, b.m]).astype(np.float64)
    dev = lambda a: torch.as_tensor(a, device="cuda")  # noqa: E731
    assert abs(adj.replay_fp64(dev(base)) - loss32) / loss32 < 1e-4
    h, gnorm = 1e-6, np.linalg.norm(g)
    errs = []
    for u in random_directions(n, 4):
        fd = (adj.replay_fp64(dev(base + h * u)) - adj.replay_fp64(dev(base - h * u))) / (2 * h)
        errs.append(abs(fd - float((g * u).sum())) / gnorm)
    assert max(errs) <= 1e-4, errs
