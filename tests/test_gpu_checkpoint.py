"""Checkpoint / resume (nbx_checkpoint_*) and the node-pool overflow guard.

* A run resumed from a checkpoint continues bit for bit (batched systems,
  compensated forces), also into a context with another walk configuration,
  multipole order or leaf size (the checkpoint restores them).
* A corrupted or truncated checkpoint is refused with NBX_ERR_FORMAT and
  changes nothing; a context too small for it is refused with NBX_ERR_ARG.
* A tree larger than the node pool reports NBX_ERR_CAPACITY; the failed tree is
  never walked (NBX_ERR_STATE until a new build), and systems that fit the pool
  still work.
"""
import numpy as np
import pytest

from nns_gb300 import ic

pytestmark = pytest.mark.gpu


def _run(ctx, s, k):
    ctx.step(s, k)
    ctx.sync()
    return np.stack([t.cpu().numpy() for t in (s.x, s.y, s.z, s.vx, s.vy, s.vz)])


def test_resume_is_bit_exact(cuda):
    from nns_gb300.barnes_hut import Context, State
    bodies, off = ic.batched_star_disks(3, seed=ic.SEED0 + 40)
    n = int(off[-1])
    ctx = Context(max_bodies=n, max_systems=3, theta=0.5, eps=0.01, dt=1e-3, compensated=1)
    ctx.set_systems(off)
    s = State.from_bodies(bodies)
    _run(ctx, s, 3)
    buf = ctx.checkpoint(s)
    want = _run(ctx, s, 4)
    ctx2 = Context(max_bodies=n + 100, max_systems=4, theta=0.9, eps=0.2, dt=5e-2)
    s2 = State.empty(n)
    ctx2.restore(s2, buf)
    assert ctx2.offsets == [int(v) for v in off]
    assert ctx2.constants() == ctx.constants()
    got = _run(ctx2, s2, 4)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("mode", ["tuned", "quadrupole_buckets"])
def test_resume_restores_the_walk_configuration(cuda, mode):
    """The checkpoint carries what sets the force bits beyond the constants: the
    walk's buffer variant and stack depth (they group candidates into rounds),
    the multipole order and the leaf size; a context with other settings resumes
    bit for bit."""
    from nns_gb300.barnes_hut import Context, State
    b = ic.plummer(30000, seed=ic.SEED0 + 41)
    n = len(b.x)
    ctx = Context(max_bodies=n, theta=0.5, eps=0.01, dt=1e-3)
    ctx.set_systems([0, n])
    ctx.set_walk(4, 1)
    ctx.set_tuning(8, 384)
    if mode == "quadrupole_buckets":
        ctx.set_multipole(1)
        ctx.set_leaf_size(4)
    s = State.from_bodies(b)
    _run(ctx, s, 2)
    buf = ctx.checkpoint(s)
    want = _run(ctx, s, 3)
    ctx2 = Context(max_bodies=n, theta=0.5, eps=0.01, dt=1e-3)
    ctx2.set_walk(8, 2)  # the one-cell walk, which has no quadrupole form: restore changes it first
    s2 = State.empty(n)
    ctx2.restore(s2, buf)
    got = _run(ctx2, s2, 3)
    assert np.array_equal(got, want)


def test_bad_checkpoints_are_refused(cuda):
    from nns_gb300._lib import NbxError
    from nns_gb300.barnes_hut import Context, State
    b = ic.star_disk(2000)
    ctx = Context(max_bodies=2000)
    ctx.set_systems([0, 2000])
    s = State.from_bodies(b)
    buf = ctx.checkpoint(s)
    x0 = s.x.cpu().numpy().copy()
    for pos, bit in ((20, 1), (5000, 4), (0, 2)):  # header field, payload, magic
        bad = buf.copy()
        bad[pos] ^= bit
        s.x.fill_(7.0)
        with pytest.raises(NbxError) as e:
            ctx.restore(s, bad)
        assert e.value.code == 12  # NBX_ERR_FORMAT
        assert float(s.x[0].item()) == 7.0  # nothing was copied
    with pytest.raises(NbxError) as e:
        ctx.restore(s, buf[:-8])
    assert e.value.code == 12
    small = Context(max_bodies=1000)
    with pytest.raises(NbxError) as e:
        small.restore(State.empty(1000), buf)
    assert e.value.code == 1  # NBX_ERR_ARG
    ctx.restore(s, buf)
    assert np.array_equal(s.x.cpu().numpy(), x0)


def _fnv1a(data: bytes, h: int = 1469598103934665603) -> int:
    for b in data:
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def test_out_of_range_settings_are_refused(cuda):
    """A checkpoint whose header hash is valid but whose settings are outside
    their ranges (multipole order 7, here) is malformed: NBX_ERR_FORMAT, and
    neither the context nor the state changes."""
    from nns_gb300._lib import NbxError
    from nns_gb300.barnes_hut import Context, State
    b = ic.star_disk(2000)
    ctx = Context(max_bodies=2000, theta=0.5, eps=0.01)
    ctx.set_systems([0, 2000])
    s = State.from_bodies(b)
    buf = ctx.checkpoint(s).copy()
    # header: magic 8, version 4, nsys 4, nbodies 8, 4 floats, 8 int32 (compensated,
    # key order, warps, variant, multipole, leaf size, stack depth, reserved), hash 8
    multipole_at = 8 + 4 + 4 + 8 + 16 + 4 * 4
    buf[multipole_at:multipole_at + 4] = np.frombuffer(np.int32(7).tobytes(), np.uint8)
    nsys = int(np.frombuffer(buf[12:16].tobytes(), np.int32)[0])
    hash_at = 72
    h = _fnv1a(bytes(buf[80:80 + 8 * (nsys + 1)]), _fnv1a(bytes(buf[:hash_at])))
    buf[hash_at:hash_at + 8] = np.frombuffer(np.uint64(h).tobytes(), np.uint8)
    t0 = ctx.constants()
    s.x.fill_(7.0)
    with pytest.raises(NbxError) as e:
        ctx.restore(s, buf)
    assert e.value.code == 12  # NBX_ERR_FORMAT
    assert float(s.x[0].item()) == 7.0 and ctx.constants() == t0


def test_node_pool_overflow_is_reported(cuda):
    from nns_gb300._lib import NbxError
    from nns_gb300.barnes_hut import Context, State
    b = ic.star_disk(1000)
    ctx = Context(max_bodies=1000, node_capacity=1001)
    ctx.set_systems([0, 1000])
    s = State.from_bodies(b)
    ctx.build(s)
    ctx.forces(s)
    with pytest.raises(NbxError) as e:
        ctx.sync()
    assert e.value.code == 4  # NBX_ERR_CAPACITY
    with pytest.raises(NbxError) as e:  # the failed tree is never walked
        ctx.forces(s)
    assert e.value.code == 9  # NBX_ERR_STATE
    small = ic.star_disk(50)
    s2 = State.from_bodies(small)
    ctx.set_systems([0, 50])
    ctx.build(s2)
    ctx.forces(s2)
    ctx.sync()
    a = s2.acc()
    assert np.isfinite(a).all() and np.abs(a).sum() > 0
