"""Multi-rank host logic on the CPU (gloo, world size 2; no GPU): system
sharding covers every system exactly once; the key-range decomposition of one
system (the reference's createRanges / newLoadDistribution / key2proc,
SpaceFillingCurves/src/Tree.cpp:165-317) balances work, keeps equal keys on one
rank and agrees with the group ranges; and a system stepped by two gloo ranks,
each walking its key range with the oracle standing in for the GPU walk and
summing accelerations over the ranks, follows the single-process trajectory
exactly."""
import os
import socket

import numpy as np
import torch
import torch.multiprocessing as mp

from nns_gb300 import ic
from nns_gb300.dist import KEY_MAX, SplitSystem, key2proc, key_decomposition, shard_systems, split_groups
from oracle import oracle as O


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, off, q):
    import torch.distributed as dist
    from nns_gb300.dist import max_over_ranks, sum_over_ranks
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    s0, s1, loc = shard_systems(off, rank, world)
    t = max_over_ranks(1.0 + rank)
    nb = sum_over_ranks(float(loc[-1]))
    q.put((rank, s0, s1, t, nb))
    dist.destroy_process_group()


def test_shard_systems_balanced():
    off = np.concatenate([[0], np.cumsum(ic.batched_sizes(512))])
    got = [shard_systems(off, r, 4) for r in range(4)]
    covered = []
    for s0, s1, loc in got:
        covered.extend(range(s0, s1))
        assert loc[0] == 0 and np.all(np.diff(loc) > 0)
    assert covered == list(range(512))
    loads = [loc[-1] for _, _, loc in got]
    assert max(loads) < 1.3 * off[-1] / 4


def _spawn(target, world, *args):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=target, args=(r, world, port, *args, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in procs), key=lambda v: v[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return res


def test_gloo_two_ranks():
    off = np.concatenate([[0], np.cumsum(ic.batched_sizes(64))])
    (r0, a0, b0, t0, n0), (r1, a1, b1, t1, n1) = _spawn(_worker, 2, off)
    assert a0 == 0 and b0 == a1 and b1 == 64
    assert t0 == t1 == 2.0
    assert n0 == n1 == float(off[-1])


def test_split_groups_balances_cost():
    rng = np.random.default_rng(3)
    cost = rng.integers(1, 1000, size=5000).astype(np.float64)
    for world in (1, 2, 3, 8):
        b = split_groups(cost, world)
        assert b[0] == 0 and b[-1] == len(cost) and np.all(np.diff(b) >= 0)
        loads = [cost[b[r]:b[r + 1]].sum() for r in range(world)]
        assert max(loads) - min(loads) <= 2 * cost.max() + 1e-9
    # equal costs: the reference's createRanges split by counts
    assert np.array_equal(split_groups(np.ones(100), 4), [0, 25, 50, 75, 100])


def test_key_ranges_and_key2proc_agree_with_group_ranges():
    """Oracle keys of a disk with planted equal 21-level keys: every body's key
    maps (key2proc) to the rank whose group range holds it, and runs of equal
    keys never straddle two ranks."""
    b = ic.star_disk(5000, seed=ic.SEED0 + 12)
    x = b.x.copy()
    for i in range(0, 5000, 97):  # pairs that share all 21 levels
        x[i + 1] = np.nextafter(x[i], np.float32(2))
        b.y[i + 1], b.z[i + 1] = b.y[i], b.z[i]
    bb = O.bbox(x, b.y, b.z)
    hi, lo = O.keys(x, b.y, b.z, bb, 42)
    perm = np.lexsort((lo, hi))
    keys = hi[perm]
    starts = np.arange(0, len(keys), 32)
    for world in (2, 3, 5):
        cost = np.random.default_rng(world).random(len(starts)) + 0.5
        bounds, ranges = key_decomposition(keys, starts, cost, world)
        assert ranges[0] == 0 and ranges[-1] == KEY_MAX and np.all(np.diff(ranges.astype(np.float64)) >= 0)
        owner_by_group = np.repeat(np.arange(world), np.diff(bounds))
        owner_by_pos = np.repeat(owner_by_group, 32)[:len(keys)]
        assert np.array_equal(key2proc(keys, ranges), owner_by_pos)


class OracleCtx:
    """A context whose walk is the oracle (the CPU stand-in for the GPU walk in
    these host-logic tests): groups of 32 sorted bodies of one system."""

    def __init__(self, m, theta_ref, eps2, dt):
        self.m, self.t, self.e2, self.dt = m, theta_ref, eps2, dt

    def build(self, s):
        self.tree = O.build(s.x.numpy(), s.y.numpy(), s.z.numpy(), self.m)
        self.len = np.zeros(self.group_count(), np.int64)

    def group_count(self):
        return (len(self.m) + 31) // 32

    def forces_groups(self, s, first, count):
        tr = self.tree
        g = np.arange(first, first + count)
        f = O.forces(s.x.numpy(), s.y.numpy(), s.z.numpy(), self.m, tr, self.t, self.e2, groups=g)
        idx = np.concatenate([tr.perm[k * 32:(k + 1) * 32] for k in g]) if count else np.zeros(0, int)
        for t, col in zip((s.ax, s.ay, s.az), range(3)):
            t[torch.as_tensor(idx)] = torch.as_tensor(f.a[idx, col])
        for k in g:
            self.len[k] = f.nlist[tr.perm[k * 32]]

    def group_stats(self):
        return torch.as_tensor(self.len), None

    def integrate(self, s):
        a = np.stack([s.ax.numpy(), s.ay.numpy(), s.az.numpy()], 1)
        out = O.update(s.x.numpy(), s.y.numpy(), s.z.numpy(), s.vx.numpy(), s.vy.numpy(), s.vz.numpy(), a,
                       self.dt)
        for t, v in zip((s.x, s.y, s.z, s.vx, s.vy, s.vz), out):
            t.copy_(torch.as_tensor(v))


class HostState:
    def __init__(self, b):
        f = lambda a: torch.as_tensor(np.array(a, np.float32))  # noqa: E731
        self.x, self.y, self.z = f(b.x), f(b.y), f(b.z)
        self.vx, self.vy, self.vz = f(b.vx), f(b.vy), f(b.vz)
        self.ax, self.ay, self.az = (torch.zeros(len(b.x)) for _ in range(3))


def _split_worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b = ic.plummer(3000, seed=ic.SEED0 + 13)
    s = HostState(b)
    sys = SplitSystem(OracleCtx(b.m, 0.25, 1e-4, 1e-3), s, rank, world)
    bounds = []
    for _ in range(3):
        sys.step(1)
        bounds.append(sys.bounds.tolist())
    q.put((rank, np.stack([s.x.numpy(), s.y.numpy(), s.z.numpy(), s.vx.numpy()]), bounds))
    dist.destroy_process_group()


def test_split_system_two_gloo_ranks_follow_the_single_rank_trajectory():
    res = _spawn(_split_worker, 2)
    b = ic.plummer(3000, seed=ic.SEED0 + 13)
    s = HostState(b)
    one = SplitSystem(OracleCtx(b.m, 0.25, 1e-4, 1e-3), s, 0, 1, allreduce=lambda ts: None)
    one.step(3)
    want = np.stack([s.x.numpy(), s.y.numpy(), s.z.numpy(), s.vx.numpy()])
    (r0, got0, bounds0), (r1, got1, bounds1) = res
    assert np.array_equal(got0, want) and np.array_equal(got1, want)
    assert bounds0 == bounds1  # both ranks agree on the ranges
    lo, mid, hi = bounds0[-1]
    assert lo == 0 and 0 < mid < hi == one.ctx.group_count()
