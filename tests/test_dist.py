"""Multi-rank host logic on CPU (gloo, world size 2): system sharding covers
every system exactly once, and timings reduce with MAX over ranks."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

from nns_gb300 import ic
from nns_gb300.dist import shard_systems


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


def test_gloo_two_ranks():
    off = np.concatenate([[0], np.cumsum(ic.batched_sizes(64))])
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, off, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, a0, b0, t0, n0), (r1, a1, b1, t1, n1) = res
    assert a0 == 0 and b0 == a1 and b1 == 64
    assert t0 == t1 == 2.0
    assert n0 == n1 == float(off[-1])
