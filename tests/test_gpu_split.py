"""The kernel side of one system split over several GPUs (nns_gb300/dist.py),
on one GPU: the walks of contiguous group ranges (nbx_forces_groups, a rank's
share: a key range of the sorted order) write exactly their groups' bodies, so
ranges that cover the groups, each walked on zeroed accelerations and summed,
give the full walk's forces bit for bit -- what the ranks' sum over NCCL
computes.  Argument and state errors are reported and leave the context usable.
(The ranks' host flow and the exchange are tested with gloo ranks on the CPU,
tests/test_dist.py.)"""
import numpy as np
import pytest
import torch

from nns_gb300 import ic
from nns_gb300.dist import split_groups

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("multipole", [0, 1], ids=["mono", "quad"])
def test_group_ranges_sum_to_the_full_walk(cuda, multipole):
    from nns_gb300.barnes_hut import Context, State
    b = ic.binary_disk(100003)
    n = len(b.x)
    ctx = Context(max_bodies=n, theta=0.5, eps=0.005, multipole=multipole)
    ctx.set_systems([0, n])
    s = State.from_bodies(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    full = s.acc()
    full_len, _ = ctx.group_stats()
    full_len = full_len.cpu().numpy()
    ng = ctx.group_count()
    assert ng == (n + 31) // 32
    for world in (2, 3, 7):
        bounds = split_groups(full_len + 1.0, world)
        total = np.zeros_like(full)
        for r in range(world):
            for t in (s.ax, s.ay, s.az):
                t.zero_()
            ctx.forces_groups(s, int(bounds[r]), int(bounds[r + 1] - bounds[r]))
            ctx.sync()
            part = s.acc()
            total += part
        assert np.array_equal(total, full)
        ln, _ = ctx.group_stats()
        assert np.array_equal(ln.cpu().numpy(), full_len)  # every group walked once, the same lists


def test_group_range_errors(cuda):
    from nns_gb300._lib import NbxError
    from nns_gb300.barnes_hut import Context, State
    b = ic.plummer(5000)
    n = len(b.x)
    ctx = Context(max_bodies=n, theta=0.5, eps=0.01)
    ctx.set_systems([0, n])
    s = State.from_bodies(b)
    with pytest.raises(NbxError) as e:
        ctx.forces_groups(s, 0, 10)
    assert e.value.code == 9  # NBX_ERR_STATE: no build yet
    ctx.build(s)
    ng = ctx.group_count()
    for first, count in ((-1, 1), (0, ng + 1), (ng, 1)):
        with pytest.raises(NbxError) as e:
            ctx.forces_groups(s, first, count)
        assert e.value.code == 1  # NBX_ERR_ARG
    ctx.forces_groups(s, ng, 0)  # an empty share is fine
    ctx.set_walk(8, 2)
    with pytest.raises(NbxError) as e:
        ctx.forces_groups(s, 0, ng)
    assert e.value.code == 1
    ctx.set_walk(8, 3)
    ctx.forces_groups(s, 0, ng)
    ctx.sync()
    assert np.isfinite(s.acc()).all() and torch.count_nonzero(s.ax).item() > 0
