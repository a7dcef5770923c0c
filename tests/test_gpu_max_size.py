"""The largest context: 2^26 bodies (nbx_params.max_bodies' limit), about 10^8
nodes, so node indices need more than 26 bits.  One full step runs
without a device error; the forces equal an FP64 evaluation of the same
interaction lists within the walk tolerance and the Barnes-Hut error against
an FP64 direct sum is the usual one."""
import numpy as np
import pytest

from nns_gb300 import ic

pytestmark = pytest.mark.gpu


def test_max_size_step(cuda):
    from nns_gb300.barnes_hut import Context, State
    n = 1 << 26
    # the benchmark's system (2^24 disk bodies of 1e-8): the same total disk mass
    b = ic.binary_disk(n, disk_mass=1e-8 * (1 << 24) / n)
    ctx = Context(max_bodies=n, theta=0.5, eps=0.005, dt=5e-4)
    ctx.set_systems([0, n])
    s = State.from_bodies(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    info = ctx.tree_info()
    assert info["status"] == 0 and info["nbodies"] == n
    assert n // 4 < info["ncells"] < n and info["nnodes"] == n + info["ncells"]
    targets = np.random.default_rng(5).choice(n, 512, replace=False).astype(np.int32)
    a = s.acc()[targets].astype(np.float64)
    assert np.isfinite(a).all()
    lists64 = ctx.forces_fp64_lists(targets)
    rel = np.linalg.norm(a - lists64, axis=1) / np.linalg.norm(lists64, axis=1)
    assert np.median(rel) < 1e-5 and rel.max() < 1e-4, (np.median(rel), rel.max())
    t, e2 = ctx.constants()
    direct = ctx.direct_fp64(s, targets, e2).cpu().numpy()
    err = np.linalg.norm(a - direct, axis=1) / np.linalg.norm(direct, axis=1)
    assert np.median(err) < 5e-3, np.median(err)
    ctx.integrate(s)
    ctx.sync()
    assert np.isfinite(s.x[:1000].cpu().numpy()).all()
