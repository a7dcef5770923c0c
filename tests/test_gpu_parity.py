"""CUDA path (libnbx.so, through its C ABI) versus the oracle.

Bit-exact: bounding box, keys order, sort permutation, canonical topology
(child slots, cell start/count/level), FP64-summed centres of mass rounded to
FP32, per-group interaction-list lengths and the update.
Forces: the same interaction lists evaluated in FP32 (rsqrt and summation
order differ) -- tolerance 1e-5 median / 1e-4 max relative error.
Both sort digit widths (8 bits in 8 passes, 9 bits in 7) give the same trees,
and out-of-range launch settings are argument errors that leave the context
usable.
"""
import numpy as np
import pytest

from nns_gb300 import ic
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MED_TOL, MAX_TOL = 1e-5, 1e-4


def _ctx(n, nsys=1, **kw):
    from nns_gb300.barnes_hut import Context
    return Context(max_bodies=n, max_systems=nsys, **kw)


def _state(b):
    from nns_gb300.barnes_hut import State
    return State.from_bodies(b)


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-30)


def _check_tree(gt, ot):
    assert np.array_equal(gt["perm"], ot.perm)
    assert np.array_equal(gt["root_child"], ot.root_child)
    assert gt["ncells"] == ot.ncells
    assert np.array_equal(gt["cell_child"], ot.cell_child)
    assert np.array_equal(gt["cell_start"], ot.cell_start)
    assert np.array_equal(gt["cell_count"], ot.cell_count)
    assert np.array_equal(gt["cell_level"], ot.cell_level)
    for k in ("cell_x", "cell_y", "cell_z", "cell_m"):
        assert np.array_equal(gt[k], getattr(ot, k)), k


CASES = {
    "disk64": lambda: ic.star_disk(64),
    "disk1000": lambda: ic.star_disk(1000),
    "disk16384": lambda: ic.star_disk(16384),
    "plummer2048": lambda: ic.plummer(2048),
    "binary4099": lambda: ic.binary_disk(4099),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("mac", ["theta0.5", "reference"])
@pytest.mark.parametrize("variant", [0, 1, 2, 3], ids=["walk64", "walk128", "walk1", "walk96"])
def test_build_and_forces_match_oracle(cuda, name, mac, variant):
    b = CASES[name]()
    n = len(b.x)
    kw = dict(theta=0.5, eps=0.01) if mac == "theta0.5" else dict(theta_ref=1.5, eps2=0.0025)
    ctx = _ctx(n, **kw)
    ctx.set_walk(8, variant)
    theta_ref, eps2 = ctx.constants()
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    gt = ctx.export_tree(0)
    ot = O.build(b.x, b.y, b.z, b.m)
    _check_tree(gt, ot)
    keys, perm = ctx.export_keys()
    hi, _ = O.keys(b.x, b.y, b.z, ot.bbox, 21)
    assert np.array_equal(perm, ot.perm)
    assert np.array_equal(keys, hi[ot.perm])
    f = O.forces(b.x, b.y, b.z, b.m, ot, theta_ref, eps2)
    nl, no = ctx.walk_stats()
    assert np.array_equal(nl, f.nlist)
    assert np.array_equal(no, f.nopen)
    rel = _rel(s.acc(), f.a)
    assert np.median(rel) <= MED_TOL and rel.max() <= MAX_TOL, (np.median(rel), rel.max())
    info = ctx.tree_info()
    assert info["ncells"] == ot.ncells and info["status"] == 0
    assert info["interactions"] == int(f.nlist.astype(np.int64).sum())


def test_golden_reference_fixture(cuda):
    """The reference's own kernels (tests/golden) against the CUDA path directly."""
    import os
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "disk16384.npz")))
    b = ic.Bodies(g["in_x"], g["in_y"], g["in_z"], g["in_vx"], g["in_vy"], g["in_vz"], g["in_m"])
    n = len(b.x)
    ctx = _ctx(n, theta_ref=1.5, eps2=0.0025)
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    gt = ctx.export_tree(0)
    for k in ("perm", "root_child", "cell_child", "cell_start", "cell_count", "cell_level"):
        assert np.array_equal(gt[k], g[k]), k
    # the reference's cell moments are FP32 atomic sums; ours are FP64 sums
    rel = _rel(s.acc(), g["a"])
    assert np.median(rel) < 1e-4, np.median(rel)


def test_deep_refinement(cuda):
    b = ic.star_disk(1024, seed=ic.SEED0 + 77)
    x = b.x.copy()
    for i in (100, 300, 500, 700, 900):
        x[i + 1] = np.nextafter(np.nextafter(x[i], np.float32(2)), np.float32(2))
        b.y[i + 1] = b.y[i]
        b.z[i + 1] = b.z[i]
    b = ic.Bodies(x, b.y, b.z, b.vx, b.vy, b.vz, b.m)
    n = len(x)
    ctx = _ctx(n, theta=0.5, eps=0.01)
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    info = ctx.tree_info()
    assert info["refined_runs"] >= 1 and info["max_level"] > 22
    ot = O.build(b.x, b.y, b.z, b.m)
    _check_tree(ctx.export_tree(0), ot)
    t, e2 = ctx.constants()
    f = O.forces(b.x, b.y, b.z, b.m, ot, t, e2)
    rel = _rel(s.acc(), f.a)
    assert np.median(rel) <= MED_TOL and rel.max() <= MAX_TOL


@pytest.mark.parametrize("n", [1, 2, 3, 31, 33, 100])
def test_small_and_ragged(cuda, n):
    b = ic.plummer(n, seed=ic.SEED0 + n)
    ctx = _ctx(n, theta=0.5, eps=0.01)
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    ot = O.build(b.x, b.y, b.z, b.m)
    _check_tree(ctx.export_tree(0), ot)
    t, e2 = ctx.constants()
    f = O.forces(b.x, b.y, b.z, b.m, ot, t, e2)
    rel = _rel(s.acc(), f.a)
    if n > 1:
        assert rel.max() <= MAX_TOL


def test_split_planes(cuda):
    g = np.arange(-8, 9) / 8.0
    X, Y, Z = np.meshgrid(g, g, np.array([-0.25, 0.0, 0.25]), indexing="ij")
    n = X.size
    b = ic.Bodies(*(np.asarray(a, np.float32) for a in (X.ravel(), Y.ravel(), Z.ravel(), np.zeros(n),
                                                        np.zeros(n), np.zeros(n), np.full(n, 1.0 / n))))
    ctx = _ctx(n, theta=0.5, eps=0.01)
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    ot = O.build(b.x, b.y, b.z, b.m)
    _check_tree(ctx.export_tree(0), ot)


def test_update_bit_exact(cuda):
    b = ic.star_disk(5000)
    n = len(b.x)
    ctx = _ctx(n, theta=0.5, eps=0.01, dt=1e-3)
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    ctx.forces(s)
    a = s.acc()
    ctx.integrate(s)
    ctx.sync()
    ref = O.update(b.x, b.y, b.z, b.vx, b.vy, b.vz, a, 1e-3)
    for got, want in zip(s.host(), ref):
        assert np.array_equal(got, want)


def test_batched_equals_unbatched(cuda):
    sizes = [1024, 37, 1, 3000, 5, 2, 2048, 777]
    parts = [ic.star_disk(k, seed=ic.SEED0 + 1 + i) for i, k in enumerate(sizes)]
    off = np.concatenate([[0], np.cumsum(sizes)])
    cat = lambda k: np.concatenate([getattr(p, k) for p in parts])  # noqa: E731
    B = ic.Bodies(cat("x"), cat("y"), cat("z"), cat("vx"), cat("vy"), cat("vz"), cat("m"))
    ctx = _ctx(int(off[-1]), nsys=len(sizes), theta=0.5, eps=0.01)
    ctx.set_systems(off)
    s = _state(B)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    accb = s.acc()
    for i, p in enumerate(parts):
        n = len(p.x)
        c1 = _ctx(n, theta=0.5, eps=0.01)
        c1.set_systems([0, n])
        s1 = _state(p)
        c1.build(s1)
        c1.forces(s1)
        c1.sync()
        assert np.array_equal(accb[off[i]:off[i + 1]], s1.acc()), i
        t1 = c1.export_tree(0)
        tb = ctx.export_tree(i)
        for k in ("perm", "root_child", "cell_child", "cell_m", "cell_x"):
            assert np.array_equal(t1[k], tb[k]), (i, k)


@pytest.mark.parametrize("stack_depth", [384, 512])
def test_batched_equals_unbatched_with_a_deep_system(cuda, stack_depth):
    """A system whose tree reaches level 39 batched with shallow ones: every
    system's walk keeps the depth-first reserve of its own tree, so each system's
    forces equal its single-system run bit for bit (with the reserve of the
    deepest system of the batch, the shallow systems' rounds and hence their
    force sums would depend on their neighbours in the batch)."""
    from adversarial import CASES
    parts = [ic.star_disk(30000, seed=ic.SEED0 + 90), CASES["deep"](), ic.plummer(40000, seed=ic.SEED0 + 91),
             ic.binary_disk(20000, seed=ic.SEED0 + 92)]
    sizes = [len(p.x) for p in parts]
    off = np.concatenate([[0], np.cumsum(sizes)])
    cat = lambda k: np.concatenate([getattr(p, k) for p in parts])  # noqa: E731
    B = ic.Bodies(cat("x"), cat("y"), cat("z"), cat("vx"), cat("vy"), cat("vz"), cat("m"))
    ctx = _ctx(int(off[-1]), nsys=len(sizes), theta=0.5, eps=0.001, stack_depth=stack_depth)
    ctx.set_systems(off)
    s = _state(B)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    accb = s.acc()
    assert ctx.tree_info()["max_level"] > 30
    for i, p in enumerate(parts):
        n = len(p.x)
        c1 = _ctx(n, theta=0.5, eps=0.001, stack_depth=stack_depth)
        c1.set_systems([0, n])
        s1 = _state(p)
        c1.build(s1)
        c1.forces(s1)
        c1.sync()
        assert np.array_equal(accb[off[i]:off[i + 1]], s1.acc()), i


def test_radix_width_gives_the_same_trees(cuda):
    """9-bit digits (7 passes, the keys generated into the alternate buffers)
    against 8-bit digits (8 passes): single systems of odd and ragged sizes and a
    batch of uneven systems give the oracle's trees and bit-identical forces;
    switching the width on a live context (nbx_set_tuning) and replaying the
    step graph gives the same state as eager steps."""
    for n in (1, 33, 4099, 16384):
        b = ic.star_disk(n) if n > 1 else ic.plummer(1)
        acc = {}
        for bits in (8, 9):
            ctx = _ctx(n, theta=0.5, eps=0.01, radix_bits=bits)
            ctx.set_systems([0, n])
            s = _state(b)
            ctx.build(s)
            ctx.forces(s)
            ctx.sync()
            _check_tree(ctx.export_tree(0), O.build(b.x, b.y, b.z, b.m))
            acc[bits] = s.acc()
        assert np.array_equal(acc[8], acc[9]), n
    sizes = [1024, 37, 3000, 5, 2048, 777]
    parts = [ic.star_disk(k, seed=ic.SEED0 + 1 + i) for i, k in enumerate(sizes)]
    off = np.concatenate([[0], np.cumsum(sizes)])
    cat = lambda k: np.concatenate([getattr(p, k) for p in parts])  # noqa: E731
    B = ic.Bodies(cat("x"), cat("y"), cat("z"), cat("vx"), cat("vy"), cat("vz"), cat("m"))
    res = {}
    for bits in (8, 9):
        ctx = _ctx(int(off[-1]), nsys=len(sizes), theta=0.5, eps=0.01, radix_bits=bits)
        ctx.set_systems(off)
        s = _state(B)
        ctx.build(s)
        ctx.forces(s)
        ctx.sync()
        for i, p in enumerate(parts):
            _check_tree(ctx.export_tree(i), O.build(p.x, p.y, p.z, p.m))
        res[bits] = s.acc()
    assert np.array_equal(res[8], res[9])
    # live switch, graph replay against eager steps
    n = int(off[-1])
    ends = []
    for graphs in (False, True):
        ctx = _ctx(n, nsys=len(sizes), theta=0.5, eps=0.01, dt=1e-3)
        ctx.set_systems(off)
        s = _state(B)
        if graphs:
            ctx.graph_step(s, 2)
            ctx.set_tuning(9, 512)
            ctx.graph_step(s, 2)
        else:
            ctx.step(s)
            ctx.step(s)
            ctx.set_tuning(9, 512)
            ctx.step(s)
            ctx.step(s)
        ctx.sync()
        ends.append(s.host())
    for a, b2 in zip(*ends):
        assert np.array_equal(a, b2)


def test_batched_equals_unbatched_hilbert(cuda):
    """Hilbert keys (key_order 1): each system of a batch equals its own
    single-system run bit for bit (keys, tree and forces)."""
    from nns_gb300.barnes_hut import Context
    sizes = [3000, 41, 1, 5000, 2, 700]
    parts = [ic.plummer(k, seed=ic.SEED0 + 60 + i) for i, k in enumerate(sizes)]
    off = np.concatenate([[0], np.cumsum(sizes)])
    cat = lambda k: np.concatenate([getattr(p, k) for p in parts])  # noqa: E731
    B = ic.Bodies(cat("x"), cat("y"), cat("z"), cat("vx"), cat("vy"), cat("vz"), cat("m"))
    ctx = Context(max_bodies=int(off[-1]), max_systems=len(sizes), theta=0.5, eps=0.01, key_order=1)
    ctx.set_systems(off)
    s = _state(B)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    accb = s.acc()
    keys_b, _ = ctx.export_keys()
    for i, p in enumerate(parts):
        n = len(p.x)
        c1 = Context(max_bodies=n, theta=0.5, eps=0.01, key_order=1)
        c1.set_systems([0, n])
        s1 = _state(p)
        c1.build(s1)
        c1.forces(s1)
        c1.sync()
        assert np.array_equal(accb[off[i]:off[i + 1]], s1.acc()), i
        k1, _ = c1.export_keys()
        assert np.array_equal(keys_b[off[i]:off[i + 1]], k1), i


@pytest.mark.parametrize("n", [4096, 262144])
def test_graph_step_equals_eager(cuda, n):
    """Five steps launched kernel by kernel, five replays of the captured step
    (graph_step), and one five-step call (which replays the graph) agree bit
    for bit; so does a second graph_step call that reuses the captured graph.
    At 262144 bodies the eager builds sort in one-sweep passes and the captured
    ones with histogram + scan + scatter passes: the same permutation."""
    import torch
    b = ic.star_disk(n)
    n = len(b.x)
    outs = []
    for how in ("eager", "graph", "steps"):
        ctx = _ctx(n, theta=0.5, eps=0.01, dt=1e-3)
        ctx.set_systems([0, n])
        s = _state(b)
        if how == "eager":
            for _ in range(5):
                ctx.step(s, 1)
        elif how == "graph":
            ctx.graph_step(s, 2)
            ctx.graph_step(s, 3, stream=torch.cuda.Stream())
        else:
            ctx.step(s, 5)
        ctx.sync()
        torch.cuda.synchronize()
        outs.append(s.host())
    for other in outs[1:]:
        for a, c in zip(outs[0], other):
            assert np.array_equal(a, c)


def test_trajectory_matches_oracle(cuda):
    b = ic.star_disk(2048)
    n = len(b.x)
    ctx = _ctx(n, theta=0.5, eps=0.01, dt=1e-3)
    ctx.set_systems([0, n])
    s = _state(b)
    x, y, z, vx, vy, vz = b.x, b.y, b.z, b.vx, b.vy, b.vz
    t, e2 = ctx.constants()
    for _ in range(10):
        ctx.step(s, 1)
        ot = O.build(x, y, z, b.m)
        f = O.forces(x, y, z, b.m, ot, t, e2)
        x, y, z, vx, vy, vz = O.update(x, y, z, vx, vy, vz, f.a, 1e-3)
    ctx.sync()
    gx = s.host()
    err = np.abs(np.stack(gx[:3], 1) - np.stack([x, y, z], 1)).max()
    assert err < 1e-5, err


@pytest.mark.parametrize("mode", [1, 2])
def test_compensated_close_to_plain(cuda, mode):
    b = ic.star_disk(8192)
    n = len(b.x)
    res = []
    for comp in (0, mode):
        ctx = _ctx(n, theta=0.5, eps=0.01, compensated=comp)
        ctx.set_systems([0, n])
        s = _state(b)
        ctx.build(s)
        ctx.forces(s)
        ctx.sync()
        res.append(s.acc())
    ot = O.build(b.x, b.y, b.z, b.m)
    f = O.forces(b.x, b.y, b.z, b.m, ot, 0.25, 1e-4)
    e_plain = _rel(res[0], f.a64)
    e_comp = _rel(res[1], f.a64)
    assert np.median(e_comp) <= np.median(e_plain) * 1.01
    assert e_comp.max() <= MAX_TOL


@pytest.mark.parametrize("warps", [4, 8, 16])
@pytest.mark.parametrize("variant", [0, 1, 3])
def test_walk_launch_shapes_agree(cuda, warps, variant):
    b = ic.plummer(5000)
    n = len(b.x)
    out = []
    for w in (8, warps):
        ctx = _ctx(n, theta=0.6, eps=0.005)
        ctx.set_walk(w, variant)
        ctx.set_systems([0, n])
        s = _state(b)
        ctx.build(s)
        ctx.forces(s)
        ctx.sync()
        out.append(s.acc())
    assert np.array_equal(out[0], out[1])


def test_potential_energy(cuda):
    b = ic.plummer(4096)
    n = len(b.x)
    ctx = _ctx(n, theta=0.5, eps=0.01)
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    phi = ctx.potential(s)
    ctx.sync()
    want = O.direct_potential_fp64(b.x, b.y, b.z, b.m, 1e-4, np.arange(n))
    rel = np.abs(phi - want) / np.abs(want)
    assert np.median(rel) < 1e-3 and rel.max() < 2e-2
    # Plummer sphere: W = -3 pi / 32 (G = M = a = 1), softened slightly
    W = 0.5 * float((b.m.astype(np.float64) * phi).sum())
    assert abs(W + 3 * np.pi / 32) < 0.02


def test_direct_fp64_matches_oracle(cuda):
    b = ic.plummer(3000)
    ctx = _ctx(len(b.x))
    ctx.set_systems([0, len(b.x)])
    s = _state(b)
    tg = np.arange(0, 3000, 7)
    got = ctx.direct_fp64(s, tg, 1e-4).cpu().numpy()
    want = O.direct_fp64(b.x, b.y, b.z, b.m, 1e-4, tg)
    assert np.allclose(got, want, rtol=1e-12, atol=1e-14)


def test_errors_are_reported(cuda):
    from nns_gb300._lib import NbxError
    b = ic.star_disk(300)
    x = b.x.copy()
    x[10] = x[11]
    b.y[10] = b.y[11]
    b.z[10] = b.z[11]
    b2 = ic.Bodies(x, b.y, b.z, b.vx, b.vy, b.vz, b.m)
    ctx = _ctx(300)
    ctx.set_systems([0, 300])
    s = _state(b2)
    ctx.build(s)
    ctx.forces(s)
    with pytest.raises(NbxError) as e:
        ctx.sync()
    assert e.value.code == 3  # NBX_ERR_DEPTH
    # NaN position
    x = b.x.copy()
    x[5] = np.nan
    s = _state(ic.Bodies(x, b.y, b.z, b.vx, b.vy, b.vz, b.m))
    ctx.build(s)
    ctx.forces(s)
    with pytest.raises(NbxError) as e:
        ctx.sync()
    assert e.value.code == 6  # NBX_ERR_NONFINITE
    # the context stays usable
    s = _state(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()


def test_stack_beyond_shared_memory_is_an_argument_error(cuda):
    """4096 stack entries per warp with 16-warp blocks need about 326 KB of shared
    memory per block (more than the device gives): the walk is not launched and
    the call reports NBX_ERR_ARG; with 4-warp blocks (83 KB) the same context
    walks and matches the oracle's lists."""
    from nns_gb300._lib import NbxError
    b = ic.star_disk(4096)
    n = len(b.x)
    ctx = _ctx(n, theta=0.5, eps=0.01, stack_depth=4096)
    ctx.set_walk(16, 3)
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    with pytest.raises(NbxError) as e:
        ctx.forces(s)
    assert e.value.code == 1  # NBX_ERR_ARG
    ctx.set_walk(4, 3)
    ctx.forces(s)
    ctx.sync()
    ot = O.build(b.x, b.y, b.z, b.m)
    t, e2 = ctx.constants()
    f = O.forces(b.x, b.y, b.z, b.m, ot, t, e2)
    nl, _ = ctx.walk_stats()
    assert np.array_equal(nl, f.nlist)


def test_kernels_wrapper_sequence(cuda):
    """The reference's BarnesHut::update sequence through the phase entry points."""
    from nns_gb300.barnes_hut import BarnesHut
    b = ic.star_disk(3000)
    n = len(b.x)
    bh = BarnesHut(b, theta_ref=1.5, eps2=0.0025, timestep=1e-3)
    bh.update(0)
    child = bh.d_child.cpu().numpy()
    ot = O.build(b.x, b.y, b.z, b.m)
    assert np.array_equal(child[:8], ot.root_child)
    assert np.array_equal(child[8 * n:8 * (n + ot.ncells)].reshape(-1, 8), ot.cell_child)
    assert int(bh.d_index.item()) == n + ot.ncells
    assert np.array_equal(bh.d_sorted[:n].cpu().numpy(), ot.perm)
    assert np.array_equal(bh.d_start[n:n + ot.ncells].cpu().numpy(), ot.cell_start)
    assert np.array_equal(bh.d_count[n:n + ot.ncells].cpu().numpy(), ot.cell_count)
    assert np.array_equal(bh.d_x[n:n + ot.ncells].cpu().numpy(), ot.cell_x)
    assert np.array_equal(bh.d_mass[n:n + ot.ncells].cpu().numpy(), ot.cell_m)
    f = O.forces(b.x, b.y, b.z, b.m, ot, 1.5, 0.0025)
    acc = np.stack([bh.d_ax[:n].cpu().numpy(), bh.d_ay[:n].cpu().numpy(), bh.d_az[:n].cpu().numpy()], 1)
    rel = _rel(acc, f.a)
    assert rel.max() <= MAX_TOL
    st = O.update(b.x, b.y, b.z, b.vx, b.vy, b.vz, acc, 1e-3)
    assert np.array_equal(bh.h_x, st[0]) and np.array_equal(bh.h_vz, st[5])
    assert set(bh.times) >= {"buildTree", "computeForces"}


def test_plummer_2p20_properties(cuda):
    """The 2^20-body Plummer workload (theta 0.6, eps 0.005): exact keys, permutation
    and tree, forces and list lengths on sampled groups, and the error against an
    FP64 direct sum on 4096 targets."""
    b = ic.plummer(1 << 20)
    n = len(b.x)
    ctx = _ctx(n, theta=0.6, eps=0.005)
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    ot = O.build(b.x, b.y, b.z, b.m)
    _check_tree(ctx.export_tree(0), ot)
    t, e2 = ctx.constants()
    groups = np.random.default_rng(1).choice(n // 32, 128, replace=False)
    f = O.forces(b.x, b.y, b.z, b.m, ot, t, e2, groups=groups)
    idx = np.concatenate([ot.perm[g * 32:(g + 1) * 32] for g in groups])
    rel = _rel(s.acc()[idx], f.a[idx])
    assert np.median(rel) <= MED_TOL and rel.max() <= MAX_TOL
    nl, _ = ctx.walk_stats()
    assert np.array_equal(nl[idx], f.nlist[idx])
    keys, perm = ctx.export_keys()
    hi, _ = O.keys(b.x, b.y, b.z, ot.bbox, 21)
    assert np.array_equal(perm, ot.perm) and np.array_equal(keys, hi[ot.perm])
    # the Barnes-Hut error itself, against an FP64 direct sum on 4096 uniform targets
    targets = np.random.default_rng(2).choice(n, 4096, replace=False).astype(np.int32)
    direct = O.direct_fp64(b.x, b.y, b.z, b.m, e2, targets)
    err = _rel(s.acc()[targets], direct)
    assert np.median(err) < 5e-3 and np.percentile(err, 99) < 5e-2, (np.median(err), np.percentile(err, 99))


@pytest.mark.parametrize("mode", [1, 2], ids=["per_level", "one_launch"])
def test_moments_modes_match_oracle(cuda, mode):
    """Both centre-of-mass passes (one launch per level; one launch where the
    last child sums its parent) give the oracle's FP64 sums bit for bit, on a
    batch of uneven systems."""
    from nns_gb300.barnes_hut import Context
    sizes = [5000, 70000, 1, 2, 33000]
    parts = [ic.plummer(k, seed=ic.SEED0 + 40 + j) for j, k in enumerate(sizes)]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    b = ic.Bodies(*(np.concatenate([getattr(q, f) for q in parts]) for f in ("x", "y", "z", "vx", "vy", "vz", "m")))
    ctx = Context(max_bodies=int(off[-1]), max_systems=len(sizes), theta=0.5, eps=0.01, moments_mode=mode)
    ctx.set_systems(off)
    s = _state(b)
    ctx.build(s)
    ctx.sync()
    for j, q in enumerate(parts):
        _check_tree(ctx.export_tree(j), O.build(q.x, q.y, q.z, q.m))


@pytest.mark.parametrize("radix_bits", [8, 9])
def test_sort_with_full_size_tiles(cuda, radix_bits):
    """2^22 bodies: the radix sort runs with 2048-key tiles (smaller systems use
    256..1024) for the bodies and the node entries, with 8-bit digits (8 passes)
    or 9-bit digits (7 passes).  The permutation equals the oracle's 42-level
    key order and the tree's moments sum to the total mass."""
    n = 1 << 22
    b = ic.binary_disk(n, seed=ic.SEED0 + 51)
    ctx = _ctx(n, theta=0.5, eps=0.005, radix_bits=radix_bits)
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    ctx.sync()
    keys, perm = ctx.export_keys()
    bb = O.bbox(b.x, b.y, b.z)
    hi, lo = O.keys(b.x, b.y, b.z, bb, 42)
    assert np.array_equal(perm, np.lexsort((lo, hi)))
    assert np.array_equal(keys, hi[perm])
    gt = ctx.export_tree(0)
    roots = gt["root_child"][gt["root_child"] >= n] - n
    total = gt["cell_m"][roots].astype(np.float64).sum() + b.m[gt["root_child"][(gt["root_child"] >= 0) & (gt["root_child"] < n)]].sum()
    assert abs(total - b.m.astype(np.float64).sum()) < 1e-5


def test_autotune_picks_a_valid_config(cuda, tmp_path, monkeypatch):
    from nns_gb300 import autotune
    monkeypatch.setenv("NBX_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    b = ic.star_disk(20000)
    n = len(b.x)
    ctx = _ctx(n, theta=0.5, eps=0.01)
    ctx.set_systems([0, n])
    s = _state(b)
    r = autotune.tune_walk(ctx, s, reps=1)
    assert (r["warps"], r["variant"]) in autotune.CANDIDATES and not r["cached"]
    assert r["stack_depth"] in autotune.STACK_DEPTHS and r["radix_bits"] in autotune.RADIX_BITS
    assert ctx.params.stack_depth == r["stack_depth"] and ctx.params.radix_bits == r["radix_bits"]
    r2 = autotune.tune_walk(ctx, s, reps=1)
    assert r2["cached"] and r2["warps"] == r["warps"] and r2["radix_bits"] == r["radix_bits"]
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    ot = O.build(b.x, b.y, b.z, b.m)
    f = O.forces(b.x, b.y, b.z, b.m, ot, 0.25, 1e-4)
    assert _rel(s.acc(), f.a).max() <= MAX_TOL


def test_fp64_list_evaluation_matches_oracle(cuda):
    """FP64 re-evaluation of the walk's own lists equals the oracle's FP64
    evaluation of the same lists; the FP32 walk is within 1e-5 median / 1e-4
    max of it (observed ~8e-7 / 1.2e-5)."""
    b = ic.binary_disk(8192)
    n = len(b.x)
    ctx = _ctx(n, theta=0.5, eps=0.005)
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    tg = np.arange(0, n, 13)
    a64 = ctx.forces_fp64_lists(tg)
    ot = O.build(b.x, b.y, b.z, b.m)
    t, e2 = ctx.constants()
    f = O.forces(b.x, b.y, b.z, b.m, ot, t, e2)
    assert np.allclose(a64, f.a64[tg], rtol=1e-10, atol=1e-14 * np.abs(f.a64).max())
    rel = _rel(s.acc()[tg], a64)
    assert np.median(rel) <= MED_TOL and rel.max() <= MAX_TOL


def test_hilbert_keys_match_reference_fixture(cuda):
    """key_order = 1 on the fixture's disk: every body's Hilbert key equals the
    reference's own Lebesgue2Hilbert of its Lebesgue key (tests/golden/
    sfc_hilbert4096.npz, made from SpaceFillingCurves/src/Tree.cpp:90-104)."""
    import os
    from nns_gb300.barnes_hut import Context
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "sfc_hilbert4096.npz")))
    n = int(g["n_disk"])
    b = ic.star_disk(n)
    ctx = Context(max_bodies=n, theta=0.5, eps=0.01, key_order=1)
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    ctx.sync()
    keys, perm = ctx.export_keys()
    assert np.array_equal(keys, g["hilbert"][:n][perm])
    assert np.array_equal(perm, np.argsort(g["hilbert"][:n], kind="stable"))


def test_hilbert_order_option(cuda):
    from nns_gb300.barnes_hut import Context
    b = ic.star_disk(20000)
    n = len(b.x)
    outs = {}
    for order in (0, 1):
        ctx = Context(max_bodies=n, theta=0.5, eps=0.01, key_order=order)
        ctx.set_systems([0, n])
        s = _state(b)
        ctx.build(s)
        ctx.forces(s)
        ctx.sync()
        keys, perm = ctx.export_keys()
        outs[order] = (keys, perm, s.acc(), ctx.tree_info())
    bb = O.bbox(b.x, b.y, b.z)
    hi, _ = O.keys(b.x, b.y, b.z, bb, 21)
    hk = O.hilbert(O.md_key(hi))  # the reference's conversion (pinned on the CPU)
    keys, perm, acc_h, info_h = outs[1]
    assert np.array_equal(keys, hk[perm])
    assert np.all(np.diff(keys.astype(np.float64)) >= 0)
    # same cells, different sibling order and walk groups; forces agree to the
    # tree-approximation level and the compact groups interact less
    _, _, acc_m, info_m = outs[0]
    assert info_h["ncells"] == info_m["ncells"]
    assert info_h["interactions"] < info_m["interactions"]
    assert np.median(_rel(acc_h, acc_m)) < 1e-3


@pytest.mark.parametrize("variant", [3, 2], ids=["walk96", "walk1"])
@pytest.mark.parametrize("name", ["collinear", "coplanar", "signed_zeros", "cluster", "deep"])
def test_adversarial_geometry(cuda, name, variant):
    """Degenerate boxes, signed zeros, bodies on split planes, a tight cluster
    and MAC decisions on cells past level 32 (the oracle is pinned to the
    reference kernels on the same sets).
    Tree, keys and every MAC decision are bit-exact; forces within tolerance."""
    from adversarial import CASES, EPS
    b = CASES[name]()
    n = len(b.x)
    ctx = _ctx(n, theta=0.5, eps=EPS.get(name, 0.01))
    ctx.set_walk(8, variant)
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    ot = O.build(b.x, b.y, b.z, b.m)
    _check_tree(ctx.export_tree(0), ot)
    keys, perm = ctx.export_keys()
    assert np.array_equal(perm, ot.perm)
    t, e2 = ctx.constants()
    f = O.forces(b.x, b.y, b.z, b.m, ot, t, e2)
    nl, no = ctx.walk_stats()
    assert np.array_equal(nl, f.nlist) and np.array_equal(no, f.nopen)
    a = s.acc().astype(np.float64)
    rel = _rel(a, f.a)
    assert np.median(rel) <= MED_TOL, np.median(rel)
    # on a line or in a plane the pulls on a body nearly cancel, so its relative
    # error is set by the summation order: each body's error is bounded relative
    # to its own force plus a floor of the set's typical force magnitude
    err = np.linalg.norm(a - f.a, axis=1)
    mag = np.linalg.norm(f.a.astype(np.float64), axis=1)
    assert (err <= MAX_TOL * (mag + np.median(mag))).all(), (err / (mag + np.median(mag))).max()


@pytest.mark.parametrize("name", ["disk20000", "plummer8192", "binary4099"])
@pytest.mark.parametrize("multipole", [0, 1], ids=["monopole", "quadrupole"])
def test_hilbert_walk_lists_match_oracle(cuda, name, multipole):
    """key_order = 1: the same cells as the Morton tree with siblings reordered,
    and walk groups of 32 consecutive bodies in Hilbert order.  A group's list is
    decided by the MAC of each (group, cell) pair alone, so the oracle's walk
    over its Morton tree with the groups taken from the Hilbert permutation gives
    the same per-body list lengths and opened-cell counts bit for bit, and
    forces within 1e-5 median / 1e-4 max (FP32 monopoles against the oracle's
    FP32 walk; quadrupoles against its FP64 evaluation with FP64 quadrupoles)."""
    import dataclasses
    from nns_gb300.barnes_hut import Context
    b = {"disk20000": lambda: ic.star_disk(20000), "plummer8192": lambda: ic.plummer(8192),
         "binary4099": lambda: ic.binary_disk(4099)}[name]()
    n = len(b.x)
    ctx = Context(max_bodies=n, theta=0.5, eps=0.01, key_order=1, multipole=multipole)
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    _, perm_h = ctx.export_keys()
    ot = O.build(b.x, b.y, b.z, b.m)
    assert ctx.tree_info()["ncells"] == ot.ncells
    oh = dataclasses.replace(ot, perm=np.ascontiguousarray(perm_h, np.int32))
    t, e2 = ctx.constants()
    q = O.quadrupoles(b.x, b.y, b.z, b.m, ot) if multipole else None
    f = O.forces(b.x, b.y, b.z, b.m, oh, t, e2, quad=q)
    nl, no = ctx.walk_stats()
    assert np.array_equal(nl, f.nlist) and np.array_equal(no, f.nopen)
    rel = _rel(s.acc(), f.a64 if multipole else f.a)
    assert np.median(rel) <= 1e-5 and rel.max() <= 1e-4, (np.median(rel), rel.max())


@pytest.mark.parametrize("name", ["collinear", "coplanar", "signed_zeros", "cluster", "deep"])
def test_hilbert_adversarial_geometry(cuda, name):
    """Hilbert order on the adversarial sets (degenerate boxes, signed zeros,
    split planes, a tight cluster, keys refined past level 21): the same cells as
    the Morton tree, bodies in non-decreasing 21-level Hilbert key order (the
    reference's Lebesgue2Hilbert), and lists bit-exact against the oracle's walk
    with the Hilbert groups."""
    import dataclasses
    from adversarial import CASES, EPS
    from nns_gb300.barnes_hut import Context
    b = CASES[name]()
    n = len(b.x)
    ctx = Context(max_bodies=n, theta=0.5, eps=EPS.get(name, 0.01), key_order=1)
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    assert ctx.tree_info()["status"] == 0
    _, perm_h = ctx.export_keys()
    assert np.array_equal(np.sort(perm_h), np.arange(n))
    ot = O.build(b.x, b.y, b.z, b.m)
    assert ctx.tree_info()["ncells"] == ot.ncells
    hi, _ = O.keys(b.x, b.y, b.z, ot.bbox, 21)
    hk = O.hilbert(O.md_key(hi))
    assert np.all(np.diff(hk[perm_h].astype(np.float64)) >= 0)
    t, e2 = ctx.constants()
    f = O.forces(b.x, b.y, b.z, b.m, dataclasses.replace(ot, perm=np.ascontiguousarray(perm_h, np.int32)), t, e2)
    nl, no = ctx.walk_stats()
    assert np.array_equal(nl, f.nlist) and np.array_equal(no, f.nopen)
    a = s.acc().astype(np.float64)
    err = np.linalg.norm(a - f.a, axis=1)
    mag = np.linalg.norm(f.a.astype(np.float64), axis=1)
    assert (err <= MAX_TOL * (mag + np.median(mag))).all(), (err / (mag + np.median(mag))).max()


@pytest.mark.parametrize("mode", [1, 2], ids=["split", "kahan"])
@pytest.mark.parametrize("name", ["collinear", "coplanar", "signed_zeros", "cluster", "deep"])
def test_compensated_adversarial_geometry(cuda, name, mode):
    """The compensated forms on the adversarial sets: the same lists as the
    plain walk and the oracle, and each body's error against the oracle's FP64
    evaluation of those lists bounded relative to its own force plus the set's
    median force, no looser than the plain walk's bound."""
    from adversarial import CASES, EPS
    b = CASES[name]()
    n = len(b.x)
    ctx = _ctx(n, theta=0.5, eps=EPS.get(name, 0.01))
    t, e2 = ctx.constants()
    ctx.set_constants(t, e2, mode)
    ctx.set_systems([0, n])
    s = _state(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    ot = O.build(b.x, b.y, b.z, b.m)
    f = O.forces(b.x, b.y, b.z, b.m, ot, t, e2)
    nl, no = ctx.walk_stats()
    assert np.array_equal(nl, f.nlist) and np.array_equal(no, f.nopen)
    a = s.acc().astype(np.float64)
    err = np.linalg.norm(a - f.a64, axis=1)
    mag = np.linalg.norm(f.a64, axis=1)
    assert np.median(_rel(a, f.a64)) <= MED_TOL
    assert (err <= MAX_TOL * (mag + np.median(mag))).all(), (err / (mag + np.median(mag))).max()


def test_sort_wait_runs_out_and_reports(cuda):
    """The bounded wait of the small-context sort (one-sweep passes): the
    self-test runs one pass whose tile waits for an earlier tile that never
    runs.  The wait gives up within a few seconds, NBX_ERR_TIMEOUT is reported
    once and cleared, and the same context then builds and walks a system
    bit-exactly against the oracle."""
    import time
    from nns_gb300._lib import lib
    b = ic.star_disk(4096)
    n = len(b.x)
    ctx = _ctx(n, theta=0.5, eps=0.01)
    ctx.set_systems([0, n])
    t0 = time.time()
    assert lib().nbx_selftest_sort_wait(ctx.h, None) == 0
    assert time.time() - t0 < 30
    assert lib().nbx_sync_status(ctx.h, None) == 8  # NBX_ERR_TIMEOUT
    assert lib().nbx_sync_status(ctx.h, None) == 0
    s = _state(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    ot = O.build(b.x, b.y, b.z, b.m)
    _check_tree(ctx.export_tree(0), ot)
    t, e2 = ctx.constants()
    f = O.forces(b.x, b.y, b.z, b.m, ot, t, e2)
    nl, _ = ctx.walk_stats()
    assert np.array_equal(nl, f.nlist)
