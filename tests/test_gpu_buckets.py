"""Leaf buckets (nbx_params.leaf_size k = 2..8; outside the parity mode: the
reference's tree has one body per leaf, Kernels.cu:284-362) against the
oracle's tree pruned the same way (oracle.bucket_tree): every cell holding at
most k bodies whose parent holds more becomes a leaf with its bodies as
children.  The interaction lists (list length and opened count per body) must
equal the oracle's walk over the pruned tree bit for bit, and the forces its
forces within 1e-5 median / 1e-4 max relative error; the cell count is the
pruned tree's.  Batched equals unbatched bit for bit, leaf_size 1 is the
reference's tree, and the reference's array export refuses bucket trees."""
import numpy as np
import pytest

from nns_gb300 import ic
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MED_TOL, MAX_TOL = 1e-5, 1e-4


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-30)


CASES = {
    "plummer8192": lambda: ic.plummer(8192),
    "disk16384": lambda: ic.star_disk(16384),
    "binary4099": lambda: ic.binary_disk(4099),
    "disk33": lambda: ic.star_disk(33),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("k", [2, 4, 8])
@pytest.mark.parametrize("multipole", [0, 1], ids=["mono", "quad"])
def test_bucket_walk_matches_oracle(cuda, name, k, multipole):
    from nns_gb300.barnes_hut import Context, State
    b = CASES[name]()
    n = len(b.x)
    ctx = Context(max_bodies=n, theta=0.5, eps=0.01, leaf_size=k, multipole=multipole)
    ctx.set_systems([0, n])
    s = State.from_bodies(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    t, e2 = ctx.constants()
    ot = O.build(b.x, b.y, b.z, b.m)
    bt = O.bucket_tree(ot, k)
    q = O.quadrupoles(b.x, b.y, b.z, b.m, ot) if multipole else None
    f = O.forces(b.x, b.y, b.z, b.m, bt, t, e2, quad=q)
    nl, no = ctx.walk_stats()
    assert np.array_equal(nl, f.nlist) and np.array_equal(no, f.nopen)
    rel = _rel(s.acc(), f.a64)
    assert np.median(rel) <= MED_TOL and rel.max() <= MAX_TOL, (np.median(rel), rel.max())
    assert ctx.tree_info()["ncells"] == O.reachable_cells(bt)


def test_buckets_shorten_the_walk_and_keep_the_error(cuda):
    """Binary star + disk at 2^18: with buckets the tree has fewer cells, the walk
    opens fewer of them, and the error against the FP64 direct sum stays at the
    one-body-per-leaf level or below (bodies of an opened bucket are exact)."""
    from nns_gb300.barnes_hut import Context, State
    b = ic.binary_disk(1 << 18)
    n = len(b.x)
    tg = np.random.default_rng(4).choice(n, 2048, replace=False)
    d = O.direct_fp64(b.x, b.y, b.z, b.m, float(np.float32(0.005) ** 2), tg)
    res = {}
    for k in (1, 4, 8):
        ctx = Context(max_bodies=n, theta=0.5, eps=0.005, leaf_size=k)
        ctx.set_systems([0, n])
        s = State.from_bodies(b)
        ctx.build(s)
        ctx.forces(s)
        ctx.sync()
        info = ctx.tree_info()
        res[k] = (np.median(_rel(s.acc()[tg], d)), info["ncells"], info["opened"])
    for k in (4, 8):
        assert res[k][1] < res[1][1] and res[k][2] < res[1][2], res
        assert res[k][0] <= res[1][0] * 1.05, res


def test_bucket_batched_and_switching(cuda):
    from nns_gb300._lib import NbxError
    from nns_gb300.barnes_hut import Context, State
    sizes = [3000, 9000, 2, 7]
    parts = [ic.plummer(k, seed=ic.SEED0 + 70 + j) for j, k in enumerate(sizes)]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    b = ic.Bodies(*(np.concatenate([getattr(q, f) for q in parts]) for f in ("x", "y", "z", "vx", "vy", "vz", "m")))
    ctx = Context(max_bodies=int(off[-1]), max_systems=len(sizes), theta=0.5, eps=0.01)
    ctx.set_systems(off)
    ctx.set_leaf_size(4)
    s = State.from_bodies(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    acc = s.acc()
    with pytest.raises(NbxError) as e:
        ctx.export_tree(0)
    assert e.value.code == 9  # NBX_ERR_STATE: the reference's format holds one body per leaf
    for j, q in enumerate(parts):
        c1 = Context(max_bodies=len(q.x), theta=0.5, eps=0.01, leaf_size=4)
        c1.set_systems([0, len(q.x)])
        s1 = State.from_bodies(q)
        c1.build(s1)
        c1.forces(s1)
        c1.sync()
        assert np.array_equal(acc[off[j]:off[j + 1]], s1.acc()), j
    # back to one body per leaf: the reference's tree again
    ctx.set_leaf_size(1)
    with pytest.raises(NbxError):
        ctx.forces(s)
    ctx.build(s)
    ctx.sync()
    ot = O.build(parts[0].x, parts[0].y, parts[0].z, parts[0].m)
    assert np.array_equal(ctx.export_tree(0)["cell_child"], ot.cell_child)


@pytest.mark.parametrize("name", ["collinear", "coplanar", "signed_zeros", "cluster", "deep"])
@pytest.mark.parametrize("k", [2, 8])
def test_bucket_adversarial_geometry(cuda, name, k):
    """Leaf buckets on the adversarial sets (degenerate boxes, signed zeros,
    split planes, a tight cluster, runs of keys refined past level 21, where the
    window test reads deltas up to 41): lists bit-exact against the oracle's
    pruned tree; each body's error bounded relative to its own force plus the
    set's median force (pulls that nearly cancel on a line or in a plane)."""
    from adversarial import CASES as ADV, EPS
    from nns_gb300.barnes_hut import Context, State
    b = ADV[name]()
    n = len(b.x)
    ctx = Context(max_bodies=n, theta=0.5, eps=EPS.get(name, 0.01), leaf_size=k)
    ctx.set_systems([0, n])
    s = State.from_bodies(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    assert ctx.tree_info()["status"] == 0
    t, e2 = ctx.constants()
    ot = O.build(b.x, b.y, b.z, b.m)
    bt = O.bucket_tree(ot, k)
    f = O.forces(b.x, b.y, b.z, b.m, bt, t, e2)
    nl, no = ctx.walk_stats()
    assert np.array_equal(nl, f.nlist) and np.array_equal(no, f.nopen)
    assert ctx.tree_info()["ncells"] == O.reachable_cells(bt)
    a = s.acc().astype(np.float64)
    err = np.linalg.norm(a - f.a, axis=1)
    mag = np.linalg.norm(f.a.astype(np.float64), axis=1)
    assert np.median(_rel(a, f.a)) <= MED_TOL
    assert (err <= MAX_TOL * (mag + np.median(mag))).all(), (err / (mag + np.median(mag))).max()
