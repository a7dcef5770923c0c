"""The quadrupole mode (nbx_params.multipole = 1, an extension: the reference's
kernels carry monopoles only) against the oracle.

The MAC does not change, so the interaction lists (per-body list length and
opened-cell count) must equal the oracle's monopole walk bit for bit; every
accepted cell adds its traceless quadrupole term, and the forces must equal
the oracle's FP64 evaluation of the same lists with FP64 quadrupoles
(orc_quad) within 1e-5 median / 1e-4 max relative error -- the FP32
arithmetic and FP32 storage of Q -- for every buffer variant and accumulation
mode.  Also: batched equals unbatched bit for bit, graph replay equals eager
steps, switching the order needs a new build, and the adjoint refuses it.
"""
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


def _run(b, variant=3, comp=0, theta=0.5, eps=0.01, warps=8):
    from nns_gb300.barnes_hut import Context, State
    n = len(b.x)
    ctx = Context(max_bodies=n, theta=theta, eps=eps, multipole=1, compensated=comp)
    ctx.set_walk(warps, variant)
    ctx.set_systems([0, n])
    s = State.from_bodies(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    return ctx, s


CASES = {
    "plummer8192": lambda: ic.plummer(8192),
    "disk16384": lambda: ic.star_disk(16384),
    "binary4099": lambda: ic.binary_disk(4099),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("variant", [0, 1, 3], ids=["walk64", "walk128", "walk96"])
@pytest.mark.parametrize("comp", [0, 1, 2], ids=["plain", "split", "kahan"])
def test_quadrupole_walk_matches_oracle(cuda, name, variant, comp):
    b = CASES[name]()
    ctx, s = _run(b, variant, comp)
    t, e2 = ctx.constants()
    ot = O.build(b.x, b.y, b.z, b.m)
    q = O.quadrupoles(b.x, b.y, b.z, b.m, ot)
    f = O.forces(b.x, b.y, b.z, b.m, ot, t, e2, quad=q)
    nl, no = ctx.walk_stats()
    assert np.array_equal(nl, f.nlist) and np.array_equal(no, f.nopen)
    rel = _rel(s.acc(), f.a64)
    assert np.median(rel) <= MED_TOL and rel.max() <= MAX_TOL, (np.median(rel), rel.max())


def test_quadrupoles_reduce_the_direct_sum_error(cuda):
    """Binary star + disk (the benchmark's recipe at 2^18 bodies): quadrupoles
    bring the forces closer to the FP64 direct sum than monopoles, on the same
    lists."""
    from nns_gb300.barnes_hut import Context, State
    b = ic.binary_disk(1 << 18)
    n = len(b.x)
    out = {}
    for mp in (0, 1):
        ctx = Context(max_bodies=n, theta=0.5, eps=0.005, multipole=mp)
        ctx.set_systems([0, n])
        s = State.from_bodies(b)
        ctx.build(s)
        ctx.forces(s)
        ctx.sync()
        out[mp] = (s.acc(), ctx.tree_info()["interactions"])
    tg = np.random.default_rng(3).choice(n, 2048, replace=False)
    d = O.direct_fp64(b.x, b.y, b.z, b.m, float(np.float32(0.005) ** 2), tg)
    e0, e1 = np.median(_rel(out[0][0][tg], d)), np.median(_rel(out[1][0][tg], d))
    assert out[0][1] == out[1][1]
    assert e1 < 0.5 * e0, (e0, e1)


def test_quadrupole_batched_equals_unbatched(cuda):
    from nns_gb300.barnes_hut import Context, State
    sizes = [3000, 20000, 1, 5000]
    parts = [ic.star_disk(k, seed=ic.SEED0 + 60 + j) for j, k in enumerate(sizes)]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    b = ic.Bodies(*(np.concatenate([getattr(q, f) for q in parts]) for f in ("x", "y", "z", "vx", "vy", "vz", "m")))
    ctx = Context(max_bodies=int(off[-1]), max_systems=len(sizes), theta=0.5, eps=0.01, multipole=1)
    ctx.set_systems(off)
    s = State.from_bodies(b)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    acc = s.acc()
    for j, q in enumerate(parts):
        _, s1 = _run(q, variant=ctx.params.walk_variant)
        assert np.array_equal(acc[off[j]:off[j + 1]], s1.acc()), j


def test_quadrupole_graph_and_switching(cuda):
    from nns_gb300._lib import NbxError
    from nns_gb300.barnes_hut import Context, State
    b = ic.plummer(6000)
    n = len(b.x)
    eager = Context(max_bodies=n, theta=0.5, eps=0.01, dt=1e-3, multipole=1)
    eager.set_systems([0, n])
    se = State.from_bodies(b)
    for _ in range(3):
        eager.step(se, 1)
    graph = Context(max_bodies=n, theta=0.5, eps=0.01, dt=1e-3)
    graph.set_systems([0, n])
    graph.set_multipole(1)
    sg = State.from_bodies(b)
    graph.graph_step(sg, 3)
    graph.sync()
    eager.sync()
    assert all(np.array_equal(u, v) for u, v in zip(se.host(), sg.host()))
    # switching the order needs a new build; back to monopoles gives the monopole walk's bits
    mono = Context(max_bodies=n, theta=0.5, eps=0.01)
    mono.set_systems([0, n])
    sm = State.from_bodies(b)
    mono.build(sm)
    mono.forces(sm)
    graph.set_multipole(0)
    s2 = State.from_bodies(b)
    with pytest.raises(NbxError) as e:
        graph.forces(s2)
    assert e.value.code == 9  # NBX_ERR_STATE
    graph.build(s2)
    graph.forces(s2)
    graph.sync()
    mono.sync()
    assert np.array_equal(s2.acc(), sm.acc())
    # the adjoint's recorded walk is monopole-only
    from nns_gb300.adjoint import Adjoint
    graph.set_multipole(1)
    with pytest.raises(NbxError) as e:
        Adjoint(graph, 4, 2, 4096, 2)
    assert e.value.code == 1  # NBX_ERR_ARG


def _quad_vs_oracle(b, eps=0.01, variant=3):
    ctx, s = _run(b, variant=variant, eps=eps)
    t, e2 = ctx.constants()
    ot = O.build(b.x, b.y, b.z, b.m)
    q = O.quadrupoles(b.x, b.y, b.z, b.m, ot)
    f = O.forces(b.x, b.y, b.z, b.m, ot, t, e2, quad=q)
    nl, no = ctx.walk_stats()
    assert ctx.tree_info()["status"] == 0
    assert np.array_equal(nl, f.nlist) and np.array_equal(no, f.nopen)
    return s.acc().astype(np.float64), f.a64


@pytest.mark.parametrize("n", [1, 2, 3, 31, 33, 100])
def test_quadrupole_small_and_ragged(cuda, n):
    """Tiny and ragged systems (root children only, a partial walk group, one
    body past a whole group): the same lists as the oracle, forces within
    1e-4 of its FP64 quadrupole evaluation (a single body feels nothing)."""
    a, a64 = _quad_vs_oracle(ic.plummer(n, seed=ic.SEED0 + n))
    if n > 1:
        assert _rel(a, a64).max() <= MAX_TOL
    else:
        assert not a.any()


@pytest.mark.parametrize("variant", [3, 1], ids=["walk96", "walk128"])
@pytest.mark.parametrize("name", ["collinear", "coplanar", "signed_zeros", "cluster", "deep"])
def test_quadrupole_adversarial_geometry(cuda, name, variant):
    """The adversarial sets of the parity tests in quadrupole mode: degenerate
    boxes (cells whose second moments vanish along an axis), signed zeros, split
    planes, a tight cluster and cells past level 32 (second moments of nearly
    coincident bodies).  Lists bit-exact; each body's error bounded relative to
    its own force plus the set's median force (pulls that nearly cancel on a
    line or in a plane leave only the summation-order error)."""
    from adversarial import CASES, EPS
    a, a64 = _quad_vs_oracle(CASES[name](), eps=EPS.get(name, 0.01), variant=variant)
    rel = _rel(a, a64)
    assert np.median(rel) <= MED_TOL, np.median(rel)
    err = np.linalg.norm(a - a64, axis=1)
    mag = np.linalg.norm(a64, axis=1)
    assert (err <= MAX_TOL * (mag + np.median(mag))).all(), (err / (mag + np.median(mag))).max()


def test_quadrupole_softening_range(cuda):
    """The quadrupole terms are evaluated in the unit vector d / r, so any normal
    softening works in the mode (the deep adversarial set above uses 1e-12); a
    zero or subnormal softening is refused in either mode, leaving the context
    unchanged."""
    from nns_gb300._lib import NbxError
    from nns_gb300.barnes_hut import Context
    ctx = Context(max_bodies=64, theta=0.5, eps=1e-15, multipole=1)
    t, e2 = ctx.constants()
    assert e2 == np.float32(1e-15) * np.float32(1e-15)
    for mp in (1, 0):
        ctx.set_multipole(mp)
        for bad in (0.0, 1e-40, float("inf")):
            with pytest.raises(NbxError):
                ctx.set_constants(t, bad)
            assert ctx.constants()[1] == e2
