"""The oracle (oracle/refemu.c) pinned against the reference's own kernels.

The fixtures in tests/golden/ are one step of 3D/CUDA/CUDA_NBody/src/Kernels.cu
run on the CPU (tests/golden/make_golden.py).  Pinned here, on the CPU:
* bounding box, sorted body order and canonical tree topology: bit-exact;
* the warp-coherent walk, given the reference's own cell moments: forces within
  1e-5 median / 1e-4 max relative error (observed ~1e-9 / 3e-6: only rsqrt and
  FMA rounding differ);
* centres of mass: the oracle's FP64-summed moments versus the reference's FP32
  atomic sums, within the FP32 accumulation error of the reference;
* the update: within the rounding of one unfused multiply-add (the reference
  host build rounds v += dt*a in two steps; the oracle and the GPU fuse them).
"""
import copy
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(p for p in glob.glob(os.path.join(HERE, "golden", "*.npz"))
                  if not os.path.basename(p).startswith(("frame_", "sfc_")))
REF_THETA, REF_EPS2 = 1.5, 0.0025  # Kernels.cu:17-18


def _load(path):
    return dict(np.load(path))


def _rel(a, b):
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-30)


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_topology_bit_exact(path):
    g = _load(path)
    x, y, z, m = g["in_x"], g["in_y"], g["in_z"], g["in_m"]
    assert np.array_equal(O.bbox(x, y, z), g["bbox"])
    t = O.build(x, y, z, m)
    assert np.array_equal(t.perm, g["perm"])
    assert np.array_equal(t.root_child, g["root_child"])
    assert np.array_equal(t.cell_child, g["cell_child"])
    assert np.array_equal(t.cell_start, g["cell_start"])
    assert np.array_equal(t.cell_count, g["cell_count"])
    assert np.array_equal(t.cell_level, g["cell_level"])


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_keys_order_is_reference_order(path):
    g = _load(path)
    x, y, z = g["in_x"], g["in_y"], g["in_z"]
    hi, lo = O.keys(x, y, z, g["bbox"], 42)
    order = np.lexsort((lo, hi))
    assert np.array_equal(order, g["perm"])


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_walk_matches_reference(path):
    g = _load(path)
    x, y, z, m = g["in_x"], g["in_y"], g["in_z"], g["in_m"]
    t = O.build(x, y, z, m)
    tr = copy.copy(t)
    tr.cell_x, tr.cell_y, tr.cell_z, tr.cell_m = g["cell_x"], g["cell_y"], g["cell_z"], g["cell_m"]
    f = O.forces(x, y, z, m, tr, REF_THETA, REF_EPS2)
    rel = _rel(f.a.astype(np.float64), g["a"].astype(np.float64))
    assert np.median(rel) <= 1e-5 and rel.max() <= 1e-4, (np.median(rel), rel.max())
    if "tight_a" in g:
        fb = g["tight_bounds"]
        d0 = O.depth0(np.array([fb[0], fb[1], 0, 0, 0, 0], np.float32), REF_THETA)
        ft = O.forces(x, y, z, m, tr, REF_THETA, REF_EPS2, depth0_value=d0)
        rel = _rel(ft.a.astype(np.float64), g["tight_a"].astype(np.float64))
        assert np.median(rel) <= 1e-5 and rel.max() <= 1e-4, (np.median(rel), rel.max())
        assert ft.nlist.mean() > f.nlist.mean()  # tighter MAC, longer lists


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_com_fp64_vs_reference_fp32(path):
    g = _load(path)
    t = O.build(g["in_x"], g["in_y"], g["in_z"], g["in_m"])
    # FP32 running sums over `count` terms: relative error bound ~ count * 2^-24
    bound = np.maximum(g["cell_count"], 2) * 2.0 ** -23
    mrel = np.abs(t.cell_m.astype(np.float64) - g["cell_m"]) / t.cell_m
    assert np.all(mrel <= bound), mrel.max()
    ext = float(max(g["bbox"][1] - g["bbox"][0], g["bbox"][3] - g["bbox"][2]))
    for k in ("x", "y", "z"):
        d = np.abs(getattr(t, "cell_" + k).astype(np.float64) - g["cell_" + k])
        assert np.all(d <= bound * ext + 1e-7), (k, d.max())


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_update_within_one_ulp(path):
    g = _load(path)
    dt = float(g["dt"])
    st = O.update(g["in_x"], g["in_y"], g["in_z"], g["in_vx"], g["in_vy"], g["in_vz"], g["a"], dt)
    sp = lambda a: np.spacing(np.abs(a).astype(np.float32)).astype(np.float64)  # noqa: E731
    a = g["a"]
    for c, k in enumerate("xyz"):
        p, v = st[c], st[3 + c]
        rv, rp = g["out_v" + k], g["out_" + k]
        # the reference rounds dt*a before adding it: one ulp of the product
        # plus one of the sum; the position inherits dt times that
        tol_v = sp(np.maximum(np.abs(v), np.abs(rv))) + sp(dt * a[:, c])
        assert np.all(np.abs(v.astype(np.float64) - rv) <= tol_v), "v" + k
        tol_p = sp(np.maximum(np.abs(p), np.abs(rp))) + sp(dt * rv) + dt * tol_v
        assert np.all(np.abs(p.astype(np.float64) - rp) <= tol_p), k


def test_deep_fixture_goes_past_level_21():
    g = _load(os.path.join(HERE, "golden", "deep1024.npz"))
    assert g["cell_level"].max() > 21


def test_direct_fp64_self_consistency():
    from nns_gb300 import ic
    b = ic.plummer(512)
    a = O.direct_fp64(b.x, b.y, b.z, b.m, 1e-4, np.arange(512))
    # total force of a self-gravitating system is zero (Newton's third law)
    tot = (a * b.m[:, None].astype(np.float64)).sum(0)
    assert np.abs(tot).max() < 1e-12


def test_hilbert_keys_are_the_reference_conversion():
    """The oracle's Lebesgue-to-Hilbert conversion equals the reference's own
    Lebesgue2Hilbert (SpaceFillingCurves/src/Tree.cpp:90-104) on its fixture
    (a seeded disk's keys and random 63-bit keys) and, where the reference code
    builds here, on fresh random keys."""
    g = _load(os.path.join(HERE, "golden", "sfc_hilbert4096.npz"))
    assert np.array_equal(O.hilbert(g["lebesgue_md"]), g["hilbert"])
    rnd = np.random.default_rng(11).integers(0, 2 ** 63, size=100000, dtype=np.uint64)
    live = O.ref_hilbert(rnd)
    if live is not None:
        assert np.array_equal(O.hilbert(rnd), live)
