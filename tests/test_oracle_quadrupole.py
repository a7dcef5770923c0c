"""The oracle's quadrupole extension (orc_quad and the quadrupole evaluation of
orc_forces), on the CPU.

The reference's kernels carry monopoles only (3D/CUDA/CUDA_NBody/src/
Kernels.cu:538-551); the quadrupole mode is this project's extension, so its
oracle is pinned to first principles instead:
* each cell's composed quadrupole equals the traceless second moment of its
  own bodies about its FP64 centre of mass, computed directly;
* the quadrupole terms leave the interaction lists unchanged and bring the
  FP64 evaluation closer to the FP64 direct sum than monopoles alone.
"""
import numpy as np

from nns_gb300 import ic
from oracle import oracle as O


def test_quadrupoles_equal_direct_second_moments():
    b = ic.plummer(3000, seed=ic.SEED0 + 9)
    t = O.build(b.x, b.y, b.z, b.m)
    q = O.quadrupoles(b.x, b.y, b.z, b.m, t)
    pos = np.stack([b.x, b.y, b.z], 1).astype(np.float64)
    m = b.m.astype(np.float64)
    for k in range(t.ncells):
        idx = t.perm[t.cell_start[k]:t.cell_start[k] + t.cell_count[k]]
        s = pos[idx] - t.cell_com64[k]
        mm = m[idx]
        m2 = np.einsum("i,ij,ik->jk", mm, s, s)
        want = 3.0 * m2 - np.trace(m2) * np.eye(3)
        got = np.array([[q[k, 0], q[k, 3], q[k, 4]], [q[k, 3], q[k, 1], q[k, 5]], [q[k, 4], q[k, 5], q[k, 2]]])
        scale = mm.sum() * (s * s).sum(1).max() + 1e-300
        assert np.abs(got - want).max() <= 1e-12 * scale, k
        assert abs(got.trace()) <= 1e-12 * scale


def test_quadrupole_evaluation_same_lists_and_closer_to_direct_sum():
    for b, th, eps in ((ic.plummer(8192), 0.5, 0.01), (ic.star_disk(8192), 0.5, 0.01)):
        n = len(b.x)
        t = O.build(b.x, b.y, b.z, b.m)
        q = O.quadrupoles(b.x, b.y, b.z, b.m, t)
        f0 = O.forces(b.x, b.y, b.z, b.m, t, th * th, eps * eps)
        f1 = O.forces(b.x, b.y, b.z, b.m, t, th * th, eps * eps, quad=q)
        assert np.array_equal(f0.nlist, f1.nlist) and np.array_equal(f0.nopen, f1.nopen)
        tg = np.arange(0, n, 7)
        d = O.direct_fp64(b.x, b.y, b.z, b.m, eps * eps, tg)
        e0 = np.linalg.norm(f0.a64[tg] - d, axis=1) / np.linalg.norm(d, axis=1)
        e1 = np.linalg.norm(f1.a64[tg] - d, axis=1) / np.linalg.norm(d, axis=1)
        assert np.median(e1) < 0.5 * np.median(e0), (np.median(e0), np.median(e1))


def test_bucket_tree_invariants():
    """oracle.bucket_tree (the leaf buckets of nbx_params.leaf_size): every leaf
    cell holds at most k bodies, its parent more, its child slots are its own
    bodies; k = 1 is the reference's tree and gives its walk."""
    b = ic.plummer(4000, seed=ic.SEED0 + 5)
    t = O.build(b.x, b.y, b.z, b.m)
    n = t.n
    for k in (1, 2, 4, 8):
        bt = O.bucket_tree(t, k)
        todo = [(c - n, -1) for c in bt.root_child if c >= n]
        cells = 0
        while todo:
            c, par = todo.pop()
            cells += 1
            ch = bt.cell_child[c]
            if (ch[ch >= 0] < n).all() and t.cell_count[c] <= k:
                assert par < 0 or t.cell_count[par] > k
                want = t.perm[t.cell_start[c]:t.cell_start[c] + t.cell_count[c]]
                assert np.array_equal(ch[ch >= 0], want)
            else:
                assert t.cell_count[c] > k or k == 1
            todo.extend((int(x) - n, c) for x in ch if x >= n)
        assert cells == O.reachable_cells(bt)
        if k == 1:
            assert cells == t.ncells
    f1 = O.forces(b.x, b.y, b.z, b.m, O.bucket_tree(t, 1), 0.25, 1e-4)
    f0 = O.forces(b.x, b.y, b.z, b.m, t, 0.25, 1e-4)
    assert np.array_equal(f0.nlist, f1.nlist) and np.array_equal(f0.a, f1.a)
