"""nbx_compute_bounding_box_noalloc (context-free, static scratch) against the
context entry point nbx_compute_bounding_box, both through the C ABI.

Two calls in a row on different body sets (the second smaller, so the first
call's partials and ticket are still in the shared scratch): the boxes must be
bit-identical (min/max are exact, so the tolerance is zero).  Oversized grids
are rejected before anything is launched, and calls after the first leave the
device's free memory unchanged.
"""
import ctypes as C

import numpy as np
import pytest

from nns_gb300 import ic

pytestmark = pytest.mark.gpu

NBX_ERR_SCRATCH = 11


def _box(seed_value=0.0):
    import torch
    return torch.full((6,), seed_value, dtype=torch.float32, device="cuda")


def _ptrs(b):
    return [C.c_void_p(b[k].data_ptr()) for k in range(6)]


def _bodies(n, seed, shift):
    import torch
    b = ic.binary_disk(n, seed=seed)
    xyz = np.stack([b.x, b.y, b.z]).astype(np.float32) + np.float32(shift)
    return torch.as_tensor(xyz, device="cuda")


def _context_box(L, ctx, xyz, out):
    n = xyz.shape[1]
    rc = L.nbx_compute_bounding_box(ctx.h, None, C.c_void_p(xyz[0].data_ptr()), C.c_void_p(xyz[1].data_ptr()),
                                    C.c_void_p(xyz[2].data_ptr()), *_ptrs(out), n, None, None)
    assert rc == 0, rc


def _noalloc_box(L, xyz, out, grid=0):
    n = xyz.shape[1]
    return L.nbx_compute_bounding_box_noalloc(None, C.c_void_p(xyz[0].data_ptr()), C.c_void_p(xyz[1].data_ptr()),
                                              C.c_void_p(xyz[2].data_ptr()), *_ptrs(out), n, grid, None)


def test_noalloc_bounding_box_matches_context_entry_point(cuda):
    import torch
    from nns_gb300._lib import lib
    from nns_gb300.barnes_hut import Context
    L = lib()
    ctx = Context(max_bodies=1 << 20)
    cases = [(_bodies(1 << 20, ic.SEED0 + 1, 0.0), 0.0),      # large grid (1216 blocks)
             (_bodies(50_000, ic.SEED0 + 2, -3.5), 0.0),      # smaller grid after it
             (_bodies(1_000, ic.SEED0 + 3, 7.0), -100.0)]     # merge into a non-zero box
    for xyz, seed_value in cases:
        want, got = _box(seed_value), _box(seed_value)
        _context_box(L, ctx, xyz, want)
        assert _noalloc_box(L, xyz, got) == 0
        torch.cuda.synchronize()
        assert torch.equal(want, got), (want.tolist(), got.tolist())
    # the box itself against numpy (origin included by the zero seed)
    xyz = cases[0][0]
    got = _box(0.0)
    assert _noalloc_box(L, xyz, got, grid=4096) == 0
    a = xyz.cpu().numpy()
    ref = np.array([min(0.0, a[0].min()), max(0.0, a[0].max()), min(0.0, a[1].min()), max(0.0, a[1].max()),
                    min(0.0, a[2].min()), max(0.0, a[2].max())], dtype=np.float32)
    assert np.array_equal(got.cpu().numpy(), ref)


def test_noalloc_bounding_box_rejects_oversized_grid(cuda):
    import torch
    from nns_gb300._lib import lib
    L = lib()
    xyz = _bodies(4096, ic.SEED0 + 4, 0.0)
    out = _box(1.0)
    assert _noalloc_box(L, xyz, out, grid=4097) == NBX_ERR_SCRATCH
    assert L.nbx_status_string(NBX_ERR_SCRATCH).decode().startswith("request exceeds")
    assert _noalloc_box(L, xyz, out, grid=-1) == 1
    torch.cuda.synchronize()
    assert torch.equal(out, _box(1.0))  # nothing launched


def test_noalloc_bounding_box_allocates_nothing(cuda):
    """The property the entry point exists for: after a first call (which may load
    the module), calls of several sizes leave the device's free memory unchanged.
    Contexts of earlier tests are collected first, so that none is freed while
    the calls are measured."""
    import gc
    import torch
    from nns_gb300._lib import lib
    L = lib()
    sets = [_bodies(n, ic.SEED0 + 10 + j, 0.5 * j) for j, n in enumerate((1 << 18, 3000, 1 << 16))]
    out = _box(0.0)
    assert _noalloc_box(L, sets[0], out) == 0  # warm-up
    gc.collect()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for xyz in sets * 3:
        for grid in (0, 1, 4096):
            assert _noalloc_box(L, xyz, out, grid=grid) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
