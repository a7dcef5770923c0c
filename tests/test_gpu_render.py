"""Headless frames on the GPU (nbx_render_frame) against the oracle's
restatement of the reference renderer (itself bit-exact with the reference).

Tolerance: the GPU's dot weights and sums are FP32 where the reference uses
FP64, so a byte may land one step lower or higher where the sum sits on a
quantisation boundary: every byte within 1, and at most 1 % of the bytes
different.
"""
import os

import numpy as np
import pytest

from nns_gb300 import ic

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _close(got, want):
    d = np.abs(got.astype(np.int16) - want.astype(np.int16))
    assert d.max() <= 1, int(d.max())
    assert (d > 0).mean() <= 0.01, float((d > 0).mean())
    assert (want > 0).sum() > 100  # the frame is not empty


def _gpu_frame(b, params, build=False, steps=0):
    from nns_gb300.barnes_hut import Context, State
    from nns_gb300.render import Frame, default_params
    n = len(b.x)
    ctx = Context(max_bodies=n, theta=0.5, eps=0.01, dt=1e-3)
    ctx.set_systems([0, n])
    s = State.from_bodies(b)
    if build or steps:
        ctx.build(s)
    if steps:
        ctx.step(s, steps)
    ctx.sync()
    p = default_params(**params)
    img = Frame(p).render(ctx, s).cpu().numpy()
    ctx.sync()
    host = [t.cpu().numpy() for t in (s.x, s.y, s.z, s.vx, s.vy, s.vz)]
    return img, host


def _oracle(host, params):
    from oracle import oracle as O
    return O.render(*host, O.RenderParams(**params))


def test_frame_natural_order(cuda):
    from oracle import oracle as O
    b = ic.star_disk(20000, seed=ic.SEED0 + 21)
    prm = dict(width=256, height=256, max_velocity_color=2.0, system_size=O.system_size(b.x, b.y, b.z))
    img, host = _gpu_frame(b, prm)
    _close(img, _oracle(host, prm))


def test_frame_sorted_order_after_steps(cuda):
    from oracle import oracle as O
    b = ic.plummer(50000, seed=ic.SEED0 + 22)
    prm = dict(width=320, height=240, render_scale=1.0, max_velocity_color=1.0, min_velocity_color=0.05,
               particle_sharpness=1.3, dot_size=7, system_size=O.system_size(b.x, b.y, b.z))
    img, host = _gpu_frame(b, prm, steps=3)
    _close(img, _oracle(host, prm))


@pytest.mark.parametrize("name", ["frame_disk4096", "frame_plummer3000"])
def test_frame_against_reference_fixture(cuda, name):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_golden
    b, p = make_golden.frame_params(name)
    want = np.load(os.path.join(HERE, "golden", name + ".npz"))["rgb"]
    prm = dict(width=p.width, height=p.height, render_scale=p.render_scale,
               max_velocity_color=p.max_velocity_color, system_size=p.system_size)
    img, _ = _gpu_frame(b, prm, build=True)
    _close(img, want)


def test_frame_full_size_default_constants(cuda):
    """1024 x 1024 with the reference's constants (velocity colour range scaled to
    the model's speeds), 2^20 bodies in the tree's sorted order."""
    from oracle import oracle as O
    b = ic.plummer(1 << 20, seed=ic.SEED0 + 23)
    prm = dict(max_velocity_color=1.5, system_size=O.system_size(b.x, b.y, b.z))
    img, host = _gpu_frame(b, prm, build=True)
    assert img.shape == (1024, 1024, 3)
    _close(img, _oracle(host, prm))


def test_frame_rejects_bad_parameters(cuda):
    import ctypes as C
    import torch
    from nns_gb300._lib import lib
    from nns_gb300.barnes_hut import Context, State
    from nns_gb300.render import default_params
    b = ic.star_disk(1000)
    ctx = Context(max_bodies=1000)
    s = State.from_bodies(b)
    buf = torch.empty(3 * 64 * 64, dtype=torch.float32, device="cuda")
    rgb = torch.empty(3 * 64 * 64, dtype=torch.uint8, device="cuda")
    for kw in (dict(system_size=0.0), dict(system_size=1.0, dot_size=17), dict(system_size=1.0, width=0)):
        p = default_params(**dict(dict(width=64, height=64), **kw))
        assert lib().nbx_render_frame(ctx.h, C.byref(s.c), 1000, C.byref(p), buf.data_ptr(), rgb.data_ptr(),
                                      None) == 1
