"""Headless-frame oracle (CPU): the C restatement of the reference renderer
against frames of the reference renderer itself (committed fixtures, and the
reference compiled here where the checkout is present).  Bit-exact."""
import os

import numpy as np
import pytest

from nns_gb300 import ic
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden(name):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_golden  # noqa: WPS433 -- fixture recipe (inputs are regenerated, seeded)
    b, p = make_golden.frame_params(name)
    want = np.load(os.path.join(HERE, "golden", name + ".npz"))["rgb"]
    return b, p, want


@pytest.mark.parametrize("name", ["frame_disk4096", "frame_plummer3000"])
def test_oracle_frame_matches_reference_fixture(name):
    b, p, want = _golden(name)
    got = O.render(b.x, b.y, b.z, b.vx, b.vy, b.vz, p)
    assert got.shape == want.shape
    assert np.array_equal(got, want)


@pytest.mark.parametrize("dot,vmin,sharp", [(7, 0.0, 1.5), (8, 0.9, 1.0), (2, 0.0, 0.5)])
def test_oracle_frame_matches_reference_renderer(dot, vmin, sharp):
    b = ic.star_disk(3000, seed=ic.SEED0 + 9)
    p = O.RenderParams(width=96, height=80, render_scale=1.5, max_velocity_color=3.0, min_velocity_color=vmin,
                       particle_sharpness=sharp, dot_size=dot, system_size=O.system_size(b.x, b.y, b.z))
    want = O.ref_render(b.x, b.y, b.z, b.vx, b.vy, b.vz, p)
    if want is None:
        pytest.skip("reference checkout not present")
    got = O.render(b.x, b.y, b.z, b.vx, b.vy, b.vz, p)
    assert np.array_equal(got, want)


def test_oracle_frame_edges():
    # bodies on the selection border, behind the minimum speed, and outside the frame
    x = np.array([0.0, 10.0, -10.0, 0.5, 0.0], np.float32)
    y = np.array([0.0, 0.0, 0.0, 0.5, 0.0], np.float32)
    z = np.zeros(5, np.float32)
    vx = np.array([1.0, 1.0, 1.0, 0.1, 0.0], np.float32)
    zero = np.zeros(5, np.float32)
    p = O.RenderParams(width=64, height=64, render_scale=1.0, max_velocity_color=1.0, min_velocity_color=0.05,
                       system_size=1.0)
    got = O.render(x, y, z, vx, zero, zero, p)
    want = O.ref_render(x, y, z, vx, zero, zero, p)
    if want is not None:
        assert np.array_equal(got, want)
    assert got[32, 32].any() and not got[0].any()


def test_ppm_writer(tmp_path):
    from nns_gb300.render import frame_path, write_ppm
    img = (np.arange(4 * 6 * 3) % 256).astype(np.uint8).reshape(4, 6, 3)
    path = frame_path(str(tmp_path / "images"), 20, 10)
    assert path.endswith("Step00003.ppm")
    write_ppm(path, img)
    data = open(path, "rb").read()
    assert data.startswith(b"P6\n6 4\n255\n") and data[len(b"P6\n6 4\n255\n"):] == img.tobytes()
