"""Initial conditions: deterministic, counter-based, recipe properties."""
import numpy as np

from nns_gb300 import ic


def test_counter_based_prefix_stable():
    a = ic.star_disk(1000)
    b = ic.star_disk(4000)
    for k in ("x", "y", "z", "vx", "m"):
        assert np.array_equal(getattr(a, k)[1:1000], getattr(b, k)[1:1000])


def test_star_disk_recipe():
    b = ic.star_disk(16384)
    assert b.m[0] == 1.0 and b.x[0] == 0 and np.all(b.m[1:] == np.float32(1e-6))
    r = np.hypot(b.x[1:], b.y[1:])
    assert r.min() >= 0.0999 and r.max() <= 1.0001
    v = np.hypot(b.vx[1:], b.vy[1:])
    assert np.allclose(v, np.sqrt(1 / r), rtol=1e-5)
    assert not ic.has_duplicates(b)


def test_plummer_truncation_and_mass():
    b = ic.plummer(20000)
    r = np.sqrt(b.x.astype(np.float64) ** 2 + b.y ** 2 + b.z ** 2)
    assert r.max() <= 20.0001
    assert abs(b.m.sum() - 1.0) < 1e-4
    # half-mass radius of a Plummer sphere is ~1.305 a
    assert abs(np.median(r) - 1.305) < 0.05


def test_binary_disk_recipe():
    b = ic.binary_disk(1000)
    assert np.allclose(b.x[:2], [0.1, -0.1]) and np.all(b.m[:2] == 0.5)
    assert np.allclose(abs(b.vy[:2]), 0.5 * np.sqrt(5.0))


def test_batched_sizes():
    s = ic.batched_sizes(512)
    assert s.min() >= 1024 and s.max() < 2 ** 17
    assert 10e6 < s.sum() < 20e6
