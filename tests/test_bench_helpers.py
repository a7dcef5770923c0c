"""Host-side helpers of bench.py (no GPU): the committed walk-traffic figure is
read from its profile, the HBM roofline arithmetic, and the guard that keeps a
failing extension section from losing the JSON line."""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import bench  # noqa: E402


def test_walk_traffic_is_read_from_the_profile():
    t = bench.walk_traffic(1 << 24)
    assert isinstance(t, int) and t > 10 ** 9


def test_hbm_roofline_arithmetic():
    r = bench.hbm_roofline(1 << 24, 0.2, {"hbm_gbs": 6000.0})
    assert r["bytes_per_body"] == 60 and r["unit"] == "GB/s"
    assert abs(r["achieved"] - 60.0 * (1 << 24) / 0.2e-3 / 1e9) < 0.1
    assert abs(r["frac"] - r["achieved"] / 6000.0) < 1e-3
    assert bench.hbm_roofline(1 << 20, 0.1, {})["frac"] is None


def test_failing_section_is_reported_not_raised():
    def boom(*_):
        raise RuntimeError("no such device")

    out = bench._section(boom, 1, 2)
    assert out == {"unavailable": "RuntimeError: no such device"}
    assert bench._section(lambda a, b: {"ok": a + b}, 1, 2) == {"ok": 3}
