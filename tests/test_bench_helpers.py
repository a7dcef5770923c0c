"""Host-side helpers of bench.py (no GPU): the committed walk-traffic figure is
read from its profile (only while the walk's source has the captured git blob
hash), the HBM roofline arithmetic, the accuracy sweep's bisection, and the guard that keeps a failing
extension section from losing the JSON line."""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import bench  # noqa: E402


def test_walk_traffic_is_read_from_the_profile(monkeypatch):
    """The figure is reported only for the walk source it was captured from."""
    blob = [ln.split(":")[1].strip() for ln in open(os.path.join(HERE, "..", "profiles",
                                                                "k_walk2_traffic_binary_disk_2p24.md"))
            if ln.startswith("walk2_cu_blob:")][0]
    monkeypatch.setattr(bench, "_git_blob_sha1", lambda path: blob)
    t = bench.walk_traffic(1 << 24)
    assert isinstance(t, int) and t > 10 ** 9
    assert bench.walk_traffic(1 << 20) is None
    monkeypatch.setattr(bench, "_git_blob_sha1", lambda path: "0" * 40)
    assert bench.walk_traffic(1 << 24) is None


def test_git_blob_hash(tmp_path):
    p = tmp_path / "f"
    p.write_bytes(b"hello\n")
    assert bench._git_blob_sha1(str(p)) == "ce013625030ba8dba906f756967f9e9ca394464a"


def test_hbm_roofline_arithmetic():
    r = bench.hbm_roofline(1 << 24, 0.2, {"hbm_gbs": 6000.0})
    assert r["bytes_per_body"] == 60 and r["unit"] == "GB/s"
    assert abs(r["achieved"] - 60.0 * (1 << 24) / 0.2e-3 / 1e9) < 0.1
    assert abs(r["frac"] - r["achieved"] / 6000.0) < 1e-3
    assert bench.hbm_roofline(1 << 20, 0.1, {})["frac"] is None
    # an untimed integrate phase gives no figure instead of a division by zero
    r0 = bench.hbm_roofline(1 << 20, 0.0, {"hbm_gbs": 6000.0})
    assert r0["achieved"] is None and r0["frac"] is None


def test_failing_section_is_reported_not_raised():
    def boom(*_):
        raise RuntimeError("no such device")

    out = bench._section(boom, 1, 2)
    assert out == {"unavailable": "RuntimeError: no such device"}
    assert bench._section(lambda a, b: {"ok": a + b}, 1, 2) == {"ok": 3}


def _fake_measure(threshold):
    """A sweep whose error meets the target at every theta <= threshold."""
    calls = []

    def measure(th, refine=False):
        calls.append((th, refine))
        return {"theta": th, "refine": refine}, th <= threshold
    return measure, calls


def test_accuracy_sweep_bisects_towards_the_last_miss():
    measure, calls = _fake_measure(0.53)
    points, at = bench.sweep_to_target(measure, (0.7, 0.6, 0.5, 0.4), 2)
    # coarse: 0.7, 0.6 miss, 0.5 meets; then 0.55 misses, 0.525 meets
    assert [c[0] for c in calls] == [0.7, 0.6, 0.5, 0.55, 0.525]
    assert [c[1] for c in calls] == [False, False, False, True, True]
    assert at["theta"] == 0.525 and len(points) == 5


def test_accuracy_sweep_edges():
    # the first theta meets the target: nothing to bisect
    measure, calls = _fake_measure(1.0)
    points, at = bench.sweep_to_target(measure, (0.7, 0.6), 2)
    assert at["theta"] == 0.7 and len(calls) == 1
    # no theta meets it: no refinement, no point at the target
    measure, calls = _fake_measure(0.1)
    points, at = bench.sweep_to_target(measure, (0.7, 0.6), 2)
    assert at is None and len(points) == 2
