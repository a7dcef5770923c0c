"""The command-line driver (nns_gb300/nbx_runner): the reference's main.cu flags,
its TIME report (main.cu:125-181) and frames written like Renderer::createFrame
(images/StepNNNNN.ppm every renderInterval steps, Renderer.cpp:149-158)."""
import os
import re
import subprocess

import pytest

pytestmark = pytest.mark.gpu


def test_runner_report_and_frames(cuda, tmp_path):
    from nns_gb300 import build
    build.build()
    out = subprocess.run([build.RUNNER, "-n", "4096", "-i", "5", "-R", "2", "-r", "-v"], cwd=tmp_path,
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    text = out.stdout
    for phase in ("reset arrays", "compute bounding boxes", "build tree", "compute COM", "sort",
                  "compute forces", "update bodies", "copy from device to host"):
        assert re.search(r"Time to %s: [0-9.e+-]+ms\n\tper step: [0-9.e+-]+ms" % phase, text), phase
    assert "TOTAL TIME (without copying)" in text
    assert "Number of particles: 4096" in text and "Number of iterations: 5" in text
    assert len(re.findall(r"Elapsed time for step \d+", text)) == 5
    frames = sorted(os.listdir(tmp_path / "images"))
    assert frames == ["Step00001.ppm", "Step00002.ppm", "Step00003.ppm"]  # steps 0, 2, 4
    data = open(tmp_path / "images" / "Step00001.ppm", "rb").read()
    head = b"P6\n1024 1024\n255\n"
    assert data.startswith(head) and len(data) == len(head) + 3 * 1024 * 1024
    assert any(data[len(head):])  # something was drawn



@pytest.mark.parametrize("model", ["ref-plummer", "disk", "plummer"])
def test_runner_models(cuda, tmp_path, model):
    from nns_gb300 import build
    build.build()
    out = subprocess.run([build.RUNNER, "-n", "2048", "-i", "2", "--model", model], cwd=tmp_path,
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    m = re.search(r"final position of body 1: (\S+) (\S+) (\S+)", out.stdout)
    assert m and all(abs(float(v)) < 1e6 for v in m.groups())


def test_reference_driver_runs_on_libnbx(cuda, tmp_path):
    """The reference's main.cu, relinked against libnbx (oracle/drop_in.py), runs
    a few steps of its own disk model through BarnesHut(parameters) and prints
    its TIME report (main.cu:125-181) through the reference's Logger."""
    from oracle import drop_in
    path = drop_in.build()
    if path is None:
        pytest.skip("the reference driver is not staged on this host")
    out = subprocess.run([path, "-n", "4096", "-i", "3"], cwd=tmp_path, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr
    text = out.stdout
    for phase in ("reset arrays", "compute bounding boxes", "build tree", "compute COM", "sort",
                  "compute forces", "update bodies", "copy from device to host"):
        m = re.search(r"Time to %s: ([0-9.e+-]+)ms" % phase, text)
        assert m and float(m.group(1)) >= 0.0, phase
    assert float(re.search(r"Time to compute forces: ([0-9.e+-]+)ms", text).group(1)) > 0.0
    assert "TOTAL TIME" in text
