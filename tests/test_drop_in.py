"""The reference's own driver (3D/CUDA/CUDA_NBody/src/main.cu) builds against
libnbx with only its two includes of KernelsWrapper.cuh and BarnesHut.cuh
pointed at include/nbx/ (oracle/drop_in.py stages it), on the CPU: it compiles,
links to libnbx.so, and answers -h before any CUDA call.  Its GPU run is in
tests/test_gpu_runner.py."""
import subprocess

import pytest


@pytest.fixture(scope="module")
def driver():
    from oracle import drop_in
    path = drop_in.build()
    if path is None:
        pytest.skip("the reference driver is not staged on this host")
    return path


def test_reference_driver_links_against_libnbx(driver):
    from oracle import drop_in
    main = open(drop_in.os.path.join(drop_in.STAGE, "src", "main.cu")).read()
    assert '#include "nbx/BarnesHut.cuh"' in main and '#include "nbx/KernelsWrapper.cuh"' in main
    assert "../include/BarnesHut.cuh" not in main and "new BarnesHut(parameters)" in main
    out = subprocess.run([driver, "-h"], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    assert "CUDA Barnes-Hut NBody code" in out.stdout and "--particles" in out.stdout
    ldd = subprocess.run(["ldd", driver], capture_output=True, text=True).stdout
    assert "libnbx.so" in ldd
