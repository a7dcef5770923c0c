"""Config-0 cross-check (CPU): forces at step 0 of the 16384-body star + disk
from the reference's own 3D/Serial tree code (staged from the checkout,
oracle/ref_shim/serial_harness.cpp) against the oracle (the CUDA path's
semantics) and an FP64 direct sum.  The Serial code's MAC (length/|d| < theta)
and softening ((d^2 + eps^2) d) differ from the CUDA path's, so the band is
loose: both are Barnes-Hut approximations of the same direct sum.  The central
star's net force nearly cancels, so medians and p99 are used, not the maximum."""
import numpy as np
import pytest

from nns_gb300 import ic
from oracle import oracle as O
from oracle import ref_cpu


def _rel(u, v):
    return np.linalg.norm(u - v, axis=1) / np.linalg.norm(v, axis=1)


def test_serial_reference_forces_config0():
    b = ic.star_disk(16384)
    a_ref = ref_cpu.serial_forces(b, 0.5, 0.01)
    if a_ref is None:
        pytest.skip("reference 3D/Serial code not staged")
    ot = O.build(b.x, b.y, b.z, b.m)
    f = O.forces(b.x, b.y, b.z, b.m, ot, 0.25, 1e-4)  # theta = 0.5, eps = 0.01
    direct = O.direct_fp64(b.x, b.y, b.z, b.m, 1e-4, np.arange(len(b.x), dtype=np.int32))
    r_ref, r_orc, r_x = _rel(a_ref, direct), _rel(f.a, direct), _rel(a_ref, f.a)
    assert np.median(r_ref) < 3e-3 and np.percentile(r_ref, 99) < 2e-2, (np.median(r_ref), np.percentile(r_ref, 99))
    assert np.median(r_orc) < 3e-4 and np.percentile(r_orc, 99) < 2e-3
    assert np.median(r_x) < 3e-3 and np.percentile(r_x, 99) < 2e-2
