"""The oracle against the reference's own kernels (compiled for the CPU) on
adversarial geometry: degenerate boxes, signed zeros, bodies on split planes,
a tight cluster and a tree past level 32.  Box, permutation and tree bit-exact."""
import numpy as np
import pytest

from adversarial import CASES
from nns_gb300 import ic
from oracle import oracle as O


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_matches_reference_kernels(name):
    b = CASES[name]()
    assert not ic.has_duplicates(b)
    ref = O.ref_step(b.x, b.y, b.z, b.vx, b.vy, b.vz, b.m, 1e-3)
    if ref is None:
        pytest.skip("reference kernels not built")
    t = O.build(b.x, b.y, b.z, b.m)
    assert np.array_equal(O.bbox(b.x, b.y, b.z), ref["bbox"])
    assert np.array_equal(t.perm, ref["perm"])
    assert np.array_equal(t.root_child, ref["root_child"])
    assert t.ncells == ref["ncells"]
    assert np.array_equal(t.cell_child, ref["cell_child"])
    assert np.array_equal(t.cell_start, ref["cell_start"])
    assert np.array_equal(t.cell_count, ref["cell_count"])
    assert np.array_equal(t.cell_level, ref["cell_level"])
