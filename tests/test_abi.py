"""The C ABI library loads and exports every symbol include/nbx.h declares.

CPU-only: no entry point that touches a GPU is called here."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "nbx.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nbx_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from nns_gb300 import build
    lib = ctypes.CDLL(build.build())
    names = _declared()
    assert len(names) >= 27
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from nns_gb300 import _lib
    assert set(_declared()) == set(_lib.SIGNATURES)


def test_status_strings_without_gpu():
    from nns_gb300 import _lib
    L = _lib.lib()
    assert L.nbx_status_string(3).decode().startswith("two bodies")
    p = _lib.nbx_params()
    L.nbx_params_default(ctypes.byref(p))
    assert p.group == 32 and p.stack_depth >= 360 and abs(p.theta - 0.5) < 1e-7


def test_create_rejects_bad_params_without_gpu():
    from nns_gb300 import _lib
    L = _lib.lib()
    p = _lib.nbx_params()
    L.nbx_params_default(ctypes.byref(p))
    p.group = 16  # the walk group is a warp
    h = ctypes.c_void_p()
    assert L.nbx_create(ctypes.byref(p), ctypes.byref(h)) == 1


def test_params_layout_and_option_ranges_without_gpu():
    """The library's defaults for the option fields at the end of nbx_params, and
    out-of-range options rejected before any CUDA call."""
    from nns_gb300 import _lib
    L = _lib.lib()
    p = _lib.nbx_params()
    L.nbx_params_default(ctypes.byref(p))
    assert p.moments_mode == 0 and p.key_order == 0 and p.node_capacity == 0
    assert p.radix_bits == 8 and p.stack_depth == 512
    for field, bad in (("moments_mode", 3), ("moments_mode", -1), ("key_order", 2), ("walk_variant", 4),
                       ("radix_bits", 7), ("radix_bits", 10), ("stack_depth", 359), ("stack_depth", 4097)):
        q = _lib.nbx_params()
        L.nbx_params_default(ctypes.byref(q))
        setattr(q, field, bad)
        h = ctypes.c_void_p()
        assert L.nbx_create(ctypes.byref(q), ctypes.byref(h)) == 1, field


def test_constants_validated_without_gpu():
    """The softening and MAC constant in use must be finite and positive, the
    squared softening a normal float (a body's own term is 0 * inf without it):
    rejected before any CUDA call, in either multipole order."""
    from nns_gb300 import _lib
    L = _lib.lib()
    cases = ((dict(eps=0.0, eps2=0.0), 1), (dict(eps=-0.0, eps2=0.0), 1), (dict(eps=1e-20, eps2=0.0), 1),
             (dict(eps2=float("inf")), 1), (dict(eps=float("nan"), eps2=0.0), 1),
             (dict(theta=0.0, theta_ref=0.0), 1), (dict(theta_ref=float("inf")), 1),
             (dict(eps=0.0, eps2=0.0, multipole=1), 1), (dict(eps=1e-20, eps2=0.0, multipole=1), 1))
    for kw, rc in cases:
        q = _lib.nbx_params()
        L.nbx_params_default(ctypes.byref(q))
        for k, v in kw.items():
            setattr(q, k, v)
        h = ctypes.c_void_p()
        assert L.nbx_create(ctypes.byref(q), ctypes.byref(h)) == rc, kw
    assert L.nbx_set_constants(None, 0.25, 1e-4, 0) == 1


def test_capacity_bounds_without_gpu():
    """max_bodies above 2^26 and node pools above 2^28 are rejected before any CUDA call."""
    from nns_gb300 import _lib
    L = _lib.lib()
    for field, bad in (("max_bodies", (1 << 26) + 1), ("node_capacity", (1 << 28) + 1)):
        q = _lib.nbx_params()
        L.nbx_params_default(ctypes.byref(q))
        q.max_bodies = 1 << 20
        setattr(q, field, bad)
        h = ctypes.c_void_p()
        assert L.nbx_create(ctypes.byref(q), ctypes.byref(h)) == 1, field


def test_set_tuning_validates_without_gpu():
    """nbx_set_tuning rejects a null context and out-of-range values before any CUDA call."""
    from nns_gb300 import _lib
    L = _lib.lib()
    assert L.nbx_set_tuning(None, 8, 512) == 1
    assert L.nbx_set_tuning(None, 9, 4096) == 1


def test_checkpoint_size_without_gpu():
    """nbx_checkpoint_bytes: the 80-byte header, nsys + 1 int64 offsets, seven float
    arrays and the 8-byte payload checksum; 0 for an empty request."""
    from nns_gb300 import _lib
    L = _lib.lib()
    for n, nsys in ((1, 1), (4096, 1), (14499946, 512), (1 << 26, 1)):
        assert L.nbx_checkpoint_bytes(n, nsys) == 80 + 8 * (nsys + 1) + 7 * 4 * n + 8
    assert L.nbx_checkpoint_bytes(0, 1) == 0 and L.nbx_checkpoint_bytes(5, 0) == 0
