"""ctypes binding of libnbx.so (the C ABI declared in include/nbx.h).

The library is loaded from the package directory.  There is no fallback: if
libnbx.so is missing the import fails with instructions to build it.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("NBX_LIB_PATH", os.path.join(HERE, "libnbx.so"))

NBX_OK = 0
STATUS_NAMES = {
    0: "NBX_OK", 1: "NBX_ERR_ARG", 2: "NBX_ERR_CUDA", 3: "NBX_ERR_DEPTH", 4: "NBX_ERR_CAPACITY",
    5: "NBX_ERR_STACK", 6: "NBX_ERR_NONFINITE", 7: "NBX_ERR_CLUSTER", 8: "NBX_ERR_TIMEOUT",
    9: "NBX_ERR_STATE", 10: "NBX_ERR_NOMEM", 11: "NBX_ERR_SCRATCH", 12: "NBX_ERR_FORMAT",
}


class nbx_params(C.Structure):
    _fields_ = [("max_bodies", C.c_int), ("max_systems", C.c_int), ("theta", C.c_float),
                ("theta_ref", C.c_float), ("eps", C.c_float), ("eps2", C.c_float),
                ("dt", C.c_float), ("dampening", C.c_float), ("gravity", C.c_float),
                ("group", C.c_int), ("stack_depth", C.c_int), ("compensated", C.c_int),
                ("leaf_size", C.c_int), ("radix_bits", C.c_int), ("walk_warps", C.c_int),
                ("device", C.c_int), ("block_size", C.c_int), ("grid_size", C.c_int),
                ("walk_variant", C.c_int), ("key_order", C.c_int), ("node_capacity", C.c_int),
                ("moments_mode", C.c_int), ("multipole", C.c_int)]


class nbx_state(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "m")]


class nbx_tree_info(C.Structure):
    _fields_ = [("nbodies", C.c_int64), ("ncells", C.c_int64), ("nnodes", C.c_int64),
                ("max_level", C.c_int32), ("nsystems", C.c_int32), ("interactions", C.c_int64),
                ("opened", C.c_int64), ("refined_runs", C.c_int32), ("status", C.c_int32),
                ("launches", C.c_int64), ("rounds", C.c_int64), ("candidates", C.c_int64)]


class nbx_render_params(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("render_scale", C.c_double),
                ("max_velocity_color", C.c_double), ("min_velocity_color", C.c_double),
                ("particle_brightness", C.c_double), ("particle_sharpness", C.c_double),
                ("dot_size", C.c_int), ("system_size", C.c_double)]


_P = C.c_void_p
_I = C.c_int
_F = C.c_float
_PF = C.POINTER(C.c_float)

# name -> (restype, argtypes); every symbol declared in include/nbx.h
SIGNATURES = {
    "nbx_params_default": (None, [C.POINTER(nbx_params)]),
    "nbx_create": (_I, [C.POINTER(nbx_params), C.POINTER(_P)]),
    "nbx_destroy": (_I, [_P]),
    "nbx_status_string": (C.c_char_p, [_I]),
    "nbx_last_error": (C.c_char_p, [_P]),
    "nbx_get_constants": (_I, [_P, _PF, _PF]),
    "nbx_set_constants": (_I, [_P, _F, _F, _I]),
    "nbx_reset_arrays": (_I, [_P] + [_P] * 16 + [_I, _I, _P, _PF]),
    "nbx_compute_bounding_box": (_I, [_P] + [_P] * 10 + [_I, _P, _PF]),
    "nbx_compute_bounding_box_noalloc": (_I, [_P] * 10 + [_I, _I, _P]),
    "nbx_build_tree": (_I, [_P] + [_P] * 14 + [_I, _I, _P, _PF]),
    "nbx_centre_of_mass": (_I, [_P] + [_P] * 5 + [_I, _P, _PF]),
    "nbx_sort": (_I, [_P] + [_P] * 5 + [_I, _P, _PF]),
    "nbx_compute_forces": (_I, [_P] + [_P] * 14 + [_I, _F, _P, _PF]),
    "nbx_update": (_I, [_P] + [_P] * 9 + [_I, _F, _F, _P, _PF]),
    "nbx_set_walk_config": (_I, [_P, _I, _I]),
    "nbx_set_tuning": (_I, [_P, _I, _I]),
    "nbx_set_multipole": (_I, [_P, _I]),
    "nbx_set_leaf_size": (_I, [_P, _I]),
    "nbx_group_count": (_I, [_P, _P]),
    "nbx_forces_groups": (_I, [_P, _P, _I, _I, _P]),
    "nbx_export_group_stats": (_I, [_P, _P, _P, _P]),
    "nbx_set_systems": (_I, [_P, _I, C.POINTER(C.c_int64)]),
    "nbx_build": (_I, [_P, C.POINTER(nbx_state), _P]),
    "nbx_forces": (_I, [_P, C.POINTER(nbx_state), _P]),
    "nbx_integrate": (_I, [_P, C.POINTER(nbx_state), _P]),
    "nbx_step": (_I, [_P, C.POINTER(nbx_state), _I, _P]),
    "nbx_graph_step": (_I, [_P, C.POINTER(nbx_state), _I, _P]),
    "nbx_sync_status": (_I, [_P, _P]),
    "nbx_selftest_sort_wait": (_I, [_P, _P]),
    "nbx_get_tree_info": (_I, [_P, _P, C.POINTER(nbx_tree_info)]),
    "nbx_export_tree": (_I, [_P, _I] + [_P] * 10 + [_I, C.POINTER(C.c_int64), _P]),
    "nbx_export_keys": (_I, [_P, _P, _P, _P]),
    "nbx_export_walk_stats": (_I, [_P, _P, _P, _P]),
    "nbx_direct_fp64": (_I, [_P, _P, _P, _P, _P, _I, _P, _I, C.c_double, _P, _P]),
    "nbx_potential": (_I, [_P, C.POINTER(nbx_state), _P, _P]),
    "nbx_forces_fp64_lists": (_I, [_P, _P, _I, _P, _P]),
    "nbx_diagnostics_fp64": (_I, [_P, C.POINTER(nbx_state), _I, _P, _P]),
    "nbx_render_params_default": (None, [C.POINTER(nbx_render_params)]),
    "nbx_checkpoint_bytes": (C.c_int64, [C.c_int64, _I]),
    "nbx_checkpoint_save": (_I, [_P, C.POINTER(nbx_state), _P, C.c_int64, C.POINTER(C.c_int64), _P]),
    "nbx_checkpoint_restore": (_I, [_P, C.POINTER(nbx_state), _P, C.c_int64, _P]),
    "nbx_render_frame": (_I, [_P, C.POINTER(nbx_state), _I, C.POINTER(nbx_render_params), _P, _P, _P]),
    "nbx_adjoint_create": (_I, [_P, _I, _I, _I, _I, C.POINTER(_P)]),
    "nbx_adjoint_destroy": (_I, [_P]),
    "nbx_adjoint_forward": (_I, [_P, _P, C.POINTER(nbx_state), _P, _P, _P, C.POINTER(C.c_double), _P]),
    "nbx_adjoint_backward": (_I, [_P, _P, C.POINTER(nbx_state)] + [_P] * 7 + [_P]),
    "nbx_adjoint_record": (_I, [_P, _P, C.POINTER(nbx_state), _P]),
    "nbx_adjoint_replay_fp64": (_I, [_P, _P, _P, C.POINTER(C.c_double), _P]),
    "nbx_adjoint_stats": (_I, [_P, C.POINTER(C.c_int64), _PF, _PF]),
}

_lib = None


class NbxError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str = ""):
        self.code = code
        name = STATUS_NAMES.get(code, str(code))
        super().__init__("%s: %s%s" % (where, name, (" (" + detail + ")") if detail else ""))


def lib():
    """The loaded libnbx.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libnbx.so not found at %s: run `python -c 'import __graft_entry__ as g; "
                              "g.build()'` (or `python nns_gb300/build.py`) first" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int, where: str, ctx=None):
    if rc != NBX_OK:
        detail = ""
        if ctx is not None:
            detail = (lib().nbx_last_error(ctx) or b"").decode()
        raise NbxError(rc, where, detail)
