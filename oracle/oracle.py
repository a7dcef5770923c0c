"""ctypes front end of the parity oracle (test infrastructure only).

Wraps ``refemu.c`` (the CPU restatement of 3D/CUDA/CUDA_NBody/src/Kernels.cu)
and, where it was built, the reference's own kernels run on the CPU
(``_ref/libref_kernels.so``).  Only tests, the smoke check and the CPU-baseline
leg of ``bench.py`` use this module, as a checker.
"""
from __future__ import annotations

import copy
import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

_lib = None
_ref = None

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(_build.build_oracle())
        L = _lib
        L.orc_bbox.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p]
        L.orc_keys.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_int, _u64p, C.c_void_p]
        L.orc_build.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, _f32p, C.c_int, C.c_int,
                                _i32p, C.POINTER(C.c_int), _i32p, _i32p, _i32p, _i32p, _i32p,
                                _f32p, _f32p, _f32p, _f32p, C.c_void_p, C.c_void_p]
        L.orc_depth0.argtypes = [_f32p, C.c_float]
        L.orc_depth0.restype = C.c_float
        L.orc_forces.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, _i32p, C.c_int, _i32p,
                                 _i32p, _f32p, _f32p, _f32p, _f32p, C.c_float, C.c_float, C.c_int,
                                 C.c_void_p, C.c_int, _f32p, _f32p, _f32p, _f64p, _f64p, _f64p,
                                 _i32p, _i32p]
        L.orc_forces.argtypes = L.orc_forces.argtypes + [C.c_void_p]
        L.orc_forces.restype = C.c_longlong
        L.orc_quad.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_int, _i32p, _f64p, _f64p, _f64p]
        L.orc_update.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p,
                                 _f32p, C.c_float, C.c_float]
        L.orc_direct_fp64.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_double, C.c_int,
                                      _i32p, _f64p, _f64p, _f64p]
        L.orc_direct_pot_fp64.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_double, C.c_int,
                                          _i32p, _f64p]
        L.orc_direct_adjoint.argtypes = [C.c_int, _f64p, _f64p, _f64p, _f64p, C.c_double, C.c_double,
                                         C.c_double, C.c_int, C.POINTER(C.c_double), _f64p, _f64p, _f64p]
    return _lib


def ref_lib():
    """The reference kernels compiled for the CPU, or None where unavailable."""
    global _ref
    if _ref is None:
        path = os.path.join(os.path.dirname(__file__), "_ref", "libref_kernels.so")
        if not os.path.exists(path):
            path = _build.build_ref_kernels()
        if not path or not os.path.exists(path):
            return None
        _ref = C.CDLL(path)
        _ref.ref_run_step.restype = C.c_int
    return _ref


_sfc = None


def ref_sfc_lib():
    """The reference's SpaceFillingCurves key code compiled for the CPU, or None."""
    global _sfc
    if _sfc is None:
        path = os.path.join(os.path.dirname(__file__), "_ref", "libref_sfc.so")
        if not os.path.exists(path):
            path = _build.build_ref_sfc()
        if not path or not os.path.exists(path):
            return None
        _sfc = C.CDLL(path)
        _sfc.ref_lebesgue2hilbert.argtypes = [_u64p, _u64p, C.c_long, C.c_int]
    return _sfc


KEY_MASK = np.uint64((1 << 63) - 1)


def md_key(cuda_key):
    """The reference MD code's Lebesgue key of the same cell path: its child number
    sonNumber = [x>=mid] + 2[y>=mid] + 4[z>=mid] (SpaceFillingCurves/src/Tree.cpp:442)
    is 7 - c for the CUDA path's c = [x<mid] + 2[y<mid] + 4[z<mid], i.e. every
    bit of the 63-bit key inverted."""
    return np.asarray(cuda_key, np.uint64) ^ KEY_MASK


# The 12-state Lebesgue-to-Hilbert tables of the reference (Tree.cpp:70-104):
# Hilbert digit and next state, indexed [state][Lebesgue child number].
HILBERT_DIGIT = np.array([[0, 7, 3, 4, 1, 6, 2, 5], [4, 3, 7, 0, 5, 2, 6, 1], [6, 1, 5, 2, 7, 0, 4, 3],
                          [2, 5, 1, 6, 3, 4, 0, 7], [0, 1, 7, 6, 3, 2, 4, 5], [6, 7, 1, 0, 5, 4, 2, 3],
                          [2, 3, 5, 4, 1, 0, 6, 7], [4, 5, 3, 2, 7, 6, 0, 1], [0, 3, 1, 2, 7, 4, 6, 5],
                          [2, 1, 3, 0, 5, 6, 4, 7], [4, 7, 5, 6, 3, 0, 2, 1], [6, 5, 7, 4, 1, 2, 0, 3]])
HILBERT_STATE = np.array([[8, 10, 3, 3, 4, 5, 4, 5], [2, 2, 11, 9, 4, 5, 4, 5], [7, 6, 7, 6, 8, 10, 1, 1],
                          [7, 6, 7, 6, 0, 0, 11, 9], [0, 8, 1, 11, 6, 8, 6, 11], [10, 0, 9, 1, 10, 7, 9, 7],
                          [10, 4, 9, 4, 10, 2, 9, 3], [5, 8, 5, 11, 2, 8, 3, 11], [4, 9, 0, 0, 7, 9, 2, 2],
                          [1, 1, 8, 5, 3, 3, 8, 6], [11, 5, 0, 0, 11, 6, 2, 2], [1, 1, 4, 10, 3, 3, 7, 10]])


def hilbert(md_lebesgue, levels=21):
    """Lebesgue2Hilbert (Tree.cpp:90-104) restated: the Hilbert key of an MD
    Lebesgue key, digit by digit from the top level, state 0 at the root."""
    k = np.asarray(md_lebesgue, np.uint64)
    out = np.zeros_like(k)
    state = np.zeros(k.shape, np.int64)
    for lv in range(levels, 0, -1):
        cell = ((k >> np.uint64(3 * (lv - 1))) & np.uint64(7)).astype(np.int64)
        out = (out << np.uint64(3)) | HILBERT_DIGIT[state, cell].astype(np.uint64)
        state = HILBERT_STATE[state, cell]
    return out


def ref_hilbert(md_lebesgue, levels=21):
    """The reference's own Lebesgue2Hilbert on the keys, or None where unavailable."""
    L = ref_sfc_lib()
    if L is None:
        return None
    k = np.ascontiguousarray(md_lebesgue, np.uint64)
    out = np.zeros_like(k)
    L.ref_lebesgue2hilbert(k, out, len(k), levels)
    return out


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def bbox(x, y, z):
    out = np.zeros(6, np.float32)
    lib().orc_bbox(len(x), _f32(x), _f32(y), _f32(z), out)
    return out


def keys(x, y, z, bb, levels=21):
    n = len(x)
    hi = np.zeros(n, np.uint64)
    lo = np.zeros(n, np.uint64)
    rc = lib().orc_keys(n, _f32(x), _f32(y), _f32(z), _f32(bb), levels, hi,
                        lo.ctypes.data_as(C.c_void_p))
    if rc:
        raise ValueError("orc_keys rc=%d" % rc)
    return hi, lo


@dataclass
class Tree:
    n: int
    bbox: np.ndarray
    perm: np.ndarray
    ncells: int
    root_child: np.ndarray
    cell_child: np.ndarray
    cell_start: np.ndarray
    cell_count: np.ndarray
    cell_level: np.ndarray
    cell_x: np.ndarray
    cell_y: np.ndarray
    cell_z: np.ndarray
    cell_m: np.ndarray
    cell_m64: np.ndarray | None = None
    cell_com64: np.ndarray | None = None


class OracleError(RuntimeError):
    def __init__(self, rc, what):
        super().__init__("%s failed with status %d" % (what, rc))
        self.rc = rc


def build(x, y, z, m, bb=None, max_depth=42):
    n = len(x)
    x, y, z, m = _f32(x), _f32(y), _f32(z), _f32(m)
    if bb is None:
        bb = bbox(x, y, z)
    bb = _f32(bb)
    cap = 2 * n + 4096
    perm = np.zeros(n, np.int32)
    nc = C.c_int(0)
    rootc = np.zeros(8, np.int32)
    cc = np.zeros(8 * cap, np.int32)
    cs = np.zeros(cap, np.int32)
    cn = np.zeros(cap, np.int32)
    cl = np.zeros(cap, np.int32)
    cx = np.zeros(cap, np.float32)
    cy = np.zeros(cap, np.float32)
    cz = np.zeros(cap, np.float32)
    cm = np.zeros(cap, np.float32)
    m64 = np.zeros(cap, np.float64)
    com64 = np.zeros(3 * cap, np.float64)
    rc = lib().orc_build(n, x, y, z, m, bb, max_depth, cap, perm, C.byref(nc), rootc, cc, cs, cn,
                         cl, cx, cy, cz, cm, m64.ctypes.data_as(C.c_void_p),
                         com64.ctypes.data_as(C.c_void_p))
    if rc:
        raise OracleError(rc, "orc_build")
    k = nc.value
    return Tree(n, bb, perm, k, rootc, cc[: 8 * k].reshape(k, 8).copy(), cs[:k].copy(),
                cn[:k].copy(), cl[:k].copy(), cx[:k].copy(), cy[:k].copy(), cz[:k].copy(),
                cm[:k].copy(), m64[:k].copy(), com64[: 3 * k].reshape(k, 3).copy())


def bucket_tree(tree: Tree, k: int) -> Tree:
    """The tree with leaf buckets of at most k bodies (nbx_params.leaf_size; the
    reference keeps one body per leaf): every cell holding at most k bodies
    whose parent holds more (or which is a root child) becomes a leaf whose
    child slots are its bodies in sorted order; the cells below it become
    unreachable.  Moments are unchanged (a bucket is the same cell)."""
    if k <= 1:
        return tree
    n, nc = tree.n, tree.ncells
    cc = tree.cell_child.copy()
    parent = np.full(nc, -1, np.int64)
    rows, cols = np.nonzero(cc >= n)
    parent[cc[rows, cols] - n] = rows
    cnt = tree.cell_count
    bucket = (cnt <= k) & ((parent < 0) | (cnt[np.maximum(parent, 0)] > k))
    for c in np.nonzero(bucket)[0]:
        cc[c, :] = -1
        cc[c, :cnt[c]] = tree.perm[tree.cell_start[c]:tree.cell_start[c] + cnt[c]]
    out = copy.copy(tree)
    out.cell_child = cc
    return out


def reachable_cells(tree: Tree) -> int:
    """Cells reachable from the root children (bucket_tree leaves some unreachable)."""
    n = tree.n
    todo = [c - n for c in tree.root_child if c >= n]
    seen = 0
    while todo:
        c = todo.pop()
        seen += 1
        todo.extend(int(ch) - n for ch in tree.cell_child[c] if ch >= n)
    return seen


def depth0(bb, theta_ref):
    return float(lib().orc_depth0(_f32(bb), C.c_float(theta_ref)))


@dataclass
class Forces:
    a: np.ndarray        # (n,3) float32, plain FP32 walk (rows of unevaluated bodies are 0)
    a64: np.ndarray      # (n,3) float64, FP64 evaluation of the same interaction lists
    nlist: np.ndarray    # (n,) interaction-list length of the body's group
    nopen: np.ndarray    # (n,) cells opened by the body's group
    total: int           # sum over evaluated bodies of the list length


def quadrupoles(x, y, z, m, tree: Tree):
    """Traceless FP64 quadrupole moments of the tree's cells about their FP64
    centres of mass, (ncells, 6) as (xx, yy, zz, xy, xz, yz) (orc_quad; the
    reference has monopoles only)."""
    k = tree.ncells
    q = np.zeros(6 * max(k, 1))
    cc = np.ascontiguousarray(tree.cell_child.reshape(-1), np.int32)
    if k == 0:
        return q[:0].reshape(0, 6)
    rc = lib().orc_quad(len(x), _f32(x), _f32(y), _f32(z), _f32(m), k, cc,
                        np.ascontiguousarray(tree.cell_m64), np.ascontiguousarray(tree.cell_com64.reshape(-1)), q)
    if rc:
        raise OracleError(rc, "orc_quad")
    return q.reshape(k, 6)


def forces(x, y, z, m, tree: Tree, theta_ref, eps2, group=32, groups=None, depth0_value=None, quad=None):
    """The warp-coherent walk (FP32 and an FP64 evaluation of the same lists).
    ``quad``: per-cell quadrupoles (quadrupoles()) added to the FP64 evaluation
    of accepted cells; the lists do not depend on it."""
    n = len(x)
    x, y, z, m = _f32(x), _f32(y), _f32(z), _f32(m)
    d0 = depth0(tree.bbox, theta_ref) if depth0_value is None else depth0_value
    ax = np.zeros(n, np.float32); ay = np.zeros(n, np.float32); az = np.zeros(n, np.float32)
    gx = np.zeros(n, np.float64); gy = np.zeros(n, np.float64); gz = np.zeros(n, np.float64)
    nl = np.zeros(n, np.int32); no = np.zeros(n, np.int32)
    cc = np.ascontiguousarray(tree.cell_child.reshape(-1), np.int32)
    if cc.size == 0:
        cc = np.full(8, -1, np.int32)
    gptr, ng = None, 0
    if groups is not None:
        garr = np.ascontiguousarray(groups, np.int32)
        gptr, ng = garr.ctypes.data_as(C.c_void_p), len(garr)
    cxa = tree.cell_x if tree.ncells else np.zeros(1, np.float32)
    cya = tree.cell_y if tree.ncells else np.zeros(1, np.float32)
    cza = tree.cell_z if tree.ncells else np.zeros(1, np.float32)
    cma = tree.cell_m if tree.ncells else np.zeros(1, np.float32)
    tot = lib().orc_forces(n, x, y, z, m, np.ascontiguousarray(tree.perm, np.int32), tree.ncells,
                           np.ascontiguousarray(tree.root_child, np.int32), cc,
                           _f32(cxa), _f32(cya), _f32(cza), _f32(cma), C.c_float(d0),
                           C.c_float(eps2), group, gptr, ng, ax, ay, az, gx, gy, gz, nl, no,
                           None if quad is None else np.ascontiguousarray(quad, np.float64).ctypes.data_as(C.c_void_p))
    if tot < 0:
        raise ValueError("orc_forces failed")
    return Forces(np.stack([ax, ay, az], 1), np.stack([gx, gy, gz], 1), nl, no, int(tot))


def update(x, y, z, vx, vy, vz, a, dt, d=1.0):
    x, y, z, vx, vy, vz = (np.array(v, np.float32) for v in (x, y, z, vx, vy, vz))
    a = np.asarray(a, np.float32)
    lib().orc_update(len(x), x, y, z, vx, vy, vz, _f32(a[:, 0]), _f32(a[:, 1]), _f32(a[:, 2]),
                     C.c_float(dt), C.c_float(d))
    return x, y, z, vx, vy, vz


def direct_fp64(x, y, z, m, eps2, targets):
    t = np.ascontiguousarray(targets, np.int32)
    ax = np.zeros(len(t)); ay = np.zeros(len(t)); az = np.zeros(len(t))
    lib().orc_direct_fp64(len(x), _f32(x), _f32(y), _f32(z), _f32(m), C.c_double(eps2), len(t),
                          t, ax, ay, az)
    return np.stack([ax, ay, az], 1)


def direct_potential_fp64(x, y, z, m, eps2, targets):
    t = np.ascontiguousarray(targets, np.int32)
    phi = np.zeros(len(t))
    lib().orc_direct_pot_fp64(len(x), _f32(x), _f32(y), _f32(z), _f32(m), C.c_double(eps2), len(t),
                              t, phi)
    return phi


def direct_adjoint_fp64(x0, v0, m, target, eps2, dt, T, d=1.0):
    """FP64 direct-sum trajectory loss and its gradients (x0, v0, target: (3,n); m: (n,))."""
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
    x0, v0, m, target = f(x0), f(v0), f(m), f(target)
    n = m.size
    gx = np.zeros((3, n)); gv = np.zeros((3, n)); gm = np.zeros(n)
    loss = C.c_double()
    rc = lib().orc_direct_adjoint(n, x0, v0, m, target, C.c_double(eps2), C.c_double(dt),
                                  C.c_double(d), T, C.byref(loss), gx, gv, gm)
    if rc:
        raise OracleError(rc, "orc_direct_adjoint")
    return loss.value, gx, gv, gm


def ref_step(x, y, z, vx, vy, vz, m, dt, force_bounds=None, stack_size=4096):
    """One step of the reference's own kernels on the CPU (None if unavailable).

    Returns a dict with the canonicalised tree, the forces (before the update)
    and the updated state.  ``force_bounds`` replaces (minX, maxX) given to the
    force kernel only, which scales its opening radius (Kernels.cu:477)."""
    R = ref_lib()
    if R is None:
        return None
    n = len(x)
    x, y, z, vx, vy, vz = (np.array(v, np.float32) for v in (x, y, z, vx, vy, vz))
    m = _f32(m)
    cap = 2 * n + 12000
    out = dict(bbox=np.zeros(6, np.float32), perm=np.zeros(n, np.int32),
               root_child=np.zeros(8, np.int32), cell_child=np.zeros(8 * cap, np.int32),
               cell_start=np.zeros(cap, np.int32), cell_count=np.zeros(cap, np.int32),
               cell_level=np.zeros(cap, np.int32), cell_x=np.zeros(cap, np.float32),
               cell_y=np.zeros(cap, np.float32), cell_z=np.zeros(cap, np.float32),
               cell_m=np.zeros(cap, np.float32), ax=np.zeros(n, np.float32),
               ay=np.zeros(n, np.float32), az=np.zeros(n, np.float32))
    nc = C.c_int(0)
    fmn, fmx = (float("nan"), float("nan")) if force_bounds is None else force_bounds
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    rc = R.ref_run_step(C.c_int(n), P(x), P(y), P(z), P(vx), P(vy), P(vz), P(m), C.c_float(dt),
                        C.c_float(fmn), C.c_float(fmx), C.c_int(stack_size), P(out["bbox"]),
                        P(out["perm"]), C.byref(nc), C.c_int(cap), P(out["root_child"]),
                        P(out["cell_child"]), P(out["cell_start"]), P(out["cell_count"]),
                        P(out["cell_level"]), P(out["cell_x"]), P(out["cell_y"]),
                        P(out["cell_z"]), P(out["cell_m"]), P(out["ax"]), P(out["ay"]),
                        P(out["az"]))
    if rc:
        raise RuntimeError("ref_run_step rc=%d" % rc)
    k = nc.value
    out["ncells"] = k
    out["cell_child"] = out["cell_child"][: 8 * k].reshape(k, 8)
    for key in ("cell_start", "cell_count", "cell_level", "cell_x", "cell_y", "cell_z", "cell_m"):
        out[key] = out[key][:k]
    out["a"] = np.stack([out.pop("ax"), out.pop("ay"), out.pop("az")], 1)
    out["state"] = (x, y, z, vx, vy, vz)
    return out


# ---- headless frame (3D/CUDA/CUDA_NBody/src/Renderer.cpp) -------------------

@dataclass
class RenderParams:
    """Renderer constants (3D/CUDA/CUDA_NBody/include/Constants.h:31-38); the
    reference passes systemSize = 2 * BarnesHut::getSystemSize() (main.cu:93-95)."""
    width: int = 1024
    height: int = 1024
    render_scale: float = 2.5
    max_velocity_color: float = 1500.0
    min_velocity_color: float = 0.0
    particle_brightness: float = 0.35
    particle_sharpness: float = 1.0
    dot_size: int = 8
    system_size: float = 1.0

    def args(self):
        return (C.c_int(self.width), C.c_int(self.height), C.c_double(self.render_scale),
                C.c_double(self.max_velocity_color), C.c_double(self.min_velocity_color),
                C.c_double(self.particle_brightness), C.c_double(self.particle_sharpness),
                C.c_int(self.dot_size), C.c_double(self.system_size))


def system_size(x, y, z) -> float:
    """2 * BarnesHut::getSystemSize() (BarnesHut.cu:417-445): twice the largest
    |coordinate|, in float."""
    m = np.float32(max(np.abs(_f32(x)).max(), np.abs(_f32(y)).max(), np.abs(_f32(z)).max(), 0.0))
    return float(np.float32(2.0) * m)


def render(x, y, z, vx, vy, vz, p: RenderParams) -> np.ndarray:
    """The oracle's frame: (height, width, 3) uint8."""
    n = len(x)
    hd = np.zeros(3 * p.width * p.height, np.float64)
    rgb = np.zeros(3 * p.width * p.height, np.uint8)
    L = lib()
    L.orc_render.restype = C.c_int
    rc = L.orc_render(C.c_int(n), *[_f32(a).ctypes.data_as(C.c_void_p) for a in (x, y, z, vx, vy, vz)],
                      *p.args(), hd.ctypes.data_as(C.c_void_p), rgb.ctypes.data_as(C.c_void_p))
    if rc:
        raise OracleError(rc, "orc_render")
    return rgb.reshape(p.height, p.width, 3)


def ref_render(x, y, z, vx, vy, vz, p: RenderParams):
    """The reference renderer's frame, or None where it was not built."""
    path = os.path.join(os.path.dirname(__file__), "_ref", "libref_render.so")
    if not os.path.exists(path):
        path = _build.build_ref_renderer()
    if not path or not os.path.exists(path):
        return None
    R = C.CDLL(path)
    R.ref_render.restype = C.c_int
    rgb = np.zeros(3 * p.width * p.height, np.uint8)
    arrs = [_f32(a) for a in (x, y, z, vx, vy, vz)]
    R.ref_render(C.c_int(len(x)), *[a.ctypes.data_as(C.c_void_p) for a in arrs], *p.args(),
                 rgb.ctypes.data_as(C.c_void_p))
    return rgb.reshape(p.height, p.width, 3)
