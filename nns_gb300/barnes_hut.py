"""Host side of the Barnes-Hut pipeline, mirroring the reference's host classes.

* ``KernelsWrapper`` -- the seven phase methods of the reference's
  KernelsWrapper (3D/CUDA/CUDA_NBody/include/KernelsWrapper.cuh:28-48), same
  names, argument order and array semantics, each returning elapsed
  milliseconds (0 when ``timing`` is False), over device tensors.
* ``BarnesHut`` -- the reference's BarnesHut host class
  (src/BarnesHut.cu:12-301): owns the SoA arrays of length numNodes = 2N+12000,
  runs one step per ``update(step)`` through the wrapper and records the
  per-phase timings.
* ``Context`` / ``State`` -- the native pipeline (many systems, CUDA graphs).

Device memory is held in torch tensors; every computation runs in libnbx.so.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib as L
from ._lib import NbxError, check, lib


def _ptr(t) -> int | None:
    return None if t is None else t.data_ptr()


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


class Context:
    """One libnbx context: tree scratch for up to ``max_bodies`` bodies (<= 2^26).

    ``key_order`` 1 orders bodies along the Hilbert curve (faster walk; lists
    differ from the reference's); ``moments_mode`` picks the centre-of-mass pass
    (0 by size, 1 per tree level, 2 one launch), all with the same sums;
    ``radix_bits`` 8 or 9 sorts the keys in 8 or 7 passes, to the same order;
    ``multipole`` 1 adds cell quadrupoles to the force and ``leaf_size`` 2..8 makes
    cells of at most that many bodies leaves (both outside the parity mode)."""

    def __init__(self, max_bodies: int, max_systems: int = 1, theta: float = 0.5,
                 theta_ref: float | None = None, eps: float = 0.05, eps2: float | None = None,
                 dt: float = 1e-3, dampening: float = 1.0, compensated: int = 0,
                 stack_depth: int = 512, device: int = 0, key_order: int = 0, node_capacity: int = 0,
                 moments_mode: int = 0, radix_bits: int = 8, multipole: int = 0, leaf_size: int = 1):
        p = L.nbx_params()
        lib().nbx_params_default(C.byref(p))
        p.max_bodies = int(max_bodies)
        p.max_systems = int(max_systems)
        p.theta = theta
        p.theta_ref = theta_ref or 0.0
        p.eps = eps
        p.eps2 = eps2 or 0.0
        p.dt = dt
        p.dampening = dampening
        p.compensated = int(compensated)
        p.stack_depth = stack_depth
        p.radix_bits = int(radix_bits)
        p.node_capacity = node_capacity
        p.moments_mode = moments_mode
        p.device = device
        p.key_order = int(key_order)
        p.multipole = int(multipole)
        p.leaf_size = int(leaf_size)
        self.params = p
        h = C.c_void_p()
        check(lib().nbx_create(C.byref(p), C.byref(h)), "nbx_create")
        self.h = h
        self.device = torch.device("cuda", device)
        self.offsets = None

    def close(self):
        if getattr(self, "h", None):
            lib().nbx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 -- interpreter shutdown
            pass

    # ---- configuration ----
    def constants(self):
        t, e = C.c_float(), C.c_float()
        check(lib().nbx_get_constants(self.h, C.byref(t), C.byref(e)), "nbx_get_constants")
        return t.value, e.value

    def set_constants(self, theta_ref: float, eps2: float, compensated: int = 0):
        """compensated: 0 plain FP32, 1 split compensation, 2 Kahan on every term."""
        check(lib().nbx_set_constants(self.h, theta_ref, eps2, int(compensated)),
              "nbx_set_constants", self.h)
        self.params.compensated = int(compensated)

    def set_walk(self, warps_per_block: int = 8, variant: int = 0):
        """Walk launch shape (4/8/16 warps per block) and variant (0 production, 2 simple)."""
        check(lib().nbx_set_walk_config(self.h, warps_per_block, variant), "nbx_set_walk_config",
              self.h)

    def set_tuning(self, radix_bits: int = 8, stack_depth: int = 512):
        """Sort digit width (8 or 9 bits: 8 or 7 passes, same order) and walk stack
        entries per warp (360..4096).  A built tree stays valid."""
        check(lib().nbx_set_tuning(self.h, int(radix_bits), int(stack_depth)), "nbx_set_tuning", self.h)
        self.params.radix_bits = int(radix_bits)
        self.params.stack_depth = int(stack_depth)

    def set_multipole(self, multipole: int):
        """0 monopoles (the reference's force), 1 with cell quadrupoles; the next
        walk needs a new build."""
        check(lib().nbx_set_multipole(self.h, int(multipole)), "nbx_set_multipole", self.h)
        self.params.multipole = int(multipole)

    def set_leaf_size(self, leaf_size: int):
        """Bodies per leaf bucket, 1 (the reference's tree) to 8; the next walk
        needs a new build."""
        check(lib().nbx_set_leaf_size(self.h, int(leaf_size)), "nbx_set_leaf_size", self.h)
        self.params.leaf_size = int(leaf_size)

    def set_systems(self, offsets):
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        check(lib().nbx_set_systems(self.h, len(off) - 1,
                                    off.ctypes.data_as(C.POINTER(C.c_int64))),
              "nbx_set_systems", self.h)
        self.offsets = off

    # ---- pipeline ----
    def build(self, s: "State", stream=None):
        check(lib().nbx_build(self.h, C.byref(s.c), _stream_ptr(stream)), "nbx_build", self.h)

    def forces(self, s: "State", stream=None):
        check(lib().nbx_forces(self.h, C.byref(s.c), _stream_ptr(stream)), "nbx_forces", self.h)

    def group_count(self) -> int:
        """Walk groups (up to 32 consecutive sorted bodies of one system)."""
        g = C.c_int()
        check(lib().nbx_group_count(self.h, C.byref(g)), "nbx_group_count", self.h)
        return g.value

    def forces_groups(self, s: "State", first: int, count: int, stream=None):
        """The walk of groups [first, first + count) only (a rank's share of a
        split system); other bodies' accelerations are left as they were."""
        check(lib().nbx_forces_groups(self.h, C.byref(s.c), int(first), int(count), _stream_ptr(stream)),
              "nbx_forces_groups", self.h)

    def group_stats(self, stream=None):
        """Per-group list length and opened cells of the last walk (int32 tensors on the device)."""
        ng = self.group_count()
        ln = torch.empty(max(ng, 1), dtype=torch.int32, device=self.device)
        op = torch.empty(max(ng, 1), dtype=torch.int32, device=self.device)
        check(lib().nbx_export_group_stats(self.h, _ptr(ln), _ptr(op), _stream_ptr(stream)),
              "nbx_export_group_stats", self.h)
        return ln[:ng], op[:ng]

    def integrate(self, s: "State", stream=None):
        check(lib().nbx_integrate(self.h, C.byref(s.c), _stream_ptr(stream)), "nbx_integrate",
              self.h)

    def step(self, s: "State", nsteps: int = 1, stream=None):
        """nsteps x (build, forces, integrate), asynchronous on ``stream``.  One step
        launches its kernels; several replay the captured step of graph_step."""
        check(lib().nbx_step(self.h, C.byref(s.c), nsteps, _stream_ptr(stream)), "nbx_step",
              self.h)

    def graph_step(self, s: "State", nsteps: int = 1, stream=None):
        """The same steps replayed from a CUDA graph captured once per state, on the
        context's own stream, ordered after and before ``stream`` by events."""
        check(lib().nbx_graph_step(self.h, C.byref(s.c), nsteps, _stream_ptr(stream)),
              "nbx_graph_step", self.h)

    def sync(self, stream=None):
        """Synchronise and raise NbxError if a kernel reported an error."""
        rc = lib().nbx_sync_status(self.h, _stream_ptr(stream))
        check(rc, "device status", self.h)

    def tree_info(self, stream=None) -> dict:
        info = L.nbx_tree_info()
        check(lib().nbx_get_tree_info(self.h, _stream_ptr(stream), C.byref(info)),
              "nbx_get_tree_info", self.h)
        return {k: getattr(info, k) for k, _ in info._fields_}

    # ---- exports (synchronous) ----
    def export_tree(self, sys: int = 0, stream=None) -> dict:
        off = self.offsets
        n = int(off[sys + 1] - off[sys])
        cap = 2 * n + 4096
        dev = self.device
        i32 = lambda k: torch.empty(k, dtype=torch.int32, device=dev)  # noqa: E731
        f32 = lambda k: torch.empty(k, dtype=torch.float32, device=dev)  # noqa: E731
        perm, root, cc = i32(n), i32(8), i32(8 * cap)
        cs, cn, cl = i32(cap), i32(cap), i32(cap)
        cx, cy, cz, cm = f32(cap), f32(cap), f32(cap), f32(cap)
        nc = C.c_int64()
        check(lib().nbx_export_tree(self.h, sys, _ptr(perm), _ptr(root), _ptr(cc), _ptr(cs),
                                    _ptr(cn), _ptr(cl), _ptr(cx), _ptr(cy), _ptr(cz), _ptr(cm),
                                    cap, C.byref(nc), _stream_ptr(stream)),
              "nbx_export_tree", self.h)
        k = nc.value
        h = lambda t: t.cpu().numpy()  # noqa: E731
        return dict(perm=h(perm), root_child=h(root), cell_child=h(cc[: 8 * k]).reshape(k, 8),
                    cell_start=h(cs[:k]), cell_count=h(cn[:k]), cell_level=h(cl[:k]),
                    cell_x=h(cx[:k]), cell_y=h(cy[:k]), cell_z=h(cz[:k]), cell_m=h(cm[:k]),
                    ncells=k)

    def export_keys(self, stream=None):
        n = int(self.offsets[-1])
        keys = torch.empty(n, dtype=torch.int64, device=self.device)
        perm = torch.empty(n, dtype=torch.int32, device=self.device)
        check(lib().nbx_export_keys(self.h, _ptr(keys), _ptr(perm), _stream_ptr(stream)),
              "nbx_export_keys", self.h)
        return keys.cpu().numpy().view(np.uint64), perm.cpu().numpy()

    def walk_stats(self, stream=None):
        n = int(self.offsets[-1])
        nl = torch.empty(n, dtype=torch.int32, device=self.device)
        no = torch.empty(n, dtype=torch.int32, device=self.device)
        check(lib().nbx_export_walk_stats(self.h, _ptr(nl), _ptr(no), _stream_ptr(stream)),
              "nbx_export_walk_stats", self.h)
        return nl.cpu().numpy(), no.cpu().numpy()

    def direct_fp64(self, s: "State", targets, eps2: float, n: int | None = None, stream=None):
        t = torch.as_tensor(np.asarray(targets, np.int32), device=self.device)
        acc = torch.zeros(3 * len(t), dtype=torch.float64, device=self.device)
        n = int(self.offsets[-1]) if n is None else n
        check(lib().nbx_direct_fp64(self.h, _ptr(s.x), _ptr(s.y), _ptr(s.z), _ptr(s.m), n,
                                    _ptr(t), len(t), eps2, _ptr(acc), _stream_ptr(stream)),
              "nbx_direct_fp64", self.h)
        return acc.view(-1, 3)

    def forces_fp64_lists(self, targets, stream=None) -> np.ndarray:
        """FP64 re-evaluation of the last walk's interaction lists for the walk
        groups holding `targets` (original indices); returns (len(targets), 3)."""
        _, perm = self.export_keys(stream)
        n = len(perm)
        pos = np.empty(n, np.int64)
        pos[perm] = np.arange(n)
        off = self.offsets
        t = np.asarray(targets, np.int64)
        sysid = np.searchsorted(off, t, side="right") - 1
        start = off[sysid] + ((pos[t] - off[sysid]) // 32) * 32
        groups = np.unique(start).astype(np.int32)
        g = torch.as_tensor(groups, device=self.device)
        acc = torch.zeros(3 * n, dtype=torch.float64, device=self.device)
        check(lib().nbx_forces_fp64_lists(self.h, _ptr(g), len(groups), _ptr(acc),
                                          _stream_ptr(stream)), "nbx_forces_fp64_lists", self.h)
        a = acc.view(3, n)[:, torch.as_tensor(t, device=self.device)]
        return a.t().cpu().numpy()

    def potential(self, s: "State", stream=None) -> np.ndarray:
        """Per-body potential over the last build's interaction lists (original order)."""
        n = int(self.offsets[-1])
        phi = torch.empty(n, dtype=torch.float32, device=self.device)
        check(lib().nbx_potential(self.h, C.byref(s.c), _ptr(phi), _stream_ptr(stream)),
              "nbx_potential", self.h)
        return phi.cpu().numpy()

    def checkpoint(self, s: "State", stream=None) -> np.ndarray:
        """Raw checkpoint of every system's bodies and the step constants (uint8 array)."""
        n = int(self.offsets[-1])
        nbytes = lib().nbx_checkpoint_bytes(n, len(self.offsets) - 1)
        buf = np.empty(nbytes, np.uint8)
        written = C.c_int64()
        check(lib().nbx_checkpoint_save(self.h, C.byref(s.c), buf.ctypes.data_as(C.c_void_p), nbytes,
                                        C.byref(written), _stream_ptr(stream)), "nbx_checkpoint_save", self.h)
        return buf[: written.value]

    def restore(self, s: "State", buf, stream=None) -> None:
        """Restores a checkpoint into this context (systems, constants) and s (bodies)."""
        b = np.ascontiguousarray(np.frombuffer(buf, np.uint8) if not isinstance(buf, np.ndarray) else buf, np.uint8)
        check(lib().nbx_checkpoint_restore(self.h, C.byref(s.c), b.ctypes.data_as(C.c_void_p), b.size,
                                           _stream_ptr(stream)), "nbx_checkpoint_restore", self.h)
        nsys = int(np.frombuffer(b[12:16].tobytes(), np.int32)[0])
        self.offsets = [int(v) for v in np.frombuffer(b[80:80 + 8 * (nsys + 1)].tobytes(), np.int64)]

    def diagnostics(self, s: "State", n: int | None = None, stream=None):
        out = torch.zeros(8, dtype=torch.float64, device=self.device)
        n = int(self.offsets[-1]) if n is None else n
        check(lib().nbx_diagnostics_fp64(self.h, C.byref(s.c), n, _ptr(out), _stream_ptr(stream)),
              "nbx_diagnostics_fp64", self.h)
        o = out.cpu().numpy()
        return dict(momentum=o[0:3], kinetic=o[3], angular_momentum=o[4:7], mass=o[7])


@dataclass
class State:
    """Device SoA state (torch tensors on one CUDA device)."""
    x: torch.Tensor
    y: torch.Tensor
    z: torch.Tensor
    vx: torch.Tensor
    vy: torch.Tensor
    vz: torch.Tensor
    ax: torch.Tensor
    ay: torch.Tensor
    az: torch.Tensor
    m: torch.Tensor

    def __post_init__(self):
        self.c = L.nbx_state(*[t.data_ptr() for t in
                               (self.x, self.y, self.z, self.vx, self.vy, self.vz, self.ax,
                                self.ay, self.az, self.m)])

    @classmethod
    def from_bodies(cls, b, device="cuda") -> "State":
        f = lambda a: torch.as_tensor(np.ascontiguousarray(a, np.float32), device=device)  # noqa: E731
        n = len(b.x)
        z = lambda: torch.zeros(n, dtype=torch.float32, device=device)  # noqa: E731
        return cls(f(b.x), f(b.y), f(b.z), f(b.vx), f(b.vy), f(b.vz), z(), z(), z(), f(b.m))

    @classmethod
    def empty(cls, n, device="cuda") -> "State":
        e = lambda: torch.zeros(n, dtype=torch.float32, device=device)  # noqa: E731
        return cls(*(e() for _ in range(10)))

    def acc(self) -> np.ndarray:
        return torch.stack([self.ax, self.ay, self.az], 1).cpu().numpy()

    def host(self):
        return tuple(t.cpu().numpy() for t in (self.x, self.y, self.z, self.vx, self.vy, self.vz))


class KernelsWrapper:
    """The reference's KernelsWrapper (include/KernelsWrapper.cuh:15-50) over libnbx.

    Methods take device tensors (or raw device pointers as ints) in the
    reference's argument order and return the elapsed time in ms."""

    def __init__(self, ctx: Context, grid_size: int = 1024, block_size: int = 256,
                 warp: int = 32, stack_size: int = 64):
        self.ctx = ctx
        self.gridSize = grid_size
        self.blockSize = block_size
        self.warp = warp
        self.stackSize = stack_size

    @staticmethod
    def _p(a):
        return a if isinstance(a, int) else a.data_ptr()

    def _call(self, fn, name, args, timing):
        ms = C.c_float(0.0)
        rc = fn(self.ctx.h, *args, _stream_ptr(None), C.byref(ms) if timing else None)
        check(rc, name, self.ctx.h)
        return ms.value if timing else 0.0

    def resetArrays(self, mutex, x, y, z, mass, count, start, sorted, child, index, minX, maxX,
                    minY, maxY, minZ, maxZ, n, m, timing=False):
        P = self._p
        return self._call(lib().nbx_reset_arrays, "resetArrays",
                          [P(mutex), P(x), P(y), P(z), P(mass), P(count), P(start), P(sorted),
                           P(child), P(index), P(minX), P(maxX), P(minY), P(maxY), P(minZ),
                           P(maxZ), n, m], timing)

    def computeBoundingBox(self, mutex, x, y, z, minX, maxX, minY, maxY, minZ, maxZ, n,
                           timing=False):
        P = self._p
        return self._call(lib().nbx_compute_bounding_box, "computeBoundingBox",
                          [P(mutex), P(x), P(y), P(z), P(minX), P(maxX), P(minY), P(maxY),
                           P(minZ), P(maxZ), n], timing)

    def buildTree(self, x, y, z, mass, count, start, child, index, minX, maxX, minY, maxY, minZ,
                  maxZ, n, m, timing=False):
        P = self._p
        return self._call(lib().nbx_build_tree, "buildTree",
                          [P(x), P(y), P(z), P(mass), P(count), P(start), P(child), P(index),
                           P(minX), P(maxX), P(minY), P(maxY), P(minZ), P(maxZ), n, m], timing)

    def centreOfMass(self, x, y, z, mass, index, n, timing=False):
        P = self._p
        return self._call(lib().nbx_centre_of_mass, "centreOfMass",
                          [P(x), P(y), P(z), P(mass), P(index), n], timing)

    def sort(self, count, start, sorted, child, index, n, timing=False):
        P = self._p
        return self._call(lib().nbx_sort, "sort",
                          [P(count), P(start), P(sorted), P(child), P(index), n], timing)

    def computeForces(self, x, y, z, vx, vy, vz, ax, ay, az, mass, sorted, child, minX, maxX, n,
                      g, timing=False):
        P = self._p
        return self._call(lib().nbx_compute_forces, "computeForces",
                          [P(x), P(y), P(z), P(vx), P(vy), P(vz), P(ax), P(ay), P(az), P(mass),
                           P(sorted), P(child), P(minX), P(maxX), n, C.c_float(g)], timing)

    def update(self, x, y, z, vx, vy, vz, ax, ay, az, n, dt, d, timing=False):
        P = self._p
        return self._call(lib().nbx_update, "update",
                          [P(x), P(y), P(z), P(vx), P(vy), P(vz), P(ax), P(ay), P(az), n,
                           C.c_float(dt), C.c_float(d)], timing)


class BarnesHut:
    """The reference's BarnesHut host class (src/BarnesHut.cu:12-301).

    ``bodies`` (an ic.Bodies) replaces the reference's hard-wired diskModel;
    arrays have numNodes = 2N+12000 entries (BarnesHut.cu:18); ``update(step)``
    runs reset, bounding box, build, centre of mass, sort, forces and update
    and copies positions and velocities back to the host (BarnesHut.cu:195-301)."""

    def __init__(self, bodies, iterations: int = 1, timestep: float = 1e-3, gravity: float = 1.0,
                 dampening: float = 1.0, theta: float = 0.5, theta_ref: float | None = None,
                 eps: float = 0.05, eps2: float | None = None, time_kernels: bool = True,
                 device: int = 0):
        n = len(bodies.x)
        self.numParticles = n
        self.numNodes = 2 * n + 12000
        self.parameters = dict(iterations=iterations, timestep=timestep, gravity=gravity,
                               dampening=dampening)
        self.timeKernels = time_kernels
        self.step = 0
        dev = torch.device("cuda", device)
        m = self.numNodes
        f = lambda: torch.zeros(m, dtype=torch.float32, device=dev)  # noqa: E731
        i = lambda k=m: torch.zeros(k, dtype=torch.int32, device=dev)  # noqa: E731
        self.d_x, self.d_y, self.d_z = f(), f(), f()
        self.d_vx, self.d_vy, self.d_vz = f(), f(), f()
        self.d_ax, self.d_ay, self.d_az = f(), f(), f()
        self.d_mass = f()
        self.d_child = i(8 * m)
        self.d_start, self.d_sorted, self.d_count = i(), i(), i()
        self.d_index, self.d_mutex = i(1), i(1)
        self.d_bbox = torch.zeros(6, dtype=torch.float32, device=dev)
        for name, arr in (("x", bodies.x), ("y", bodies.y), ("z", bodies.z), ("vx", bodies.vx),
                          ("vy", bodies.vy), ("vz", bodies.vz), ("mass", bodies.m)):
            getattr(self, "d_" + name)[:n] = torch.as_tensor(np.asarray(arr, np.float32), device=dev)
        self.ctx = Context(max_bodies=n, theta=theta, theta_ref=theta_ref, eps=eps, eps2=eps2,
                           dt=timestep, dampening=dampening, device=device)
        self.KernelHandler = KernelsWrapper(self.ctx)
        self.times = {k: [] for k in ("resetArrays", "computeBoundingBox", "buildTree",
                                      "centreOfMass", "sort", "computeForces", "update",
                                      "copyDeviceToHost", "all")}
        self.h_x = self.h_y = self.h_z = self.h_vx = self.h_vy = self.h_vz = None

    def _bb(self, k):
        return self.d_bbox[k:k + 1]

    def update(self, step: int | None = None):
        K, n, m, t = self.KernelHandler, self.numParticles, self.numNodes, self.timeKernels
        bb = [self._bb(k) for k in range(6)]
        start = torch.cuda.Event(enable_timing=True)
        stop = torch.cuda.Event(enable_timing=True)
        start.record()
        r = {}
        r["resetArrays"] = K.resetArrays(self.d_mutex, self.d_x, self.d_y, self.d_z, self.d_mass,
                                         self.d_count, self.d_start, self.d_sorted, self.d_child,
                                         self.d_index, *bb, n, m, t)
        r["computeBoundingBox"] = K.computeBoundingBox(self.d_mutex, self.d_x, self.d_y, self.d_z,
                                                       *bb, n, t)
        r["buildTree"] = K.buildTree(self.d_x, self.d_y, self.d_z, self.d_mass, self.d_count,
                                     self.d_start, self.d_child, self.d_index, *bb, n, m, t)
        r["centreOfMass"] = K.centreOfMass(self.d_x, self.d_y, self.d_z, self.d_mass,
                                           self.d_index, n, t)
        r["sort"] = K.sort(self.d_count, self.d_start, self.d_sorted, self.d_child, self.d_index,
                           n, t)
        r["computeForces"] = K.computeForces(self.d_x, self.d_y, self.d_z, self.d_vx, self.d_vy,
                                             self.d_vz, self.d_ax, self.d_ay, self.d_az,
                                             self.d_mass, self.d_sorted, self.d_child, bb[0],
                                             bb[1], n, self.parameters["gravity"], t)
        r["update"] = K.update(self.d_x, self.d_y, self.d_z, self.d_vx, self.d_vy, self.d_vz,
                               self.d_ax, self.d_ay, self.d_az, n, self.parameters["timestep"],
                               self.parameters["dampening"], t)
        c0 = torch.cuda.Event(enable_timing=True)
        c1 = torch.cuda.Event(enable_timing=True)
        c0.record()
        self.h_x, self.h_y, self.h_z = (a[:n].cpu().numpy() for a in (self.d_x, self.d_y, self.d_z))
        self.h_vx, self.h_vy, self.h_vz = (a[:n].cpu().numpy() for a in (self.d_vx, self.d_vy, self.d_vz))
        c1.record()
        stop.record()
        stop.synchronize()
        r["copyDeviceToHost"] = c0.elapsed_time(c1)
        r["all"] = start.elapsed_time(stop)
        for k, v in r.items():
            self.times[k].append(v)
        self.step += 1
        return r
