"""Synthetic initial conditions for the Barnes-Hut workloads.

All draws come from a counter-based SplitMix64 stream: draw ``k`` of body
``i`` under seed ``s`` is a pure function of ``(s, i, k)``, so every run (CPU
or GPU, any host) sees identical bodies.  Positions, velocities and masses are
generated in FP64 and cast to FP32 SoA arrays.

The disk velocity convention (clockwise, ``vx = v sin(phi)``, ``vy = -v cos(phi)``)
follows BarnesHut::diskModel (3D/CUDA/CUDA_NBody/src/BarnesHut.cu:404-405);
the radius laws, masses and units are the workload definitions (G = 1).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SEED0 = 20261203
_GOLD = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix(z: np.ndarray) -> np.ndarray:
    z = z.astype(np.uint64, copy=True)
    with np.errstate(over="ignore"):
        z ^= z >> np.uint64(30)
        z *= _M1
        z ^= z >> np.uint64(27)
        z *= _M2
        z ^= z >> np.uint64(31)
    return z


def uniform(seed: int, idx: np.ndarray, draw: int) -> np.ndarray:
    """U[0,1) doubles for bodies ``idx`` and draw number ``draw``."""
    idx = np.asarray(idx, dtype=np.uint64)
    with np.errstate(over="ignore"):
        base = _mix(np.array([seed], np.uint64) * _GOLD + np.uint64(draw) * np.uint64(0xD1B54A32D192ED03))
        z = _mix(base + (idx + np.uint64(1)) * _GOLD)
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed: int, idx: np.ndarray, draw: int) -> np.ndarray:
    """Standard normals by Box-Muller over draws (draw, draw+1)."""
    u1 = uniform(seed, idx, draw)
    u2 = uniform(seed, idx, draw + 1)
    return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * np.pi * u2)


@dataclass
class Bodies:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    vx: np.ndarray
    vy: np.ndarray
    vz: np.ndarray
    m: np.ndarray

    @property
    def n(self) -> int:
        return len(self.x)

    def arrays(self):
        return self.x, self.y, self.z, self.vx, self.vy, self.vz, self.m


def _pack(x, y, z, vx, vy, vz, m) -> Bodies:
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
    return Bodies(f(x), f(y), f(z), f(vx), f(vy), f(vz), f(m))


def _disk(seed, idx, rmin, rmax, zfrac, mass_in):
    r = rmin + (rmax - rmin) * uniform(seed, idx, 0)
    phi = 2.0 * np.pi * uniform(seed, idx, 1)
    zz = zfrac * r * normal(seed, idx, 2)
    v = np.sqrt(mass_in / r)
    return r * np.cos(phi), r * np.sin(phi), zz, v * np.sin(phi), -v * np.cos(phi), np.zeros_like(r)


def star_disk(n: int, seed: int = SEED0, disk_mass: float = 1e-6, rmin: float = 0.1,
              rmax: float = 1.0, zfrac: float = 0.01) -> Bodies:
    """Central star of mass 1 at the origin plus n-1 disk bodies of mass disk_mass
    (radius uniform in [rmin, rmax], z ~ N(0, (zfrac*r)^2), Keplerian speed sqrt(1/r))."""
    idx = np.arange(n - 1, dtype=np.uint64)
    x, y, z, vx, vy, vz = _disk(seed, idx, rmin, rmax, zfrac, 1.0)
    m = np.full(n - 1, disk_mass)
    cat = lambda s, a: np.concatenate([[s], a])  # noqa: E731
    return _pack(cat(0.0, x), cat(0.0, y), cat(0.0, z), cat(0.0, vx), cat(0.0, vy), cat(0.0, vz),
                 cat(1.0, m))


def binary_disk(n: int, seed: int = SEED0, disk_mass: float = 1e-8, rmin: float = 0.3,
                rmax: float = 2.0, zfrac: float = 0.01, sep: float = 0.2) -> Bodies:
    """Two 0.5-mass stars on a circular orbit (separation sep) plus n-2 disk bodies."""
    idx = np.arange(n - 2, dtype=np.uint64)
    x, y, z, vx, vy, vz = _disk(seed, idx, rmin, rmax, zfrac, 1.0)
    vs = 0.5 * np.sqrt(1.0 / sep)
    sx = [0.5 * sep, -0.5 * sep]
    svy = [-vs, vs]  # clockwise, as the disk
    m = np.full(n - 2, disk_mass)
    return _pack(np.concatenate([sx, x]), np.concatenate([[0.0, 0.0], y]),
                 np.concatenate([[0.0, 0.0], z]), np.concatenate([[0.0, 0.0], vx]),
                 np.concatenate([svy, vy]), np.concatenate([[0.0, 0.0], vz]),
                 np.concatenate([[0.5, 0.5], m]))


def plummer(n: int, seed: int = SEED0, a: float = 1.0, rmax: float = 20.0) -> Bodies:
    """Plummer sphere, total mass 1, scale radius a, truncated at rmax*a (G=1).
    Radius from the inverse mass CDF; speed by von Neumann rejection on
    q^2 (1-q^2)^(7/2) (bound 0.1), v = q * sqrt(2) * (1+r^2/a^2)^(-1/4)."""
    idx = np.arange(n, dtype=np.uint64)
    umax = (1.0 + 1.0 / (rmax * rmax)) ** -1.5
    u = uniform(seed, idx, 0) * umax
    u = np.maximum(u, 1e-300)
    r = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
    ct = 2.0 * uniform(seed, idx, 1) - 1.0
    st = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
    ph = 2.0 * np.pi * uniform(seed, idx, 2)
    x, y, z = r * st * np.cos(ph), r * st * np.sin(ph), r * ct
    q = np.zeros(n)
    todo = np.arange(n)
    draw = 3
    while todo.size:
        qq = uniform(seed, idx[todo], draw)
        tt = 0.1 * uniform(seed, idx[todo], draw + 1)
        ok = tt < qq * qq * (1.0 - qq * qq) ** 3.5
        q[todo[ok]] = qq[ok]
        todo = todo[~ok]
        draw += 2
        if draw > 4000:
            raise RuntimeError("rejection sampler did not converge")
    v = q * np.sqrt(2.0) * (1.0 + (r / a) ** 2) ** -0.25
    ct2 = 2.0 * uniform(seed, idx, 1001) - 1.0
    st2 = np.sqrt(np.maximum(0.0, 1.0 - ct2 * ct2))
    ph2 = 2.0 * np.pi * uniform(seed, idx, 1002)
    m = np.full(n, 1.0 / n)
    return _pack(x, y, z, v * st2 * np.cos(ph2), v * st2 * np.sin(ph2), v * ct2, m)


def batched_sizes(nsys: int = 512, seed: int = SEED0, lo: float = 10.0, hi: float = 17.0) -> np.ndarray:
    """System sizes floor(2^U[lo,hi]) for the batched workload."""
    u = uniform(seed, np.arange(nsys, dtype=np.uint64), 7)
    return np.floor(2.0 ** (lo + (hi - lo) * u)).astype(np.int64)


def batched_star_disks(nsys: int = 512, seed: int = SEED0):
    """Independent star+disk systems, system i seeded with seed+1+i.
    Returns (Bodies concatenated, offsets[nsys+1])."""
    sizes = batched_sizes(nsys, seed)
    parts = [star_disk(int(s), seed + 1 + i) for i, s in enumerate(sizes)]
    off = np.zeros(nsys + 1, np.int64)
    off[1:] = np.cumsum(sizes)
    cat = lambda k: np.concatenate([getattr(p, k) for p in parts])  # noqa: E731
    return _pack(cat("x"), cat("y"), cat("z"), cat("vx"), cat("vy"), cat("vz"), cat("m")), off


def has_duplicates(b: Bodies) -> bool:
    p = np.stack([b.x, b.y, b.z], 1)
    return len(np.unique(p, axis=0)) != len(p)
