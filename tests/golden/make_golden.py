"""Generates the golden fixtures of this directory from the reference itself.

Each fixture is one Barnes-Hut step of the reference's own kernels
(3D/CUDA/CUDA_NBody/src/Kernels.cu, compiled unmodified for the CPU by
oracle/build.py and run by oracle/ref_shim/ref_harness.cpp): bounding box,
insertion tree (canonicalised to depth-first cell numbering), the reference's
FP32 centres of mass, the sorted body order, the warp-coherent forces and the
state after the update.  The reference's hard-wired constants apply
(eps^2 = 0.0025, theta = 1.5, Kernels.cu:17-18); the "tight" variants hand the
force kernel a wider (minX, maxX) so that its opening radius equals that of
theta_ref = 0.25 (theta = 0.5), see ``force_bounds``.

Run from the repository root where the reference checkout is present:
    python tests/golden/make_golden.py            (every fixture)
    python tests/golden/make_golden.py hilbert    (sfc_hilbert4096.npz only)
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from nns_gb300 import ic  # noqa: E402
from oracle import oracle as O  # noqa: E402

DT = 1e-3


def lattice():
    """Bodies exactly on subdivision planes (multiples of 1/8 inside [-1,1])."""
    g = np.arange(-8, 9) / 8.0
    X, Y, Z = np.meshgrid(g, g, np.array([-0.25, 0.0, 0.25]), indexing="ij")
    x, y, z = X.ravel(), Y.ravel(), Z.ravel()
    n = len(x)
    b = ic.Bodies(*(np.asarray(a, np.float32) for a in (x, y, z, np.zeros(n), np.zeros(n),
                                                        np.zeros(n), np.full(n, 1.0 / n))))
    return b


def deep_pairs():
    """A disk with close pairs that separate only below subdivision level 21."""
    b = ic.star_disk(1024, seed=ic.SEED0 + 77)
    x, y, z = b.x.copy(), b.y.copy(), b.z.copy()
    for k, i in enumerate((100, 300, 500, 700, 900)):
        j = i + 1
        x[j] = np.nextafter(np.nextafter(x[i], np.float32(2)), np.float32(2))
        y[j] = y[i]
        z[j] = z[i]
    return ic.Bodies(x, y, z, b.vx, b.vy, b.vz, b.m)


CASES = {
    "disk64": (lambda: ic.star_disk(64), False),
    "disk1000": (lambda: ic.star_disk(1000), False),
    "plummer2048": (lambda: ic.plummer(2048), True),
    "lattice867": (lattice, True),
    "deep1024": (deep_pairs, False),
    "disk16384": (lambda: ic.star_disk(16384), True),
}


def tight_bounds(bb):
    rad = 0.5 * float(bb[1] - bb[0]) * math.sqrt(1.5 / 0.25)
    return float(bb[0]), float(np.float32(bb[0]) + np.float32(2.0 * rad))


def make(name, gen, with_tight):
    b = gen()
    assert not ic.has_duplicates(b), name
    out = {}
    ref = O.ref_step(b.x, b.y, b.z, b.vx, b.vy, b.vz, b.m, DT)
    # the reference drops a body that is a direct child of the root (Kernels.cu:505-516)
    assert (ref["root_child"] == -1).sum() + (ref["root_child"] >= len(b.x)).sum() == 8, name
    for k in ("x", "y", "z", "vx", "vy", "vz", "m"):
        out["in_" + k] = getattr(b, k)
    for k in ("bbox", "perm", "root_child", "cell_child", "cell_start", "cell_count",
              "cell_level", "cell_x", "cell_y", "cell_z", "cell_m", "a"):
        out[k] = ref[k]
    for k, v in zip(("x", "y", "z", "vx", "vy", "vz"), ref["state"]):
        out["out_" + k] = v
    if with_tight:
        fb = tight_bounds(ref["bbox"])
        reft = O.ref_step(b.x, b.y, b.z, b.vx, b.vy, b.vz, b.m, DT, force_bounds=fb)
        out["tight_bounds"] = np.array(fb, np.float32)
        out["tight_a"] = reft["a"]
    out["dt"] = np.float32(DT)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    return path, len(b.x), ref["ncells"]


# Headless frames of the reference renderer (3D/CUDA/CUDA_NBody/src/Renderer.cpp,
# compiled from the checkout by oracle/build.py): inputs are regenerated from the
# seeded initial conditions, only the frame bytes are stored.
FRAMES = {
    # name: (generator, n, width, height, max_velocity_color, render_scale)
    "frame_disk4096": (ic.star_disk, 4096, 160, 128, 2.0, 2.5),
    "frame_plummer3000": (ic.plummer, 3000, 128, 128, 1.0, 1.0),
}


def frame_params(name):
    gen, n, w, h, vmax, scale = FRAMES[name]
    b = gen(n)
    p = O.RenderParams(width=w, height=h, render_scale=scale, max_velocity_color=vmax,
                       system_size=O.system_size(b.x, b.y, b.z))
    return b, p


def make_frames():
    for name in FRAMES:
        b, p = frame_params(name)
        rgb = O.ref_render(b.x, b.y, b.z, b.vx, b.vy, b.vz, p)
        if rgb is None:
            raise SystemExit("the reference renderer could not be built")
        np.savez_compressed(os.path.join(HERE, name + ".npz"), rgb=rgb)
        print(name, rgb.shape, int((rgb > 0).sum()), "lit bytes")


# Hilbert keys of the reference's own Lebesgue2Hilbert
# (MolecularDynamics/BarnesHutParallel/SpaceFillingCurves/src/Tree.cpp:90-104,
# compiled for the CPU by oracle/build.py): the 21-level keys of a seeded disk
# (converted to the MD code's child numbering) and random 63-bit keys.
def make_hilbert():
    b = ic.star_disk(4096)
    bb = O.bbox(b.x, b.y, b.z)
    hi, _ = O.keys(b.x, b.y, b.z, bb, 21)
    rnd = np.random.default_rng(20261203).integers(0, 2 ** 63, size=4096, dtype=np.uint64)
    leb = np.concatenate([O.md_key(hi), rnd])
    hil = O.ref_hilbert(leb)
    if hil is None:
        raise SystemExit("the reference SpaceFillingCurves code could not be built")
    path = os.path.join(HERE, "sfc_hilbert4096.npz")
    np.savez_compressed(path, n_disk=np.int64(len(b.x)), lebesgue_md=leb, hilbert=hil)
    print("sfc_hilbert4096", len(leb), "keys", "%.1f KB" % (os.path.getsize(path) / 1024))


def main():
    if O.ref_lib() is None:
        raise SystemExit("the reference checkout is needed to generate fixtures")
    if sys.argv[1:] == ["hilbert"]:
        make_hilbert()
        return
    make_hilbert()
    make_frames()
    for name, (gen, tight) in CASES.items():
        path, n, nc = make(name, gen, tight)
        print("%-14s n=%-6d cells=%-6d %7.1f KB" % (name, n, nc, os.path.getsize(path) / 1024))


if __name__ == "__main__":
    main()
