"""Build recipe for the parity oracle (test infrastructure only).

* ``oracle/liboracle.so`` -- the C restatement ``refemu.c`` (always built).
* ``oracle/_ref/libref_kernels.so`` -- the reference's own CUDA kernel source
  (3D/CUDA/CUDA_NBody/src/Kernels.cu) compiled unmodified with g++ against the
  CPU stand-in ``ref_shim/cuda.h``.  Built only where the reference checkout is
  present; its outputs go to ``oracle/_ref/`` only.
* ``oracle/_ref/libref_render.so`` -- the reference's renderer
  (3D/CUDA/CUDA_NBody/src/Renderer.cpp, Body.cpp, Logger.cpp) with the C entry
  point ``ref_shim/render_harness.cpp``, for the headless-frame parity.
* ``oracle/_ref/libref_sfc.so`` -- the reference's SpaceFillingCurves tree code
  (MolecularDynamics/BarnesHutParallel/SpaceFillingCurves/src/Tree.cpp) against the
  single-process ``ref_shim/mpi.h``, for its Lebesgue-to-Hilbert key conversion.
* ``oracle/_ref/omp/`` -- the reference's 3D/OpenMP tree code, staged from the
  checkout (see ``ref_cpu.py``) and compiled against a harness for the timed
  CPU baseline.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout: NBX_REFERENCE_ROOT, else a directory named
# "reference" beside the repository.  Where neither exists the recipes build
# only what needs no checkout.
REF_ROOT = os.environ.get("NBX_REFERENCE_ROOT") or os.path.join(
    os.path.dirname(os.path.dirname(os.path.abspath(__file__))), os.pardir, "reference")
REF_ROOT = os.path.normpath(REF_ROOT)
REF_CUDA = os.path.join(REF_ROOT, "3D", "CUDA", "CUDA_NBody")
REF_SFC = os.path.join(REF_ROOT, "MolecularDynamics", "BarnesHutParallel", "SpaceFillingCurves")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def build_oracle() -> str:
    out = os.path.join(HERE, "liboracle.so")
    src = os.path.join(HERE, "refemu.c")
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
              src, "-o", out, "-lm"])
    return out


def reference_present() -> bool:
    return os.path.isfile(os.path.join(REF_CUDA, "src", "Kernels.cu"))


def build_ref_kernels() -> str | None:
    """Compile the reference kernels for the CPU (only where the checkout exists)."""
    if not reference_present():
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libref_kernels.so")
    shim = os.path.join(HERE, "ref_shim")
    srcs = [os.path.join(shim, "fiber.cpp"), os.path.join(shim, "ref_harness.cpp")]
    newest = max(os.path.getmtime(s) for s in srcs + [os.path.join(shim, "cuda.h")])
    if os.path.exists(out) and os.path.getmtime(out) >= newest:
        return out
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
          "-I", shim, "-I", os.path.join(REF_CUDA, "include"),
          "-x", "c++", os.path.join(REF_CUDA, "src", "Kernels.cu"), "-x", "none"] + srcs
         + ["-o", out])
    return out


def build_ref_renderer() -> str | None:
    """Compile the reference's renderer sources with a C entry point (only where
    the checkout exists)."""
    if not reference_present():
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libref_render.so")
    harness = os.path.join(HERE, "ref_shim", "render_harness.cpp")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(harness):
        return out
    srcs = [os.path.join(REF_CUDA, "src", f) for f in ("Renderer.cpp", "Body.cpp", "Logger.cpp")]
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
          "-I", os.path.join(REF_CUDA, "include")] + srcs + [harness, "-o", out])
    return out


def build_ref_sfc() -> str | None:
    """Compile the reference's SpaceFillingCurves tree code (Tree.cpp with the
    Logger, Particle and Domain sources it needs) for the CPU against the
    single-process ref_shim/mpi.h, with the C entry point
    ref_shim/sfc_harness.cpp (only where the checkout exists)."""
    if not os.path.isfile(os.path.join(REF_SFC, "src", "Tree.cpp")):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libref_sfc.so")
    shim = os.path.join(HERE, "ref_shim")
    harness = os.path.join(shim, "sfc_harness.cpp")
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(harness),
                                                            os.path.getmtime(os.path.join(shim, "mpi.h"))):
        return out
    srcs = [os.path.join(REF_SFC, "src", f) for f in ("Tree.cpp", "Logger.cpp", "Particle.cpp", "Domain.cpp")]
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-w", "-Wl,--no-undefined", "-I", shim,
          "-I", os.path.join(REF_SFC, "include")] + srcs + [harness, "-o", out])
    return out


def build_all() -> None:
    build_oracle()
    build_ref_kernels()
    build_ref_renderer()
    build_ref_sfc()
    from . import ref_cpu  # noqa: WPS433 -- staged reference CPU code
    ref_cpu.build()


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(HERE))
    from oracle import build as _b  # noqa

    _b.build_all()
    print("oracle built")
