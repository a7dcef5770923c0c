"""The reference's own driver relinked against libnbx (test infrastructure only).

``stage()`` copies the reference driver, 3D/CUDA/CUDA_NBody/src/main.cu, and the
application files it uses besides the Barnes-Hut path (Body, Logger, Renderer
and Timer sources and headers, Constants.h, cxxopts.h) into the git-ignored
``oracle/_ref/cuda_main/``, with ONE documented change: main.cu's two includes
of the reference's KernelsWrapper.cuh and BarnesHut.cuh point to libnbx's
drop-in headers (include/nbx/KernelsWrapper.cuh, include/nbx/BarnesHut.cuh).
Nothing else of main.cu changes: it constructs ``new BarnesHut(parameters)``,
calls ``update(i)``, reads ``h_x[i]`` and the ``time_*`` arrays and prints its
TIME report through the reference's Logger.

``build()`` compiles that staged tree with g++ against ``include/`` and links
it to ``nns_gb300/libnbx.so``: the proof that the reference's driver builds
against the drop-in.  The staged tree travels with the repository, so the GPU
host builds and runs it without the checkout.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF_ROOT = os.environ.get("NBX_REFERENCE_ROOT") or os.path.normpath(os.path.join(ROOT, os.pardir, "reference"))
REF_CUDA = os.path.join(REF_ROOT, "3D", "CUDA", "CUDA_NBody")
STAGE = os.path.join(HERE, "_ref", "cuda_main")
RUNNER = os.path.join(STAGE, "runner")
SOURCES = ("main.cu", "Body.cpp", "Logger.cpp", "Renderer.cpp", "Timer.cpp")
HEADERS = ("Body.h", "Constants.h", "Logger.h", "Renderer.h", "Timer.h", "cxxopts.h")
SWITCH = {'#include "../include/KernelsWrapper.cuh"': '#include "nbx/KernelsWrapper.cuh"',
          '#include "../include/BarnesHut.cuh"': '#include "nbx/BarnesHut.cuh"'}


def stage() -> bool:
    """Stage the driver from the checkout (where present); True when a staged tree exists."""
    if not os.path.isfile(os.path.join(REF_CUDA, "src", "main.cu")):
        return os.path.isfile(os.path.join(STAGE, "src", "main.cu"))
    for sub, names in (("src", SOURCES), ("include", HEADERS)):
        os.makedirs(os.path.join(STAGE, sub), exist_ok=True)
        for fn in names:
            shutil.copy(os.path.join(REF_CUDA, sub, fn), os.path.join(STAGE, sub, fn))
    p = os.path.join(STAGE, "src", "main.cu")
    text = open(p).read()
    for old, new in SWITCH.items():
        if old not in text:
            raise RuntimeError("main.cu no longer has the line %r" % old)
        text = text.replace(old, new)
    open(p, "w").write(text)
    return True


def build() -> str | None:
    """Compile the staged driver against include/ and link libnbx.so (None when
    nothing is staged)."""
    if not stage():
        return None
    from nns_gb300 import build as nb
    lib = nb.build()
    cuda = os.path.dirname(os.path.dirname(nb.nvcc()))
    srcs = [os.path.join(STAGE, "src", f) for f in SOURCES]
    newest = max(os.path.getmtime(f) for f in srcs + [lib] + nb._headers())
    if os.path.exists(RUNNER) and os.path.getmtime(RUNNER) >= newest:
        return RUNNER
    cmd = ["g++", "-O2", "-std=c++17", "-w", "-I", os.path.join(STAGE, "include"), "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), "-x", "c++", srcs[0], "-x", "none"] + srcs[1:] + \
        ["-o", RUNNER, "-L", os.path.dirname(lib), "-lnbx", "-Wl,-rpath," + os.path.dirname(lib),
         "-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference driver build against libnbx failed:\n" + r.stderr[-4000:])
    return RUNNER
