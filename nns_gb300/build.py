"""Build recipe of libnbx.so (the CUDA kernels and the C ABI) for sm_103a.

Each translation unit under ``csrc/`` is compiled by nvcc in parallel and the
objects are linked into ``nns_gb300/libnbx.so`` (in-tree; git-ignored).  No
torch, no cmake: plain nvcc, so the library has no torch types in its ABI.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.environ.get("NBX_BUILD_DIR", os.path.join(HERE, "_build"))
LIB = os.environ.get("NBX_LIB_PATH", os.path.join(HERE, "libnbx.so"))
# extra nvcc flags (e.g. -D tuning macros of csrc/walk2.cu) and a separate
# object directory, for building variants side by side
EXTRA = os.environ.get("NBX_NVCC_EXTRA", "").split()
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-Xptxas", "-v"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) +
                  glob.glob(os.path.join(HERE, "..", "include", "*.h")) +
                  glob.glob(os.path.join(HERE, "..", "include", "nbx", "*.hpp")) +
                  glob.glob(os.path.join(HERE, "driver", "*.cpp")))


def _compile(src: str) -> tuple[str, str]:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + EXTRA + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    if LIB == os.path.join(HERE, "libnbx.so") and not os.path.exists(os.path.join(HERE, "nbx_runner")):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _sources() + _headers())


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every kernel TU for sm_103a and link libnbx.so; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(_compile, srcs))
    if verbose:
        for (_, log) in results:
            print(log)
    with open(os.path.join(BUILD, "ptxas.log"), "w") as f:
        for src, (_, log) in zip(srcs, results):
            f.write("== %s\n%s\n" % (os.path.basename(src), log))
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    if LIB == os.path.join(HERE, "libnbx.so"):
        build_runner()
    return LIB


RUNNER = os.path.join(HERE, "nbx_runner")


def build_runner() -> str:
    """The command-line driver (driver/nbx_runner.cpp) linked against libnbx.so."""
    src = os.path.join(HERE, "driver", "nbx_runner.cpp")
    inc = os.path.join(HERE, "..", "include")
    cuda = os.path.dirname(os.path.dirname(nvcc()))
    cmd = ["g++", "-O2", "-std=c++17", "-I", inc, "-I", os.path.join(cuda, "include"), src, "-o", RUNNER,
           "-L", HERE, "-lnbx", "-Wl,-rpath,$ORIGIN", "-L", os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nbx_runner build failed:\n%s" % r.stderr[-3000:])
    return RUNNER


if __name__ == "__main__":
    print(build(force=True, verbose=False))
