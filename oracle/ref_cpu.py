"""The reference's 3D/OpenMP and 3D/Serial tree codes as the timed CPU baselines.

TEST/BASELINE INFRASTRUCTURE ONLY.  ``stage()`` copies the reference's own
sources (3D/OpenMP/OpenMP_NBody/src and include, minus the boost-dependent
main.cpp / ConfigParser.cpp and the renderer) into the git-ignored
``oracle/_ref/omp/`` and applies two documented changes:
  * include/Constants.h is replaced by a shim with G = dt^2, TO_METERS = 1
    (units of oracle/ref_shim/omp_harness.cpp);
  * Interaction.cpp:130 initialises the bounding box it otherwise reads
    uninitialised (`double xMin, ..., zMax = 0;`).
The staged tree travels with the repository to the GPU host, where ``build()``
compiles it (g++ -O3 -fopenmp) together with the harness.  ``stage_serial()``
does the same for 3D/Serial/NBody into ``oracle/_ref/serial/`` (Constants.h
replaced by a shim with the same units), timed on one thread.
"""
from __future__ import annotations

import json
import os
import re
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout: NBX_REFERENCE_ROOT, else a directory named
# "reference" beside the repository.  Where neither exists the recipes build
# only what needs no checkout.
REF_ROOT = os.environ.get("NBX_REFERENCE_ROOT") or os.path.join(
    os.path.dirname(os.path.dirname(os.path.abspath(__file__))), os.pardir, "reference")
REF_ROOT = os.path.normpath(REF_ROOT)
REF_OMP = os.path.join(REF_ROOT, "3D", "OpenMP", "OpenMP_NBody")
STAGE = os.path.join(HERE, "_ref", "omp")
RUNNER = os.path.join(STAGE, "runner")
HARNESS = os.path.join(HERE, "ref_shim", "omp_harness.cpp")
SKIP = {"main.cpp", "ConfigParser.cpp", "Renderer.cpp", "InitializeDistribution.cpp"}

CONSTANTS_SHIM = """#ifndef CONSTANTS_H_
#define CONSTANTS_H_
/* staged shim: G = dt^2 and TO_METERS = 1 make one reference step one
 * kick-drift step of length dt with G = 1 (see omp_harness.cpp, which sets G
 * from the NBX_REF_DT environment variable, default NBX_DT) */
#ifndef NBX_DT
#define NBX_DT 5e-4
#endif
const double PI = 3.14159265358979323846;
const double TO_METERS = 1.0;
extern double G;
extern int NUM_BODIES;
extern int NUM_SUNS;
extern double SYSTEM_SIZE;
extern double SYSTEM_THICKNESS;
extern double INNER_BOUND;
extern double SOFTENING;
extern double SOLAR_MASS;
extern double EXTRA_MASS;
extern double MAX_DISTANCE;
extern int TIME_STEP;
extern int STEP_COUNT;
extern bool BINARY;
extern double BINARY_SEPARATION;
#define DEBUG_INFO false
#endif
"""


REF_SERIAL = os.path.join(REF_ROOT, "3D", "Serial", "NBody")
STAGE_SERIAL = os.path.join(HERE, "_ref", "serial")
RUNNER_SERIAL = os.path.join(STAGE_SERIAL, "runner")
HARNESS_SERIAL = os.path.join(HERE, "ref_shim", "serial_harness.cpp")

SERIAL_CONSTANTS_SHIM = """#ifndef CONSTANTS_H_
#define CONSTANTS_H_
/* staged shim for 3D/Serial: G = dt^2 and TO_METERS = 1 make one reference
 * step one kick-drift step of length dt with G = 1 (see serial_harness.cpp) */
#ifndef NBX_DT
#define NBX_DT 5e-4
#endif
const double PI = 3.14159265358979323846;
const double TO_METERS = 1.0;
extern double G;  /* dt^2 for timed steps, 1 for force checks (set by the harness) */
extern int NUM_BODIES;
extern int NUM_SUNS;
extern double SYSTEM_SIZE;
extern double SOFTENING;
extern double MAX_DISTANCE;
const int TIME_STEP = 1;
#define DEBUG_INFO false
#endif
"""


def stage_serial() -> bool:
    """Copy the reference's 3D/Serial sources into oracle/_ref/serial."""
    if not os.path.isdir(REF_SERIAL):
        return os.path.isdir(os.path.join(STAGE_SERIAL, "src"))
    for sub in ("src", "include"):
        d = os.path.join(STAGE_SERIAL, sub)
        os.makedirs(d, exist_ok=True)
        for fn in os.listdir(os.path.join(REF_SERIAL, sub)):
            if fn in SKIP:
                continue
            shutil.copy(os.path.join(REF_SERIAL, sub, fn), os.path.join(d, fn))
    with open(os.path.join(STAGE_SERIAL, "include", "Constants.h"), "w") as f:
        f.write(SERIAL_CONSTANTS_SHIM)
    return True


def build_serial(dt: float = 5e-4) -> str | None:
    if not stage_serial():
        return None
    srcs = sorted(os.path.join(STAGE_SERIAL, "src", f) for f in os.listdir(os.path.join(STAGE_SERIAL, "src"))
                  if f.endswith(".cpp"))
    stamp = os.path.join(STAGE_SERIAL, "dt.txt")
    newest = max(os.path.getmtime(x) for x in srcs + [HARNESS_SERIAL])
    if (os.path.exists(RUNNER_SERIAL) and os.path.getmtime(RUNNER_SERIAL) >= newest and os.path.exists(stamp)
            and open(stamp).read() == repr(dt)):
        return RUNNER_SERIAL
    cmd = ["g++", "-O3", "-std=c++14", "-DNBX_DT=%r" % dt, "-I", os.path.join(STAGE_SERIAL, "include"),
           HARNESS_SERIAL] + srcs + ["-o", RUNNER_SERIAL]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference Serial build failed:\n" + r.stderr[-3000:])
    open(stamp, "w").write(repr(dt))
    return RUNNER_SERIAL


def stage() -> bool:
    """Copy the reference sources into oracle/_ref/omp (only where the checkout exists)."""
    if not os.path.isdir(REF_OMP):
        return os.path.isdir(os.path.join(STAGE, "src"))
    for sub in ("src", "include"):
        d = os.path.join(STAGE, sub)
        os.makedirs(d, exist_ok=True)
        for fn in os.listdir(os.path.join(REF_OMP, sub)):
            if fn in SKIP or fn.startswith("cxxopts") or fn.startswith("ConfigParser"):
                continue
            shutil.copy(os.path.join(REF_OMP, sub, fn), os.path.join(d, fn))
    with open(os.path.join(STAGE, "include", "Constants.h"), "w") as f:
        f.write(CONSTANTS_SHIM)
    p = os.path.join(STAGE, "src", "Interaction.cpp")
    s = open(p).read()
    s2 = re.sub(r"double xMin, xMax, yMin, yMax, zMin, zMax = 0;",
                "double xMin = 0, xMax = 0, yMin = 0, yMax = 0, zMin = 0, zMax = 0;", s)
    open(p, "w").write(s2)
    return True


def build(dt: float = 5e-4) -> str | None:
    """Compile the staged OpenMP code with the harness (dt is set per run through
    NBX_REF_DT, so one build serves every configuration)."""
    del dt
    if not stage():
        return None
    srcs = sorted(os.path.join(STAGE, "src", f) for f in os.listdir(os.path.join(STAGE, "src"))
                  if f.endswith(".cpp"))
    newest = max(os.path.getmtime(x) for x in srcs + [HARNESS, os.path.join(STAGE, "include", "Constants.h")])
    if os.path.exists(RUNNER) and os.path.getmtime(RUNNER) >= newest:
        return RUNNER
    cmd = ["g++", "-O3", "-std=c++14", "-fopenmp", "-I", os.path.join(STAGE, "include"), HARNESS] + srcs \
        + ["-o", RUNNER]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference OpenMP build failed:\n" + r.stderr[-3000:])
    return RUNNER


def _write_input(path, b, theta, eps, dt):
    n = len(b.x)
    with open(path, "wb") as f:
        np.array([n], np.int32).tofile(f)
        np.array([theta, eps], np.float32).tofile(f)
        for a in (b.x, b.y, b.z):
            np.asarray(a, np.float32).tofile(f)
        for a in (b.vx, b.vy, b.vz):
            (np.asarray(a, np.float64) * dt).astype(np.float32).tofile(f)
        np.asarray(b.m, np.float32).tofile(f)


def run(b, theta, eps, dt, steps, warmup, mode="sample", k=65536, threads=None, seed=1, code="omp"):
    runner = build(dt) if code == "omp" else build_serial(dt)
    if runner is None:
        return None
    env = dict(os.environ)
    env["NBX_REF_DT"] = repr(float(dt))
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    with tempfile.TemporaryDirectory() as td:
        inp = os.path.join(td, "in.bin")
        _write_input(inp, b, theta, eps, dt)
        args = [runner, mode, inp, str(steps), str(warmup)]
        if mode == "sample":
            args += [str(k), str(seed)]
        r = subprocess.run(args, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError("reference runner failed: %s" % r.stderr[-2000:])
    out = r.stdout[r.stdout.index("{"):]
    return json.loads(out)


def _workload(n):
    from nns_gb300 import ic
    return ic.binary_disk(n)


def bench_openmp(n, steps, warmup, theta, eps, dt, k=16384, b=None):
    """The n/k model of a reference OpenMP step (an extrapolation, not a
    measured step): the full tree is built once (serially, as the reference
    does) and its time charged to every step; each step runs the reference's
    parallel force loop on k random bodies and its update; step time = build +
    force * n / k + update."""
    b = _workload(n) if b is None else b
    res = run(b, theta, eps, dt, steps, max(0, min(warmup, 1)), "sample", k)
    if res is None:
        return None
    per = [sum(s) for s in res["steps"]]
    t = float(np.median(per))
    return {"steps_per_s": 1.0 / t, "cores": res["threads"], "extrapolated": True, "k": k, "n_over_k": n / k,
            "sample": "reference serial tree build over all %d bodies (timed once) + per step "
                      "the reference OpenMP force loop over %d random bodies scaled by n/k + "
                      "update; median of %d steps" % (n, k, len(per)),
            "phases_s": {"build": float(np.median([s[0] for s in res["steps"]])),
                         "force_scaled": float(np.median([s[1] for s in res["steps"]])),
                         "update": float(np.median([s[2] for s in res["steps"]]))}}


def full_openmp(b, theta, eps, dt, steps):
    """Whole, unsampled reference OpenMP steps (Interaction::interactBodies: tree
    build, parallel force loop over every body, update), timed per step."""
    res = run(b, theta, eps, dt, steps, 0, "full")
    if res is None:
        return None
    per = [float(sum(s)) for s in res["steps"]]
    return {"steps": len(per), "s_per_step": per, "median_s_per_step": float(np.median(per)),
            "steps_per_s": 1.0 / float(np.median(per)), "cores": res["threads"], "n": len(b.x)}


def reference_arm(n, theta, eps, dt, k=16384):
    """The reference arm: whole reference OpenMP steps, measured.

    * the benchmark workload (binary star + disk of n bodies): one whole step;
    * the n/k model of the same step (k sampled bodies), with its error against
      the measured step;
    * config 0 (star + disk, 16384 bodies, theta 0.5, eps 0.01, dt 1e-3): all 10
      steps;
    * config 1 (Plummer, 2^20 bodies, theta 0.6, eps 0.005, dt 1e-3): one step.
    """
    from nns_gb300 import ic
    b = _workload(n)
    full = full_openmp(b, theta, eps, dt, 1)
    if full is None:
        return None
    model = bench_openmp(n, 1, 0, theta, eps, dt, k, b=b)
    del b
    t_full = full["median_s_per_step"]
    t_model = 1.0 / model["steps_per_s"]
    c0 = full_openmp(ic.star_disk(16384), 0.5, 0.01, 1e-3, 10)
    c1 = full_openmp(ic.plummer(1 << 20), 0.6, 0.005, 1e-3, 1)
    return {"full": full, "model": dict(model, rel_error_vs_full=(t_model - t_full) / t_full),
            "config0_star_disk_16384": c0, "config1_plummer_2^20": c1}


def bench_serial(n, theta, eps, dt, k=1024, steps=1):
    """The reference's 3D/Serial code on one core: serial tree build over all
    bodies (timed once) + per step its force loop over k random bodies scaled by
    n/k + its update."""
    b = _workload(n)
    res = run(b, theta, eps, dt, steps, 0, "sample", k, code="serial")
    if res is None:
        return None
    per = [sum(x) for x in res["steps"]]
    return {"value": 1.0 / float(np.median(per)), "unit": "steps/s", "cores": 1, "kind": "reference",
            "sample": "reference 3D/Serial: tree build over all %d bodies (timed once) + force loop over %d "
                      "random bodies scaled by n/k + update, one thread" % (n, k),
            "phases_s": {"build": float(np.median([x[0] for x in res["steps"]])),
                         "force_scaled": float(np.median([x[1] for x in res["steps"]])),
                         "update": float(np.median([x[2] for x in res["steps"]]))}}


def serial_forces(b, theta, eps):
    """Accelerations (n, 3) of the reference's 3D/Serial tree code with G = 1
    (its MAC length/|d| < theta and softening (d^2+eps^2) d), or None where the
    code is not staged."""
    runner = build_serial()
    if runner is None:
        return None
    n = len(b.x)
    with tempfile.TemporaryDirectory() as td:
        inp, out = os.path.join(td, "in.bin"), os.path.join(td, "acc.bin")
        _write_input(inp, b, theta, eps, 1.0)
        r = subprocess.run([runner, "forces", inp, out], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference serial runner failed: %s" % r.stderr[-2000:])
        return np.fromfile(out, np.float64).reshape(n, 3)


def cpu_baseline(n, theta, eps, dt, k=4096):
    """One bounded sample (one step of the n/k model) for the cpu_baseline key of
    the GPU arm; the measured whole step is the reference arm's."""
    r = bench_openmp(n, 1, 0, theta, eps, dt, k)
    if r is None:
        return {"unavailable": "reference CPU code not staged on this host"}
    return {"value": r["steps_per_s"], "unit": "steps/s", "cores": r["cores"], "kind": "reference",
            "extrapolated": True, "k": k, "n_over_k": n / k, "sample": r["sample"], "phases_s": r["phases_s"]}
