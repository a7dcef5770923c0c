"""Benchmark: 16M-body Barnes-Hut steps/s on one GB300 (plain vs compensated FP32).

Workload (the precision-form configuration): binary star + disk, N = 2^24,
two 0.5-mass stars at separation 0.2, 2^24-2 disk bodies of mass 1e-8 with
radius U[0.3,2], theta = 0.5, eps = 0.005, dt = 5e-4.  Synthetic inputs from the
counter-based generator in nns_gb300.ic.  A step is one full pass of the hot
path: bounding box, keys, key sort, tree, moments, warp-coherent walk and
kick-drift.  The inputs (2^24 bodies: 0.7 GB of state plus 4 GB of tree) are far
larger than L2, so no flush is needed between steps.

Prints one JSON line (see README section "bench contract").
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "16M-body BH steps/s, plain vs compensated FP32 @1e-4 err; adjoint/fwd cost"
N_DEFAULT = 1 << 24
THETA, EPS, DT = 0.5, 0.005, 5e-4
RUN_STEPS = 20  # the precision form's run length: energy drift is reported over it
FLOP_PER_INTERACTION = 20


def workload_config(n, world):
    return {"workload": "binary_disk_2^24 precision form", "n": n, "theta": THETA, "eps": EPS,
            "dt": DT, "group": 32, "l2": "inputs larger than L2 (no flush)",
            "parallelism": ("key-range split of one system over %d GPUs" % world) if world > 1 else "single"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="nbx", choices=["nbx", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--targets", type=int, default=8192)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--batched-systems", type=int, default=512)
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-hilbert", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-buckets", action="store_true")
    ap.add_argument("--no-configs", action="store_true")
    ap.add_argument("--fd-directions", type=int, default=16)
    ap.add_argument("--adjoint-steps", type=int, default=100)
    ap.add_argument("--adjoint-checkpoint", type=int, default=10)
    ap.add_argument("--only", choices=["batched", "adjoint"], default=None,
                    help="run one extension section alone and print its JSON object")
    return ap.parse_args()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), \
        int(os.environ.get("LOCAL_RANK", 0))


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = float(f[2])
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        finally:
            os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def peak_fp32_tflops(nsm: int, mhz: float) -> float:
    return nsm * 128 * 2 * mhz * 1e6 / 1e12


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        return {}


def run_reference(args, rank):
    """CPU reference arm: the reference's own 3D/OpenMP tree code on all host
    cores, whole unsampled steps (tree build, force loop over every body,
    update).  One whole step of the 2^24 workload takes one to two minutes, so
    the arm times one such step whatever --steps/--warmup ask (recorded under
    "requested"), then the n/k model of the same step with its measured error,
    and whole steps of the 16384-body (10 steps) and 2^20-body (1 step) configs."""
    if rank != 0:
        return None
    from oracle import ref_cpu
    res = ref_cpu.reference_arm(args.n, THETA, EPS, DT)
    if res is None:
        return {"impl": "reference", "unavailable": "reference CPU code was not staged/built on this host"}
    full = res["full"]
    v = full["steps_per_s"]
    line = {"metric": METRIC, "impl": "reference", "value": v, "unit": "steps/s",
            "n_gpus": int(os.environ.get("WORLD_SIZE", args.gpus)), "steps": full["steps"], "warmup": 0,
            "ms_per_step": 1000.0 * full["median_s_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (nns_gb300.ic binary_disk)",
            "config": workload_config(args.n, int(os.environ.get("WORLD_SIZE", 1))),
            "requested": {"steps": args.steps, "warmup": args.warmup},
            "cpu_baseline": {"value": v, "unit": "steps/s", "cores": full["cores"], "kind": "reference",
                             "extrapolated": False,
                             "sample": "%d whole reference OpenMP step(s) of all %d bodies (Interaction::"
                                       "interactBodies), unsampled" % (full["steps"], args.n)},
            "model": res["model"],
            "configs": {"star_disk_16384": res["config0_star_disk_16384"],
                        "plummer_2^20": res["config1_plummer_2^20"]},
            "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    return line


def bench_batched(args, local):
    """Batched form: independent star+disk systems (N_i = floor(2^U[10,17]), seed
    20261203+1+i), theta 0.5, eps 0.01, dt 1e-3, all systems in one launch per phase,
    each step replayed from a CUDA graph; against the same systems stepped one
    at a time through single-system contexts with the same kernels."""
    import torch
    from nns_gb300 import autotune, ic
    from nns_gb300.barnes_hut import Context, State
    bodies, off = ic.batched_star_disks(args.batched_systems)
    rank, world, _ = dist_info()
    nsys_all = len(off) - 1
    if world > 1:
        # several ranks: each steps its own contiguous share of the systems (no exchange)
        from nns_gb300.dist import shard_systems
        s0, s1, loc = shard_systems(off, rank, world)
        a0, a1 = int(off[s0]), int(off[s1])
        bodies = ic.Bodies(*(arr[a0:a1] for arr in bodies.arrays()))
        off = loc
    nsys = len(off) - 1
    ntot = int(off[-1])
    ctx = Context(max_bodies=ntot, max_systems=nsys, theta=0.5, eps=0.01, dt=1e-3, device=local)
    ctx.set_systems(off)
    s = State.from_bodies(bodies, device="cuda:%d" % local)
    tune = autotune.tune_walk(ctx, s, use_cache=False)
    # per-system forces of the batch against single-system runs of every system
    # (bit for bit); the single-system contexts are then timed one at a time
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    accb = s.acc()
    ctxs, states = [], []
    for i in range(nsys):
        a, b = int(off[i]), int(off[i + 1])
        sub = ic.Bodies(*(arr[a:b] for arr in bodies.arrays()))
        c1 = Context(max_bodies=b - a, theta=0.5, eps=0.01, dt=1e-3, device=local)
        # the same walk configuration: the launch shape, buffer width and stack depth
        # set the order of the force sums (not the lists)
        c1.set_walk(tune["warps"], tune["variant"])
        c1.set_tuning(tune["radix_bits"], tune["stack_depth"])
        c1.set_systems([0, b - a])
        ctxs.append(c1)
        states.append(State.from_bodies(sub, device="cuda:%d" % local))
    equal = 0
    for i, (c1, s1) in enumerate(zip(ctxs, states)):
        c1.build(s1)
        c1.forces(s1)
        c1.sync()
        equal += bool(np.array_equal(accb[int(off[i]):int(off[i + 1])], s1.acc()))
    steps = max(2, args.steps)
    ctx.graph_step(s, max(1, args.warmup))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    ctx.graph_step(s, steps)
    e1.record()
    torch.cuda.synchronize()
    ctx.sync()
    t_batch = e0.elapsed_time(e1) / steps
    inter = ctx.tree_info()["interactions"]
    if world > 1:
        from nns_gb300.dist import max_over_ranks, sum_over_ranks
        t_batch = max_over_ranks(t_batch, device="cuda")
        inter = int(sum_over_ranks(float(inter), device="cuda"))
    # one system at a time (eager launches, one context per system)
    for c1, s1 in zip(ctxs, states):
        c1.step(s1, 1)
    torch.cuda.synchronize()
    single_steps = 2
    e0.record()
    for _ in range(single_steps):
        for c1, s1 in zip(ctxs, states):
            c1.step(s1, 1)
    e1.record()
    torch.cuda.synchronize()
    t_single = e0.elapsed_time(e1) / single_steps
    # the same, each system replayed from its own captured graph (on a side
    # stream, so no call synchronises): the strongest single-system usage
    gs = torch.cuda.Stream()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(gs):
        for c1, s1 in zip(ctxs, states):
            c1.graph_step(s1, 1, stream=gs)  # capture, then one step
        gs.synchronize()
        g0.record(gs)
        for _ in range(single_steps):
            for c1, s1 in zip(ctxs, states):
                c1.graph_step(s1, 1, stream=gs)
        g1.record(gs)
    torch.cuda.synchronize()
    t_single_graph = g0.elapsed_time(g1) / single_steps
    return {"systems": nsys_all, "bodies": ntot, "steps": steps, "ranks": world,
            "ms_per_step": round(t_batch, 3),
            "systems_steps_per_s": round(nsys_all * 1000.0 / t_batch, 2),
            "one_at_a_time_ms_per_step": round(t_single, 3),
            "one_at_a_time_systems_steps_per_s": round(nsys * 1000.0 / t_single, 2),
            "speedup_vs_one_at_a_time": round(t_single / t_batch, 3),  # this rank's systems
            "one_at_a_time_graphs_ms_per_step": round(t_single_graph, 3),
            "speedup_vs_one_at_a_time_graphs": round(t_single_graph / t_batch, 3),
            "interactions_per_step": inter,
            "per_system_forces_bitwise_equal_unbatched": {"systems_checked": nsys, "equal": equal},
            "walk_config": {k: tune[k] for k in ("warps", "variant", "stack_depth", "radix_bits")}}


def bench_adjoint(args, local):
    """Differentiation form: Plummer N=65536, theta 0.5, eps 0.01, dt 1e-3, 100 steps,
    L = sum |x(T) - x*|^2 with x* = x(T) + N(0, 0.01^2); checkpoints every 10 steps.
    Reports adjoint/forward time, device memory, and the gradient error against
    FP64 central finite differences (h = 1e-6) of the FP64 replay of the same
    trajectory (recorded interaction lists) along random unit directions."""
    import torch
    from nns_gb300 import ic
    from nns_gb300.adjoint import Adjoint, random_directions
    from nns_gb300.barnes_hut import Context, State
    n, T, C = 65536, args.adjoint_steps, args.adjoint_checkpoint
    b = ic.plummer(n)
    ctx = Context(max_bodies=n, theta=0.5, eps=0.01, dt=1e-3, device=local)
    ctx.set_systems([0, n])
    s = State.from_bodies(b, device="cuda:%d" % local)
    ctx.step(s, T)
    ctx.sync()
    rng = np.random.default_rng(20261203)
    xt = np.stack([t.cpu().numpy() for t in (s.x, s.y, s.z)])
    target = torch.as_tensor((xt + 0.01 * rng.standard_normal(xt.shape)).astype(np.float32),
                             device="cuda:%d" % local)
    free0 = torch.cuda.mem_get_info(local)[0]
    adj = Adjoint(ctx, T, C, 8192, C)
    times = []
    for _ in range(2):  # the second run is timed warm
        s = State.from_bodies(b, device="cuda:%d" % local)
        loss = adj.forward(s, target)
        gx, gv, gm = adj.backward(s)
        st = adj.stats()
        times.append((st["forward_ms"], st["backward_ms"]))
    free1 = torch.cuda.mem_get_info(local)[0]
    fwd_ms, bwd_ms = times[-1]
    g = np.concatenate([gx.cpu().numpy(), gv.cpu().numpy(), gm.cpu().numpy()[None]]).astype(np.float64)
    out = {"n": n, "steps": T, "checkpoint_every": C, "loss": loss,
           "forward_ms_per_step": round(fwd_ms / T, 3), "adjoint_ms_per_step": round(bwd_ms / T, 3),
           "adjoint_to_forward_ratio": round(bwd_ms / fwd_ms, 3),
           "adjoint_device_bytes": st["bytes"],
           "device_bytes_in_use_delta": int(free0 - free1)}
    del adj
    torch.cuda.empty_cache()
    if args.fd_directions > 0:
        ver = Adjoint(ctx, T, C, 8192, T)
        s = State.from_bodies(b, device="cuda:%d" % local)
        ver.forward(s, target)
        ver.record(State.from_bodies(b, device="cuda:%d" % local))
        base = np.stack([b.x, b.y, b.z, b.vx, b.vy, b.vz, b.m]).astype(np.float64)
        dev = lambda a: torch.as_tensor(a, device="cuda:%d" % local)  # noqa: E731
        loss64 = ver.replay_fp64(dev(base))
        h = 1e-6
        gn = float(np.linalg.norm(g))
        errs = []
        for u in random_directions(n, args.fd_directions):
            fd = (ver.replay_fp64(dev(base + h * u)) - ver.replay_fp64(dev(base - h * u))) / (2 * h)
            errs.append(abs(fd - float((g * u).sum())) / gn)
        out["fd_check"] = {"directions": args.fd_directions, "h": h,
                           "max_err_over_grad_norm": float(max(errs)),
                           "median_err_over_grad_norm": float(np.median(errs)),
                           "loss_fp64_replay": loss64,
                           "loss_rel_diff_fp32_vs_fp64": abs(loss64 - loss) / loss}
        del ver
        torch.cuda.empty_cache()
    return out


def bench_hilbert(args, local, b, targets, acc64, tune) -> dict:
    """The same workload with Hilbert-ordered keys (nbx_params.key_order = 1):
    the same cells with siblings reordered, so the walk groups are more
    compact.  Not the parity mode: its interaction lists are not the
    reference's.  Plain FP32 steps from the initial state."""
    import torch
    from nns_gb300.barnes_hut import Context, State
    n = len(b.x)
    ctx = Context(max_bodies=n, theta=THETA, eps=EPS, dt=DT, device=local, key_order=1)
    if tune:
        ctx.set_walk(tune["warps"], tune["variant"])
    ctx.set_systems([0, n])
    s = State.from_bodies(b, device="cuda:%d" % local)
    ctx.build(s)
    ctx.forces(s)
    ctx.sync()
    a = s.acc()[targets].astype(np.float64)
    rel = np.linalg.norm(a - acc64, axis=1) / np.linalg.norm(acc64, axis=1)
    for _ in range(args.warmup):
        ctx.step(s)
    k = max(3, min(args.steps, 5))
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(k)]
    torch.cuda.synchronize()
    for e in ev:
        e[0].record()
        ctx.build(s)
        e[1].record()
        ctx.forces(s)
        e[2].record()
        ctx.integrate(s)
        e[3].record()
    torch.cuda.synchronize()
    info = ctx.tree_info()
    ctx.sync()
    ms = sum(e[0].elapsed_time(e[3]) for e in ev) / k
    return {"value": round(1000.0 / ms, 4), "unit": "steps/s", "ms_per_step": round(ms, 3), "steps": k,
            "phase_ms": {"build": round(sum(e[0].elapsed_time(e[1]) for e in ev) / k, 3),
                         "walk": round(sum(e[1].elapsed_time(e[2]) for e in ev) / k, 3),
                         "integrate": round(sum(e[2].elapsed_time(e[3]) for e in ev) / k, 3)},
            "interactions_per_step": info["interactions"],  # counters restart at every build
            "force_error_vs_fp64_direct": {"median": float(np.median(rel)),
                                           "p99": float(np.quantile(rel, 0.99)), "max": float(rel.max())},
            "note": "key_order=1: same cells and MAC, Hilbert sibling order; the walk groups and so the "
                    "interaction lists differ from the reference's (not the parity mode)"}


# the other single-system configurations: name, bodies, theta, eps, dt, steps
OTHER_CONFIGS = (("star_disk_16384", "star_disk", 16384, 0.5, 0.01, 1e-3, 10),
                 ("plummer_2^20", "plummer", 1 << 20, 0.6, 0.005, 1e-3, 100))


def bench_configs(args, local, tune) -> dict:
    """The other single-system configurations at their own theta, eps, dt and
    step counts (the reference arm times whole steps of the same two): the
    16384-body star + disk (10 steps) and the 2^20-body Plummer sphere (100
    steps).  Per configuration: the force error against the FP64 direct sum on
    4096 random targets at the initial state; all its steps replayed from one
    CUDA graph, timed with CUDA events after one warm-up replay (steps/s); and
    three eager steps with per-phase events for the walk's FP32 fraction."""
    import torch
    from nns_gb300 import ic
    from nns_gb300.barnes_hut import Context, State
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    peaks = measured_peaks()
    peak = peak_fp32_tflops(nsm, peaks.get("sm_max_mhz") or 2070.0)
    out = {}
    for name, kind, n, theta, eps, dt, steps in OTHER_CONFIGS:
        b = getattr(ic, kind)(n)
        ctx = Context(max_bodies=n, theta=theta, eps=eps, dt=dt, device=local)
        if tune:
            ctx.set_walk(tune["warps"], tune["variant"])
        ctx.set_systems([0, n])
        s = State.from_bodies(b, device="cuda:%d" % local)
        eps2 = float(np.float32(eps) * np.float32(eps))
        targets = np.sort(np.random.default_rng(12345).choice(n, size=min(4096, n), replace=False))
        acc64 = ctx.direct_fp64(s, targets, eps2).cpu().numpy()
        ctx.build(s)
        ctx.forces(s)
        ctx.sync()
        a = s.acc()[targets].astype(np.float64)
        rel = np.linalg.norm(a - acc64, axis=1) / np.linalg.norm(acc64, axis=1)
        ctx.graph_step(s, steps)  # warm-up replay (captures the graph)
        ctx.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        ctx.graph_step(s, steps)
        e1.record()
        torch.cuda.synchronize()
        ctx.sync()
        ms = e0.elapsed_time(e1) / steps
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(3)]
        torch.cuda.synchronize()
        for e in ev:
            e[0].record()
            ctx.build(s)
            e[1].record()
            ctx.forces(s)
            e[2].record()
            ctx.integrate(s)
        torch.cuda.synchronize()
        info = ctx.tree_info()
        ctx.sync()
        walk_ms = sum(e[1].elapsed_time(e[2]) for e in ev) / len(ev)
        tflops = info["interactions"] * FLOP_PER_INTERACTION / (walk_ms * 1e-3) / 1e12
        out[name] = {"n": n, "theta": theta, "eps": eps, "dt": dt, "steps": steps,
                     "steps_per_s": round(1000.0 / ms, 2), "ms_per_step": round(ms, 4),
                     "build_ms": round(sum(e[0].elapsed_time(e[1]) for e in ev) / len(ev), 4),
                     "walk_ms": round(walk_ms, 4), "interactions_per_step": info["interactions"],
                     "interactions_per_s": round(info["interactions"] * 1000.0 / ms, 1),
                     "walk_fp32_frac": round(tflops / peak, 4),
                     "force_error_vs_fp64_direct": {"median": float(np.median(rel)),
                                                    "p99": float(np.quantile(rel, 0.99)), "max": float(rel.max())}}
        del ctx, s
        torch.cuda.empty_cache()
    out["note"] = ("each configuration's steps replayed from one CUDA graph (steps_per_s); walk_fp32_frac from "
                   "three eager steps against the nominal FP32 peak; the reference arm's line times whole "
                   "steps of the same configurations")
    return out


ACCURACY_TARGET = 1e-4
ACCURACY_REFINE = 2
ACCURACY_THETAS = {(0, 0): (0.4, 0.3, 0.25, 0.2, 0.15, 0.125, 0.1),
                   (1, 0): (0.7, 0.65, 0.6, 0.55, 0.5, 0.45, 0.4, 0.35, 0.3),
                   (1, 1): (0.55, 0.5, 0.45, 0.4, 0.35, 0.3)}


def sweep_to_target(measure, thetas, refine: int):
    """Opening angles from large to small until measure(theta) -> (point, ok)
    meets the target, then `refine` bisection steps between that theta and the
    last one that missed (measure(theta, refine=True)).  Returns (points,
    at_target): every measured point, and the point of the largest theta that
    met the target (None when none did)."""
    points, at_target, above = [], None, None
    for th in thetas:
        pt, ok = measure(th)
        points.append(pt)
        if ok:
            at_target = pt
            break
        above = th
    if at_target is not None and above is not None:
        lo, hi = at_target["theta"], above
        for _ in range(refine):
            mid = round(0.5 * (lo + hi), 6)
            pt, ok = measure(mid, refine=True)
            points.append(pt)
            if ok:
                at_target, lo = pt, mid
            else:
                hi = mid
    return points, at_target


def bench_accuracy(args, local, b, targets, acc64, tune, multipole=0, key_order=0) -> dict:
    """The same workload at smaller opening angles, until the median force error
    against the FP64 direct sum reaches 1e-4 (the headline's theta 0.5 meets
    1e-4 only as FP32 arithmetic error of its own lists).  multipole 0: the
    parity-mode walk (monopoles, the reference's MAC with theta_ref = theta^2);
    1: the same lists with cell quadrupoles; key_order 1: Hilbert order (compact
    walk groups, other lists).  Per theta the error on the same 8192 targets,
    then plain FP32 steps timed with CUDA events after one warm-up step.  Once a
    theta meets the target, ACCURACY_REFINE bisection steps between it and the
    last theta that missed find a larger theta that still meets it."""
    import torch
    from nns_gb300.barnes_hut import Context, State
    n = len(b.x)
    ctx = Context(max_bodies=n, theta=THETA, eps=EPS, dt=DT, device=local, multipole=multipole,
                  key_order=key_order)
    ctx.set_systems([0, n])
    walk = None
    if multipole:
        # the quadrupole walk stages more per candidate: its own launch shape
        from nns_gb300 import autotune
        tq = autotune.tune_walk(ctx, State.from_bodies(b, device="cuda:%d" % local), use_cache=False,
                                stack_depths=(512,), radix_bits=(8,))
        walk = {"warps": tq["warps"], "variant": tq["variant"], "ms": tq["ms"]}
    elif tune:
        ctx.set_walk(tune["warps"], tune["variant"])
    _, eps2 = ctx.constants()

    def measure(th, refine=False):
        ctx.set_constants(float(np.float32(th) * np.float32(th)), eps2, 0)
        s = State.from_bodies(b, device="cuda:%d" % local)
        ctx.build(s)
        ctx.forces(s)
        ctx.sync()
        a = s.acc()[targets].astype(np.float64)
        rel = np.linalg.norm(a - acc64, axis=1) / np.linalg.norm(acc64, axis=1)
        ctx.step(s)
        k = 2
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(k)]
        torch.cuda.synchronize()
        for e in ev:
            e[0].record()
            ctx.build(s)
            ctx.forces(s)
            e[1].record()
            ctx.integrate(s)
            e[2].record()
        torch.cuda.synchronize()
        info = ctx.tree_info()
        ctx.sync()
        ms = sum(e[0].elapsed_time(e[2]) for e in ev) / k
        pt = {"theta": th, "steps_per_s": round(1000.0 / ms, 4), "ms_per_step": round(ms, 3), "steps": k,
              "interactions_per_step": info["interactions"],
              "force_error_vs_fp64_direct": {"median": float(np.median(rel)), "p99": float(np.quantile(rel, 0.99)),
                                             "max": float(rel.max())}}
        if refine:
            pt["refine"] = True
        del s
        return pt, bool(np.median(rel) <= ACCURACY_TARGET)

    points, at_target = sweep_to_target(measure, ACCURACY_THETAS[(multipole, key_order)], ACCURACY_REFINE)
    kind = ("parity-mode walk (monopoles, the reference MAC)" if multipole == 0 else
            "quadrupole mode (the reference MAC and lists, plus cell quadrupoles; not the parity mode)")
    if key_order:
        kind += ", Hilbert key order (other walk groups and lists)"
    return {"multipole": multipole, "key_order": key_order, "target_median": ACCURACY_TARGET, "points": points,
            "at_target": at_target,
            "walk_config": walk,
            "note": "%s; the first theta in %s whose median error meets the target, then %d bisection steps "
                    "towards the last theta that missed it (points marked refine); at_target is the largest "
                    "theta measured that meets it" % (kind, list(ACCURACY_THETAS[(multipole, key_order)]),
                                                       ACCURACY_REFINE)}


LEAF_SIZES = (1, 2, 4, 8)


def bench_buckets(args, local, b, targets, acc64, tune) -> dict:
    """Leaf buckets (nbx_params.leaf_size; outside the parity mode): the same
    workload at theta 0.5 with cells of at most k bodies as leaves.  Per k the
    error against the FP64 direct sum on the same targets, the cells and
    interactions, and plain FP32 steps timed with CUDA events after one warm-up
    step; then the autotuner's leaf-size stage picks k over build + walk steps."""
    import torch
    from nns_gb300 import autotune
    from nns_gb300.barnes_hut import Context, State
    n = len(b.x)
    ctx = Context(max_bodies=n, theta=THETA, eps=EPS, dt=DT, device=local)
    if tune:
        ctx.set_walk(tune["warps"], tune["variant"])
    ctx.set_systems([0, n])
    points = []
    for k in LEAF_SIZES:
        ctx.set_leaf_size(k)
        s = State.from_bodies(b, device="cuda:%d" % local)
        ctx.build(s)
        ctx.forces(s)
        ctx.sync()
        a = s.acc()[targets].astype(np.float64)
        rel = np.linalg.norm(a - acc64, axis=1) / np.linalg.norm(acc64, axis=1)
        ctx.step(s)
        reps = 3
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(reps)]
        torch.cuda.synchronize()
        for e in ev:
            e[0].record()
            ctx.build(s)
            ctx.forces(s)
            e[1].record()
            ctx.integrate(s)
            e[2].record()
        torch.cuda.synchronize()
        info = ctx.tree_info()
        ctx.sync()
        ms = sum(e[0].elapsed_time(e[2]) for e in ev) / reps
        points.append({"leaf_size": k, "steps_per_s": round(1000.0 / ms, 4), "ms_per_step": round(ms, 3),
                       "steps": reps, "cells": info["ncells"], "interactions_per_step": info["interactions"],
                       "opened_cells_per_step": info["opened"],
                       "force_error_vs_fp64_direct": {"median": float(np.median(rel)),
                                                      "p99": float(np.quantile(rel, 0.99))}})
        del s
    s = State.from_bodies(b, device="cuda:%d" % local)
    tb = autotune.tune_walk(ctx, s, use_cache=False, candidates=((ctx_warps(tune), ctx_variant(tune)),),
                            stack_depths=(512,), radix_bits=(8,), leaf_sizes=LEAF_SIZES)
    return {"theta": THETA, "points": points, "autotune_leaf_size": tb["leaf_size"], "autotune_ms": tb["ms_leaf"],
            "note": "leaf_size 1 is the reference's tree (the parity mode); k > 1 changes the tree and the lists"}


def ctx_warps(tune):
    return tune["warps"] if tune and "warps" in tune else 8


def ctx_variant(tune):
    return tune["variant"] if tune and "variant" in tune else 3


def error_target(errs, errs32, accuracy, accuracy_quad, accuracy_quad_h=None) -> dict:
    """Which reading of the metric's 1e-4 force error the headline meets: the FP32
    arithmetic error against an FP64 evaluation of the same interaction lists
    (met), and the total error against the FP64 direct sum (not at theta 0.5;
    the accuracy sections give the steps/s at the theta that meets it, with
    monopoles, with quadrupoles, and with quadrupoles in Hilbert order)."""
    def at_target(acc):
        at = acc.get("at_target") if isinstance(acc, dict) else None
        return None if at is None else {"theta": at["theta"], "median": at["force_error_vs_fp64_direct"]["median"],
                                        "steps_per_s": at["steps_per_s"],
                                        "interactions_per_step": at["interactions_per_step"]}
    return {"target_median_rel": ACCURACY_TARGET,
            "fp32_vs_fp64_same_lists": {"theta": THETA,
                                        "plain": errs32["plain"]["median"],
                                        "compensated": errs32["compensated"]["median"],
                                        "met": bool(errs32["plain"]["median"] <= ACCURACY_TARGET and
                                                    errs32["compensated"]["median"] <= ACCURACY_TARGET)},
            "vs_fp64_direct": {"theta": THETA, "plain": errs["plain"]["median"],
                               "compensated": errs["compensated"]["median"],
                               "met": bool(errs["plain"]["median"] <= ACCURACY_TARGET)},
            "vs_fp64_direct_at_target": at_target(accuracy),
            "vs_fp64_direct_at_target_quadrupole": at_target(accuracy_quad),
            "vs_fp64_direct_at_target_quadrupole_hilbert": at_target(accuracy_quad_h)}


def _section(fn, *a):
    """An extension section of the JSON line; a failure there is reported in
    the section and does not cost the headline measurement."""
    import torch
    try:
        return fn(*a)
    except Exception as e:  # noqa: BLE001 -- reported in the line
        if torch.cuda.is_available():
            torch.cuda.synchronize()
        return {"unavailable": "%s: %s" % (type(e).__name__, str(e)[:200])}


def total_energy(ctx, s) -> float:
    """K + W of the current state: K from the FP64 diagnostics, W = 1/2 sum m phi
    with phi from a Barnes-Hut walk over a fresh tree (accumulated in FP64)."""
    ctx.build(s)
    phi = ctx.potential(s).astype(np.float64)
    m = s.m.cpu().numpy().astype(np.float64)
    return float(ctx.diagnostics(s)["kinetic"]) + 0.5 * float((m * phi).sum())


def hbm_roofline(n: int, integ_ms: float, peaks: dict) -> dict:
    """The kick-drift kernel (k_update4, 16-byte accesses, one launch per step
    for a multiple of 4 bodies, bracketed alone by the integrate phase events):
    36 B read + 24 B written per body against the measured copy bandwidth."""
    peak = peaks.get("hbm_gbs")
    if not integ_ms > 0:
        return {"bound": "hbm", "kernel": "k_update4", "achieved": None, "peak": peak, "unit": "GB/s", "frac": None,
                "bytes_per_body": 60, "note": "the integrate phase was not timed"}
    achieved = 60.0 * n / (integ_ms * 1e-3) / 1e9
    return {"bound": "hbm", "kernel": "k_update4", "achieved": round(achieved, 1),
            "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4) if peak else None,
            "bytes_per_body": 60, "peak_kind": "measured copy bandwidth (MEASURED_PEAKS.json hbm_gbs)"}


def _git_blob_sha1(path: str) -> str:
    """The git blob hash of a file (sha1 of "blob <size>\\0" + content)."""
    import hashlib
    data = open(path, "rb").read()
    return hashlib.sha1(b"blob %d\0" % len(data) + data).hexdigest()


def walk_traffic(n: int):
    """DRAM bytes (read + write) of one walk launch at this size, from the committed
    ncu summary of the benchmark workload (profiles/), or None for other sizes or
    when the walk's source differs from the captured one (the summary records the
    git blob hash of walk2.cu)."""
    if n != N_DEFAULT:
        return None
    traffic = blob = None
    try:
        for line in open(os.path.join(ROOT, "profiles", "k_walk2_traffic_binary_disk_2p24.md")):
            if line.startswith("traffic_bytes_per_launch:"):
                traffic = int(line.split(":")[1])
            elif line.startswith("walk2_cu_blob:"):
                blob = line.split(":")[1].strip()
    except (OSError, ValueError):
        return None
    if blob != _git_blob_sha1(os.path.join(ROOT, "nns_gb300", "csrc", "walk2.cu")):
        return None
    return traffic


def bench_graph_steps(ctx, s, steps: int) -> dict:
    """The same plain steps replayed from a CUDA graph captured once
    (nbx_graph_step), timed with CUDA events after a warm-up replay: graph-
    launched steps/s beside the eager steps of `value` (at this size the launch
    overhead the graph removes is a small share of a step)."""
    import torch
    ctx.graph_step(s, 2)  # capture and warm up
    ctx.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    ctx.graph_step(s, steps)
    e1.record()
    torch.cuda.synchronize()
    ctx.sync()
    ms = e0.elapsed_time(e1) / steps
    return {"value": round(1000.0 / ms, 4), "unit": "steps/s", "ms_per_step": round(ms, 3), "steps": steps}


def bench_frame(ctx, s, b, reps: int = 5) -> dict:
    """One headless frame of the current state with the reference renderer's
    constants (1024 x 1024, dot 8; system size from the initial state, as
    main.cu:93-95), timed with CUDA events on the current stream."""
    import torch
    from nns_gb300.render import Frame, default_params
    half = float(max(np.abs(b.x).max(), np.abs(b.y).max(), np.abs(b.z).max()))
    fr = Frame(default_params(system_size=float(np.float32(2.0) * np.float32(half))))
    for _ in range(2):
        fr.render(ctx, s)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        img = fr.render(ctx, s)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    n = s.x.numel()
    return {"width": fr.p.width, "height": fr.p.height, "ms_per_frame": round(ms, 3),
            "bodies_per_s": round(n / (ms * 1e-3), 1), "lit_bytes": int((img > 0).sum().item())}


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.impl == "reference":
        line = run_reference(args, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return

    import torch
    from nns_gb300 import ic
    from nns_gb300.barnes_hut import Context, State

    torch.cuda.set_device(local)
    if args.only:
        section = bench_batched(args, local) if args.only == "batched" else bench_adjoint(args, local)
        if rank == 0:
            print(json.dumps({args.only: section}), flush=True)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    n = args.n
    b = ic.binary_disk(n)
    ctx = Context(max_bodies=n, theta=THETA, eps=EPS, dt=DT, device=local)
    ctx.set_systems([0, n])
    s = State.from_bodies(b, device="cuda:%d" % local)
    stream = torch.cuda.current_stream()
    tune = None
    if not args.no_tune:
        from nns_gb300 import autotune
        try:
            tune = autotune.tune_walk(ctx, s, use_cache=False)
        except Exception as e:  # noqa: BLE001 -- the default launch shape stays; reported
            tune = {"unavailable": str(e)[:200]}

    # several ranks: the system is split by key ranges of walk groups (each rank
    # walks its share of a replicated tree; the accelerations are summed over
    # NCCL); one rank: the plain step
    split = None
    if world > 1:
        from nns_gb300.dist import SplitSystem
        split = SplitSystem(ctx, s, rank, world)

    def timed(nsteps, phase=True):
        if split is not None:
            return timed_split(nsteps)
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(nsteps)]
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        inter = 0
        launches0 = ctx.tree_info()["launches"]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t0.record()
        for k in range(nsteps):
            ev[k][0].record()
            ctx.build(s)
            ev[k][1].record()
            ctx.forces(s)
            ev[k][2].record()
            ctx.integrate(s)
            ev[k][3].record()
        t1.record()
        torch.cuda.synchronize()
        info = ctx.tree_info()
        if info["status"]:
            ctx.sync()
        total = t0.elapsed_time(t1)
        build = sum(e[0].elapsed_time(e[1]) for e in ev)
        walk = sum(e[1].elapsed_time(e[2]) for e in ev)
        integ = sum(e[2].elapsed_time(e[3]) for e in ev)
        return dict(ms=total, build_ms=build, walk_ms=walk, integ_ms=integ,
                    interactions=info["interactions"], opened=info["opened"],
                    rounds=info["rounds"], candidates=info["candidates"],
                    launches=info["launches"] - launches0,
                    ncells=info["ncells"], max_level=info["max_level"])

    def timed_split(nsteps):
        """Steps of the key-range split, phases timed with CUDA events on this
        rank: build, this rank's walk plus the acceleration all-reduce (and the
        group-cost all-reduce that rebalances the ranges), integrate."""
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(nsteps)]
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        launches0 = ctx.tree_info()["launches"]
        torch.distributed.barrier()
        torch.cuda.synchronize()
        t0.record()
        inter = 0
        for k in range(nsteps):
            ev[k][0].record()
            ctx.build(s)
            ev[k][1].record()
            split.forces(build=False)
            ev[k][2].record()
            inter += ctx.tree_info()["interactions"]  # this rank's groups
            ctx.integrate(s)
            ev[k][3].record()
        t1.record()
        torch.cuda.synchronize()
        torch.distributed.barrier()
        total = t0.elapsed_time(t1)
        info = ctx.tree_info()
        from nns_gb300.dist import sum_over_ranks
        inter = int(sum_over_ranks(float(inter), device="cuda")) // max(nsteps, 1)
        return dict(ms=total, build_ms=sum(e[0].elapsed_time(e[1]) for e in ev),
                    walk_ms=sum(e[1].elapsed_time(e[2]) for e in ev),
                    integ_ms=sum(e[2].elapsed_time(e[3]) for e in ev), interactions=inter, opened=0,
                    rounds=0, candidates=0, launches=info["launches"] - launches0, ncells=info["ncells"],
                    max_level=info["max_level"])

    # ---- error at the initial state (outside any timed region)
    rng = np.random.default_rng(12345)
    targets = np.sort(rng.choice(n, size=min(args.targets, n), replace=False))
    acc64 = ctx.direct_fp64(s, targets, float(np.float32(EPS) * np.float32(EPS))).cpu().numpy()
    errs, errs32 = {}, {}
    lists64 = None
    stat = lambda rel: {"median": float(np.median(rel)), "p99": float(np.quantile(rel, 0.99)),  # noqa: E731
                        "max": float(rel.max())}
    for comp in (False, True):
        t_ref, e2 = ctx.constants()
        ctx.set_constants(t_ref, e2, comp)
        ctx.build(s)
        ctx.forces(s)
        ctx.sync()
        a = s.acc()[targets].astype(np.float64)
        if lists64 is None:
            lists64 = ctx.forces_fp64_lists(targets)
        rel = np.linalg.norm(a - acc64, axis=1) / np.linalg.norm(acc64, axis=1)
        errs["compensated" if comp else "plain"] = stat(rel)
        rel32 = np.linalg.norm(a - lists64, axis=1) / np.linalg.norm(lists64, axis=1)
        errs32["compensated" if comp else "plain"] = stat(rel32)
    t_ref, e2 = ctx.constants()
    ctx.set_constants(t_ref, e2, False)
    diag0 = ctx.diagnostics(s)
    energy0 = total_energy(ctx, s)
    initial = [t.clone() for t in (s.x, s.y, s.z, s.vx, s.vy, s.vz)]

    # ---- plain FP32: warmup + timed
    timed(args.warmup)
    with Clocks(local) as clk:
        plain = timed(args.steps)
    clocks = clk.summary()
    extra = max(0, RUN_STEPS - args.warmup - args.steps)  # untimed, to the end of the run
    timed(extra)
    energy1 = total_energy(ctx, s)
    diag1 = ctx.diagnostics(s)
    # ---- compensated FP32, the same steps from the same initial state
    for t, c in zip((s.x, s.y, s.z, s.vx, s.vy, s.vz), initial):
        t.copy_(c)
    del initial
    ctx.set_constants(t_ref, e2, True)
    timed(args.warmup)
    comp = timed(args.steps)
    timed(extra)
    ctx.set_constants(t_ref, e2, False)
    energy2 = total_energy(ctx, s)
    nst = args.warmup + args.steps + extra
    energy = {"plain": {"steps": nst, "rel_drift": (energy1 - energy0) / abs(energy0)},
              "compensated": {"steps": nst, "rel_drift": (energy2 - energy0) / abs(energy0)},
              "e0": energy0, "how": "K (FP64 sum) + W = 1/2 sum m phi, phi from the Barnes-Hut walk; "
                                    "both forms from the same initial state"}

    # ---- end to end through the public API with host buffers (pinned): every
    # step copies its inputs in and its results out.  Two device states are
    # used in turn so that the copies of one step overlap the compute of the
    # other (copy-in stream, compute stream, copy-out stream, ordered by events).
    host = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
            for a in (b.x, b.y, b.z, b.vx, b.vy, b.vz, b.m)]
    outs = [[torch.empty(n, dtype=torch.float32).pin_memory() for _ in range(6)] for _ in range(2)]
    states = [s, State.empty(n, device="cuda:%d" % local)]
    dev_in = [[t.x, t.y, t.z, t.vx, t.vy, t.vz, t.m] for t in states]
    h2d = sum(t.numel() * 4 for t in host)
    d2h = sum(t.numel() * 4 for t in outs[0])
    s_comp, s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    ev_in = [torch.cuda.Event() for _ in range(2)]
    ev_out = [torch.cuda.Event() for _ in range(2)]
    ev_done = [torch.cuda.Event() for _ in range(2)]
    cur = torch.cuda.current_stream()
    torch.cuda.synchronize()
    for e in ev_done:
        e.record(cur)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(cur)
    for st_ in (s_comp, s_in, s_out):
        st_.wait_event(e0)
    for k in range(args.steps):
        i = k % 2
        with torch.cuda.stream(s_in):
            s_in.wait_event(ev_done[i])  # the previous results of this state were read out
            for d, h in zip(dev_in[i], host):
                d.copy_(h, non_blocking=True)
            ev_in[i].record(s_in)
        s_comp.wait_event(ev_in[i])
        ctx.step(states[i], 1, stream=s_comp)
        ev_out[i].record(s_comp)
        with torch.cuda.stream(s_out):
            s_out.wait_event(ev_out[i])
            for o, d in zip(outs[i], dev_in[i][:6]):
                o.copy_(d, non_blocking=True)
            ev_done[i].record(s_out)
    for st_ in (s_in, s_comp, s_out):
        cur.wait_stream(st_)
    e1.record(cur)
    torch.cuda.synchronize()
    del states[1], dev_in[1]
    e2e_ms = e0.elapsed_time(e1) / args.steps
    ctx.sync()
    frame = bench_frame(ctx, s, b)
    graph = _section(bench_graph_steps, ctx, s, args.steps) if world == 1 else None

    ms_plain = plain["ms"] / args.steps
    ms_comp = comp["ms"] / args.steps
    walk_ms = plain["walk_ms"] / args.steps
    inter_per_step = plain["interactions"]
    flops = inter_per_step * FLOP_PER_INTERACTION
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    peaks = measured_peaks()
    max_mhz = peaks.get("sm_max_mhz") or clocks.get("sm_max_mhz") or 2070.0
    peak = peak_fp32_tflops(nsm, max_mhz)
    achieved = flops / (walk_ms * 1e-3) / 1e12
    if world > 1:
        # the interactions are summed over the ranks, each walking its share on its own GPU: per GPU
        from nns_gb300.dist import max_over_ranks
        achieved = flops / (max_over_ranks(walk_ms, device="cuda") * 1e-3) / 1e12 / world
    steps_per_s = 1000.0 / ms_plain

    if world > 1:
        # one system walked by all ranks: its steps/s is the job's (strong scaling)
        from nns_gb300.dist import max_over_ranks
        ms_plain = max_over_ranks(ms_plain, device="cuda")
        steps_per_s = 1000.0 / ms_plain

    batched = None
    del ctx, s
    torch.cuda.empty_cache()
    accuracy = accuracy_quad = accuracy_quad_h = None
    if not args.no_accuracy:
        accuracy = _section(bench_accuracy, args, local, b, targets, acc64,
                            tune if tune and "warps" in tune else None, 0)
        torch.cuda.empty_cache()
        accuracy_quad = _section(bench_accuracy, args, local, b, targets, acc64,
                                 tune if tune and "warps" in tune else None, 1)
        torch.cuda.empty_cache()
        accuracy_quad_h = _section(bench_accuracy, args, local, b, targets, acc64,
                                   tune if tune and "warps" in tune else None, 1, 1)
        torch.cuda.empty_cache()
    buckets = None
    if not args.no_buckets:
        buckets = _section(bench_buckets, args, local, b, targets, acc64, tune if tune and "warps" in tune else None)
        torch.cuda.empty_cache()
    hilbert = None
    if not args.no_hilbert:
        hilbert = _section(bench_hilbert, args, local, b, targets, acc64, tune if tune and "warps" in tune else None)
        torch.cuda.empty_cache()
    configs = None
    if not args.no_configs:
        configs = _section(bench_configs, args, local, tune if tune and "warps" in tune else None)
        torch.cuda.empty_cache()
    if not args.no_batched:
        batched = _section(bench_batched, args, local)
        torch.cuda.empty_cache()
    adjoint = None
    if not args.no_adjoint:
        adjoint = _section(bench_adjoint, args, local)
        torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            from oracle import ref_cpu
            cpu = ref_cpu.cpu_baseline(n, THETA, EPS, DT)
        except Exception as e:  # noqa: BLE001 -- reported, never fatal
            cpu = {"unavailable": str(e)[:200]}
        try:
            cpu_serial = ref_cpu.bench_serial(n, THETA, EPS, DT, k=512)
        except Exception as e:  # noqa: BLE001 -- reported, never fatal
            cpu_serial = {"unavailable": str(e)[:200]}
        if isinstance(cpu, dict) and cpu_serial is not None:
            cpu["serial"] = cpu_serial

    line = {
        "metric": METRIC, "value": round(steps_per_s, 4), "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_plain, 3),
        "higher_is_better": True, "scaling": "strong" if world > 1 else "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (nns_gb300.ic binary_disk, seed 20261203)",
        "config": workload_config(n, world),
        "compensated": {"value": round(1000.0 / ms_comp, 4), "unit": "steps/s",
                        "ms_per_step": round(ms_comp, 3),
                        "ratio_to_plain_time": round(ms_comp / ms_plain, 4)},
        "force_error_vs_fp64_direct": errs,
        "fp32_error_vs_fp64_same_lists": errs32,
        "error_target": error_target(errs, errs32, accuracy, accuracy_quad, accuracy_quad_h),
        "accuracy": accuracy,
        "accuracy_quadrupole": accuracy_quad,
        "accuracy_quadrupole_hilbert": accuracy_quad_h,
        "frame": frame,
        "energy_drift": energy,
        "interactions_per_step": inter_per_step,
        "opened_cells_per_step": plain["opened"],
        "walk_rounds_per_step": plain["rounds"],
        "walk_candidates_per_step": plain["candidates"],
        "interactions_per_s": inter_per_step * steps_per_s,
        "phase_ms": {"build": round(plain["build_ms"] / args.steps, 3), "walk": round(walk_ms, 3),
                     "integrate": round(plain["integ_ms"] / args.steps, 3)},
        "tree": {"cells": plain["ncells"], "max_level": plain["max_level"]},
        "roofline": {"bound": "fp32", "kernel": "k_walk2", "achieved": round(achieved, 3),
                     "peak": round(peak, 2), "unit": "TFLOP/s", "frac": round(achieved / peak, 4),
                     "traffic": walk_traffic(n) if world == 1 else None,
                     "peak_kind": "nominal FP32 FMA peak (SMs x 128 x 2 x max SM clock %g MHz)" % max_mhz,
                     **({"note": "per GPU: each rank walks its key range; the walk phase includes the "
                                 "acceleration and group-cost all-reduces"} if world > 1 else {})},
        "roofline_hbm": hbm_roofline(n, plain["integ_ms"] / args.steps, peaks),
        "diagnostics_fp64": {"momentum_drift": float(np.abs(diag1["momentum"] - diag0["momentum"]).max()),
                             "kinetic_rel_change": float((diag1["kinetic"] - diag0["kinetic"]) / diag0["kinetic"])},
        "e2e": {"value": round(1000.0 / e2e_ms, 4), "unit": "steps/s", "h2d_bytes_per_step": h2d,
                "pipeline": "two device states: the copies of one step overlap the compute of the other",
                "d2h_bytes_per_step": d2h},
        "graph": graph,
        "hilbert": hilbert,
        "configs": configs,
        "buckets": buckets,
        "batched": batched,
        "adjoint": adjoint,
        "autotune": tune,
        "gpu_launches": plain["launches"],
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
