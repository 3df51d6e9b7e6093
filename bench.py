#!/usr/bin/env python3
"""Headline benchmark: simulated steps per second of the contact hot path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload batch|wall|wall_nomerge|tower|funnel]

A step is one RigidBodySystem.advanceTime of every scene of the workload:
collision detection, contact setup, warm start, the projected Gauss-Seidel
solve, integration and sleeping.  The default workload is the batched one
(512 independent bins).  Every scene of every arm is iterated until its
relative LCP residual is <= 1e-6 (checked every 10 sweeps, cap SWEEP_CAP).

- `value`: the batched FP32 solve with previous-frame warm start and the
  conjugate-gradient (NNCG) acceleration of each sweep, simulated scene-steps
  per second with the state resident in HBM (device time of K steps, CUDA
  events on the library's stream).  `e2e`: the same steps through the C ABI
  with the body state pushed from and read back into pinned host buffers.
- `plain_gpu_pgs`: the same batched FP32 kernels, same scenes, steps and
  residual rule, plain projected Gauss-Seidel (no acceleration).
- `plain_gpu_pgs_one_scene_at_a_time`: plain FP32 PGS on the same kernels,
  one scene per launch sequence (a sample of the scenes).
- `fp64_drop_in_one_scene_at_a_time`: the FP64 drop-in's coloured solve, one
  scene at a time (a sample).
- `--impl reference`: the CPU restatement of the reference path (the oracle,
  FP64 Gauss-Seidel in list order with the same stopping rule) on all 512
  scenes over all host cores, timed by wall clock.
Scenes are independent, so several GPUs each run their own batch ("weak"
scaling, no collective): value = all ranks' scene-steps / max time.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from adaptivemerging_gb300 import abi, scenes  # noqa: E402

METRIC = "sim steps/s at LCP residual<=1e-6: warm-start+batched vs plain GPU PGS, 1 GB300"
FP64_BYTES_PER_CONTACT_SWEEP = 736   # J 288 + b,D 48 + lambda r/w 48 + dv of 2 bodies r/w 192 + minv,jinv 160
# compulsory HBM traffic of the batched sweep launches per step: per contact the
# 96 B record and the 16 B multiplier slot read once, the FP64 multipliers
# (24 B) and the contact state (4 B) written once; per body in contact its
# inverse mass and inertia (8 + 72 B), flags and compact id (8 B) read and its
# FP64 delta-v (48 B) written.  Everything else the sweeps touch stays in shared
# memory for the whole solve.
SWEEP_HBM_BYTES_PER_CONTACT = 96 + 16 + 24 + 4
SWEEP_HBM_BYTES_PER_BODY = 8 + 72 + 8 + 48
# cycles of one contact update on the sweep's dependent chain (arithmetic
# only, record in registers; measured with clock64 on one GB300)
CHAIN_CYCLES_PER_CONTACT = 170
BATCH_SCENES = 512
BATCH_SAMPLE_STRIDE = 32             # CPU baseline: every 32nd scene, one core
PLAIN_SAMPLE_STRIDE = 32             # one-scene-at-a-time arms: every 32nd scene
SWEEP_CAP = 20000                    # sweep cap of the residual-targeted solves
RESIDUAL_TARGET = 1e-6
STEADY = (20, 40)                    # the steady window: steps 21..60


FUNNEL_CLUMPS = 20000
FUNNEL_PLATFORM_MOTION = ((0.0, 1.0, 0.0), 0.05, 0.5)   # axis, amplitude (m), frequency (Hz)


def workload(name, n_scenes=BATCH_SCENES, order=None):
    # the full-solve order of single scenes: the mixed-precision coloured solve
    if order is None:
        order = "mixed"
    """Scene (or list of scenes), parameters, dt and a description of the named
    workload.  `n_scenes` shrinks the batch for profiling runs only; the
    benchmark figure is the 512-bin batch."""
    if name == "batch":
        sc = scenes.batch_scenes(n_scenes, seed=3)
        P = abi.default_params(gravity_amount=9.81, friction_override=0, restitution_override=1,
                               restitution=0.0, iterations=SWEEP_CAP, enable_merging=0)
        return sc, P, 0.005, {
            "workload": f"{n_scenes} independent bins, body counts log-uniform 20..2000, boxes U(0.1,1.0) m and "
                        "spheres U(0.05,0.5) m, density U(500,2000), per-scene mu U(0.3,0.8), 4 pinned walls + plane",
            "scenes": n_scenes, "bodies": int(sum(x.n for x in sc)), "dt": 0.005,
            "pgs": f"FP32 projected Gauss-Seidel with box friction, previous-frame warm start, each sweep wrapped "
                   f"in a nonsmooth nonlinear conjugate-gradient step; one CTA per scene (size-class launches) or "
                   f"a 2-8 CTA cluster for the largest; each scene swept until its relative LCP residual <= "
                   f"{RESIDUAL_TARGET:g} (checked every 10 sweeps, cap {SWEEP_CAP})",
            "merging": "off", "precision": "fp32 solve, fp64 collision/contact setup/integration"}
    so = {"reference": abi.AM_ORDER_REFERENCE, "coloured": abi.AM_ORDER_COLOURED, "mixed": abi.AM_ORDER_MIXED}[order]
    otext = {"reference": "list order (bit-exact)", "coloured": "coloured, FP64 sweeps",
             "mixed": "coloured, FP32 sweeps on the correction to an FP64 base point, FP64 refinement "
                      "every 100 sweeps"}[order]
    if name in ("wall", "wall_nomerge"):
        merging = name == "wall"
        sc = scenes.wall(cols=40, rows=25, seed=2)
        P = abi.default_params(gravity_amount=9.81, friction_override=1, friction=0.5, restitution_override=1,
                               restitution=0.0, iterations=200, enable_merging=int(merging),
                               solver_order=so)
        return sc, P, 0.005, {
            "workload": "brick wall 40x25 (0.4x0.2x0.2 m, 1000 kg/m3) + 50 kg sphere at 15 m/s",
            "bodies": int(sc.n), "dt": 0.005, "pgs_iterations": 200, "mu": 0.5,
            "merging": "on" if merging else "off", "pgs_order": f"full solve {otext}; exact single sweep",
            "precision": "fp64 state and multipliers"}
    if name == "funnel":
        sc = scenes.funnel_clumps(FUNNEL_CLUMPS, seed=5)
        P = abi.default_params(gravity_amount=9.81, friction_override=1, friction=0.7, restitution_override=1,
                               restitution=0.0, iterations=100, enable_merging=1, enable_sleeping=0,
                               solver_order=so)
        return sc, P, 0.002, {
            "workload": f"{FUNNEL_CLUMPS} sphere-tree clumps (4-16 spheres of r U(0.02, 0.08) m each) poured through "
                        "a funnel of four pinned panels (half-widths 3 m to 0.5 m) onto a platform oscillating "
                        "vertically at 0.5 Hz, 0.05 m (am_set_kinematic); sleeping off so that nothing rests "
                        "asleep on the moving platform",
            "bodies": int(sc.n), "clumps": FUNNEL_CLUMPS, "dt": 0.002, "pgs_iterations": 100, "mu": 0.7,
            "merging": "on", "pgs_order": f"full solve {otext}; exact single sweep",
            "precision": "fp64 state and multipliers"}
    if name == "tower":
        sc = scenes.tower(25, seed=1)
        P = abi.default_params(gravity_amount=9.81, friction_override=1, friction=0.6, restitution_override=1,
                               restitution=0.0, iterations=100, enable_merging=0,
                               solver_order=so)
        return sc, P, 0.01, {"workload": "tower of 25 boxes 1.0x0.5x1.0 m", "bodies": int(sc.n), "dt": 0.01,
                             "pgs_iterations": 100, "mu": 0.6, "merging": "off", "pgs_order": otext,
                             "precision": "fp64 state and multipliers"}
    raise SystemExit(f"unknown workload {name}")


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("AM_BENCH_GLOO") is None else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, x, device=None):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _oracle_scene_time(job):
    """One scene on the oracle: `warmup` untimed steps, then the seconds of
    `steps` timed steps (runs in a worker process)."""
    scene, P, dt, warmup, steps = job
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_binding import Oracle
    o = Oracle(scene, P)
    o.set_residual_target(RESIDUAL_TARGET, 10)
    o.step(dt, warmup)
    t0 = time.perf_counter()
    o.step(dt, steps)
    return time.perf_counter() - t0


def _reference_params(P):
    """The oracle's parameters for the batched workload: the reference's
    Gauss-Seidel in list order, stopped by the same residual rule as the GPU
    arms (the reference's own max-change test switched off)."""
    P.solver_order = abi.AM_ORDER_REFERENCE
    P.iterations = SWEEP_CAP
    P.tolerance = 0.0
    return P


def oracle_batch_sample(sc_list, P, dt, warmup, steps, stride=BATCH_SAMPLE_STRIDE):
    """Oracle on every `stride`-th scene from the initial state, one core:
    `warmup` untimed steps, then `steps` timed steps.  Returns scene-steps/s
    of one core and a description of the sample."""
    P = _reference_params(P)
    sample = sc_list[::stride]
    ts = [_oracle_scene_time((s, P, dt, warmup, steps)) for s in sample]
    t = sum(ts)
    return steps * len(sample) / t, (
        f"{len(sample)} of {len(sc_list)} scenes (every {stride}th), steps {warmup + 1}..{warmup + steps} from the "
        f"initial state, {t:.1f} s on one core; the reference's FP64 Gauss-Seidel in list order, stopped at "
        f"relative LCP residual <= {RESIDUAL_TARGET:g} (checked every 10 sweeps, cap {SWEEP_CAP}) like the GPU arms")


def cpu_baseline(name, max_seconds=15.0, warmup=20, steps=10, n_scenes=BATCH_SCENES):
    """Oracle (single-threaded CPU restatement of the reference path) on the
    same workload: steps/s over a bounded sample."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_binding import Oracle
    sc, P, dt, _ = workload(name, n_scenes)
    if name == "batch":
        v, desc = oracle_batch_sample(sc, P, dt, warmup, steps)
        return {"value": v, "unit": "scene-steps/s", "cores": 1, "kind": "port", "sample": desc}
    P.solver_order = abi.AM_ORDER_REFERENCE
    o = Oracle(sc, P)
    gpu_warmup = warmup
    if name == "funnel":
        # the oracle's all-pairs broad phase makes the pour's warm-up too long
        # for a bounded sample: it times the first steps instead
        o.set_kinematic(scenes.FUNNEL_PLATFORM, *FUNNEL_PLATFORM_MOTION, dt)
        warmup = 0
    o.step(dt, warmup)             # the GPU arm's warm-up, so both time the same steps
    t0 = time.perf_counter()
    n = 0
    while n < steps and time.perf_counter() - t0 < max_seconds:
        o.step(dt)
        n += 1
    el = time.perf_counter() - t0
    gpu_window = f"{gpu_warmup + 1}..{gpu_warmup + steps}"
    return {"value": n / el, "unit": "steps/s", "cores": 1, "kind": "port",
            "sample": f"steps {warmup + 1}..{warmup + n} of the same scene (the GPU arm times steps "
                      f"{gpu_window}), {el:.1f} s, single thread, reference order"}


_BARRIER = None


def _ref_init(barrier):
    global _BARRIER
    _BARRIER = barrier


def _ref_worker(job):
    """A share of the scenes on one core: warm-up steps, then (after every
    worker is ready) the timed steps.  Returns the monotonic clock at the start
    and end of the timed steps."""
    scenes_, P, dt, warmup, steps = job
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_binding import Oracle
    ors = []
    for s in scenes_:
        o = Oracle(s, P)
        o.set_residual_target(RESIDUAL_TARGET, 10)
        o.step(dt, warmup)
        ors.append(o)
    _BARRIER.wait()
    t0 = time.monotonic()
    for _ in range(steps):
        for o in ors:
            o.step(dt)
    return t0, time.monotonic()


def oracle_batch_wall(sc_list, P, dt, warmup, steps, workers):
    """Every scene of the batch on the oracle, spread over `workers` processes
    (largest scenes first, each to the least loaded worker).  All workers warm
    up, meet at a barrier, and step their scenes; the timed region is the wall
    clock from the first start to the last end."""
    import multiprocessing as mp
    P = _reference_params(P)
    workers = max(1, min(workers, len(sc_list)))
    order = sorted(range(len(sc_list)), key=lambda k: -sc_list[k].n)
    load = [0.0] * workers
    share = [[] for _ in range(workers)]
    for k in order:
        w = min(range(workers), key=lambda i: load[i])
        share[w].append(sc_list[k])
        load[w] += sc_list[k].n ** 1.6
    ctx = mp.get_context("spawn")
    bar = ctx.Barrier(workers)
    with ctx.Pool(workers, initializer=_ref_init, initargs=(bar,)) as pool:
        res = pool.map(_ref_worker, [(sh, P, dt, warmup, steps) for sh in share], chunksize=1)
    wall = max(t1 for _, t1 in res) - min(t0 for t0, _ in res)
    return wall, (f"all {len(sc_list)} scenes, steps {warmup + 1}..{warmup + steps} from the initial state, on "
                  f"{workers} worker processes (one core each), wall clock from the first timed step to the last; "
                  f"the reference's FP64 Gauss-Seidel in list order, stopped at relative LCP residual <= "
                  f"{RESIDUAL_TARGET:g} (checked every 10 sweeps, cap {SWEEP_CAP}) like the GPU arms")


def run_reference(args):
    ws, rank, _ = dist_init()
    if rank != 0:
        return
    sc, P, dt, cfg = workload(args.workload, args.scenes, args.order)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_binding import Oracle
    P.solver_order = abi.AM_ORDER_REFERENCE
    unit = "steps/s"
    cores = 1
    if args.workload == "batch":
        cores = max(1, len(os.sched_getaffinity(0)))
        el, desc = oracle_batch_wall(sc, P, dt, args.warmup, args.steps, cores)
        cores = min(cores, len(sc))
        v = args.steps * len(sc) / el
        unit = "scene-steps/s"
        cfg = dict(cfg, pgs=f"FP64 projected Gauss-Seidel with box friction in the reference's list order "
                            f"(PGS.java:73-194), previous-frame warm start, stopped at relative LCP residual <= "
                            f"{RESIDUAL_TARGET:g} (checked every 10 sweeps, cap {SWEEP_CAP})",
                   precision="fp64 throughout (the oracle, a C++ restatement of the reference path)",
                   parallelism=f"scenes spread over {cores} host cores")
    else:
        o = Oracle(sc, P)
        warm, steps = args.warmup, args.steps
        if args.workload == "funnel":
            # all-pairs broad phase on one core: the first steps of the pour,
            # at most about 30 s of them
            o.set_kinematic(scenes.FUNNEL_PLATFORM, *FUNNEL_PLATFORM_MOTION, dt)
            warm = 0
        o.step(dt, warm)
        t0 = time.perf_counter()
        n = 0
        while n < steps and (args.workload != "funnel" or time.perf_counter() - t0 < 30.0):
            o.step(dt)
            n += 1
        el = time.perf_counter() - t0
        v = n / el
        desc = f"{n} steps after {warm} warm-up steps, single thread"
        cfg = dict(cfg, pgs_order="reference list order", precision="fp64 throughout (the oracle)")
    nsteps = args.steps if args.workload == "batch" else n
    out = {"metric": METRIC, "value": v, "unit": unit, "n_gpus": ws, "steps": nsteps,
           "warmup": args.warmup, "ms_per_step": 1e3 * el / nsteps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
           "config": cfg,
           "cpu_baseline": {"value": v, "unit": unit, "cores": cores, "kind": "port", "sample": desc},
           "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def fp64_drop_in_one_scene_at_a_time(sc_list, dt, warmup, steps, flush):
    """The FP64 drop-in, one scene per context and launch sequence (coloured
    full solve, stop at the same relative residual), on every
    PLAIN_SAMPLE_STRIDE-th scene.  CUDA-event time per scene-step."""
    import torch
    from adaptivemerging_gb300 import native
    P = abi.default_params(gravity_amount=9.81, friction_override=0, restitution_override=1, restitution=0.0,
                           iterations=SWEEP_CAP, tolerance=0.0, enable_merging=0,
                           solver_order=abi.AM_ORDER_COLOURED)
    sample = sc_list[::PLAIN_SAMPLE_STRIDE]
    tot_ms, n, conv, sweeps = 0.0, 0, 0, []
    for s in sample:
        g = native.System(s, P)
        g.set_residual_target(RESIDUAL_TARGET, 10)
        stream = torch.cuda.ExternalStream(g.stream_handle())
        for _ in range(warmup):
            g.step(dt)
        for _ in range(steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.step(dt)
            e1.record(stream)
            e1.synchronize()
            tot_ms += e0.elapsed_time(e1)
            st = g.stats()
            conv += int(st.residual_rel <= RESIDUAL_TARGET)
            sweeps.append(st.sweeps)
            n += 1
        g.close()
    return {"value": 1e3 * n / tot_ms, "unit": "scene-steps/s",
            "sample": f"{len(sample)} of {len(sc_list)} scenes (every {PLAIN_SAMPLE_STRIDE}th) stepped one at a "
                      f"time, steps {warmup + 1}..{warmup + steps}, FP64 coloured PGS to relative residual <= "
                      f"{RESIDUAL_TARGET:g} (cap {SWEEP_CAP})",
            "frac_scene_steps_residual_le_1e-6": conv / max(1, n), "pgs_sweeps_mean": float(np.mean(sweeps))}


def _batch_system(sc, P, threads, accel, stage=0):
    from adaptivemerging_gb300 import native
    g = native.BatchSystem(sc, P, threads=threads, residual_target=RESIDUAL_TARGET, check_every=10)
    g.set_accel(accel)
    if stage:
        g.set_stage(stage)
    return g


def time_batch_window(g, dt, steps, flush, stream, pin=None, n_units=None):
    """K timed steps of a BatchSystem (device time on its stream, L2 flushed
    between steps).  With `pin` (pinned host body state), every step also
    pushes the state before and reads it back after (the end-to-end figure).
    Per step: sweeps and residual of every scene and the critical path."""
    import torch
    g.reset_perf()
    p0 = g.perf()
    out = {"ms": 0.0, "e2e_s": 0.0, "put_get_s": [0.0, 0.0], "contacts": [], "sweeps_mean": [], "conv": [],
           "res_max": [], "floor_cycles": 0, "sweeps_total": 0}
    for _ in range(steps):
        flush.fill_(1.0)                     # L2 flush between timed steps
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        ta = time.perf_counter()
        if pin is not None:
            g.put_bodies_struct(pin)         # H2D of the host-owned state
        tb = time.perf_counter()
        e0.record(stream)
        g.step(dt)
        e1.record(stream)
        tc = time.perf_counter()
        if pin is not None:
            g.get_bodies_struct(pin)         # D2H of the new state
        td = time.perf_counter()
        e1.synchronize()
        out["ms"] += e0.elapsed_time(e1)
        out["e2e_s"] += td - ta
        out["put_get_s"][0] += tb - ta
        out["put_get_s"][1] += td - tc
        st = g.stats()
        bs = g.batch_stats()
        ss = g.scene_stats()
        chain = g.scene_chain()
        out["contacts"].append(st.n_contacts)
        out["sweeps_mean"].append(bs.sweeps_sum / max(1, bs.n_scenes))
        out["conv"].append(float(np.mean(ss["residual"] <= RESIDUAL_TARGET)))
        out["res_max"].append(float(ss["residual"].max()))
        out["floor_cycles"] += int((ss["sweeps"].astype(np.int64) * chain).max()) * CHAIN_CYCLES_PER_CONTACT
        out["sweeps_total"] += int(ss["sweeps"].sum())
    torch.cuda.synchronize()
    p1 = g.perf()
    out["launches"] = int(p1.launches - p0.launches)
    out["pgs_ms"] = p1.pgs_ms - p0.pgs_ms
    out["contact_sweeps"] = int(p1.contact_sweeps - p0.contact_sweeps)
    out["phases_ms"] = g.step_phases()
    bst = g.batch_stats()
    out["last"] = {"cta_threads": int(bst.threads), "stage_slots": int(bst.stage_slots),
                   "resident_scenes": int(bst.resident_scenes), "cluster_scenes": int(bst.cluster_scenes),
                   "cluster_size": int(bst.cluster_size)}
    return out


def summarise_window(w, steps, n_units, first, label):
    ms = w["ms"] / steps
    return {"value": 1e3 * n_units / ms, "unit": "scene-steps/s", "ms_per_step": ms,
            "window": f"steps {first + 1}..{first + steps} from the initial state ({label})",
            "frac_scene_steps_residual_le_1e-6": float(np.mean(w["conv"])),
            "residual_rel_max": float(np.max(w["res_max"])), "pgs_sweeps_mean": float(np.mean(w["sweeps_mean"])),
            "contacts_mean": float(np.mean(w["contacts"])),
            "phases_ms_per_step": {k: v / steps for k, v in w["phases_ms"].items()}}


def plain_fp32_one_scene_at_a_time(sc_list, P, dt, warmup, steps, flush):
    """Plain FP32 PGS on the batched kernels, one scene per context and
    launch sequence, on every PLAIN_SAMPLE_STRIDE-th scene."""
    import torch
    sample = sc_list[::PLAIN_SAMPLE_STRIDE]
    tot_ms, n, conv = 0.0, 0, []
    for s in sample:
        g = _batch_system([s], P, 0, 0)
        stream = torch.cuda.ExternalStream(g.stream_handle())
        for _ in range(warmup):
            g.step(dt)
        w = time_batch_window(g, dt, steps, flush, stream)
        tot_ms += w["ms"]
        n += steps
        conv += w["conv"]
        g.close()
    return {"value": 1e3 * n / tot_ms, "unit": "scene-steps/s",
            "sample": f"{len(sample)} of {len(sc_list)} scenes (every {PLAIN_SAMPLE_STRIDE}th), each alone in its "
                      f"own context, steps {warmup + 1}..{warmup + steps}, plain FP32 PGS on the batched kernels "
                      f"to relative residual <= {RESIDUAL_TARGET:g} (cap {SWEEP_CAP})",
            "frac_scene_steps_residual_le_1e-6": float(np.mean(conv))}


def learned_protocol(sc_list, P, dt, collect_steps=100, compare_steps=30, stride=4):
    """Learned warm start against the plain previous-frame start: two copies
    of every `stride`-th scene step in lockstep; the first records (features,
    converged impulse) pairs and trains the network on the device, the
    second then takes the learned start.  Contact-sweeps of the two over the
    next `compare_steps` steps, same residual target."""
    from adaptivemerging_gb300 import native
    sample = sc_list[::stride]
    a = native.BatchSystem(sample, P, threads=0, residual_target=RESIDUAL_TARGET, check_every=10)
    b = native.BatchSystem(sample, P, threads=0, residual_target=RESIDUAL_TARGET, check_every=10)
    a.learned_collect(True, 2_000_000)
    for _ in range(collect_steps):
        a.step(dt)
        b.step(dt)
    n = a.learned_info()["n_samples"]
    t0 = time.perf_counter()
    loss = a.learned_train(epochs=1, batch=min(4096, max(64, n // 8)), lr=1e-3, normalise=True)
    loss = a.learned_train(epochs=20, batch=min(4096, max(64, n // 8)), lr=1e-3, normalise=False)
    train_s = time.perf_counter() - t0
    w, nm = a.learned_weights()
    b.learned_weights(set_w=w, set_norm=nm)
    b.learned_use(1)
    a.learned_collect(False)
    cs = [0, 0]
    conv = [0, 0]
    falls = 0
    for _ in range(compare_steps):
        for k, g in enumerate((a, b)):
            g.step(dt)
            st = g.batch_stats()
            cs[k] += st.contact_sweeps
            conv[k] += st.converged
        falls += b.learned_info()["fallback_scenes"]
    return {"scenes": len(sample), "samples": n, "train_seconds": train_s, "train_loss": loss,
            "contact_sweeps_plain": cs[0], "contact_sweeps_learned": cs[1],
            "sweeps_saved_frac": 1.0 - cs[1] / max(1, cs[0]),
            "converged_scene_steps_plain": conv[0], "converged_scene_steps_learned": conv[1],
            "fallback_scene_steps": falls, "scene_steps": compare_steps * len(sample),
            "protocol": f"{collect_steps} recording steps, 21 epochs of Adam on the device, then {compare_steps} "
                        f"steps in lockstep; learned start for fresh contacts, BF16 tensor-core inference"}


def run_ours(args):
    import torch
    from adaptivemerging_gb300 import build, native
    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    if local == 0:                    # one compiler per node; the others wait for the library
        build.build()
    barrier(ws)
    sc, P, dt, cfg = workload(args.workload, args.scenes, args.order)
    batch = args.workload == "batch"
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    if batch:
        sysm = _batch_system(sc, P, args.threads, 1, args.stage)
        n_units = len(sc)
    else:
        sysm = native.System(sc, P)
        n_units = 1
        if args.workload == "funnel":
            sysm.set_kinematic(scenes.FUNNEL_PLATFORM, *FUNNEL_PLATFORM_MOTION, dt)
    stream = torch.cuda.ExternalStream(sysm.stream_handle())
    # host-owned body state in pinned memory: every timed step pushes it to the
    # device, steps, and reads it back (the end-to-end figure); the device
    # time of the step alone is the `value` figure, on the same steps
    n = sysm.n
    pin = {k: torch.zeros(m * n, dtype=torch.float64, pin_memory=True) for k, m in
           (("x", 3), ("R", 9), ("v", 3), ("omega", 3))}
    pin_i = {k: torch.zeros(n, dtype=torch.int32, pin_memory=True) for k in ("sleeping", "parent")}
    st_s = abi.am_body_state()
    for k, t in pin.items():
        setattr(st_s, k, C.cast(t.data_ptr(), C.POINTER(C.c_double)))
    for k, t in pin_i.items():
        setattr(st_s, k, C.cast(t.data_ptr(), C.POINTER(C.c_int32)))
    h2d = sum(t.numel() * 8 for t in pin.values())
    d2h = h2d + sum(t.numel() * 4 for t in pin_i.values())
    for _ in range(args.warmup):
        sysm.step(dt)
    sysm.get_bodies_struct(st_s)
    barrier(ws)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    if args.profile:
        torch.cuda.profiler.start()
    if batch:
        w = time_batch_window(sysm, dt, args.steps, flush, stream, pin=st_s)
        total_ms, e2e_s, split = w["ms"], w["e2e_s"], w["put_get_s"]
        launches = w["launches"]
        pgs_ms = w["pgs_ms"]
    else:
        sysm.reset_perf()
        p0 = sysm.perf()
        total_ms = e2e_s = 0.0
        split = [0.0, 0.0]
        res = []
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            ta = time.perf_counter()
            sysm.put_bodies_struct(st_s)
            tb = time.perf_counter()
            e0.record(stream)
            sysm.step(dt)
            e1.record(stream)
            tc = time.perf_counter()
            sysm.get_bodies_struct(st_s)
            td = time.perf_counter()
            e1.synchronize()
            total_ms += e0.elapsed_time(e1)
            e2e_s += td - ta
            split[0] += tb - ta
            split[1] += td - tc
            res.append(sysm.stats().residual_rel)
        p1 = sysm.perf()
        launches = int(p1.launches - p0.launches)
        pgs_ms = p1.pgs_ms - p0.pgs_ms
        window_events = {"merge_events": int(p1.merge_events - p0.merge_events),
                         "unmerge_events": int(p1.unmerge_events - p0.unmerge_events),
                         "merge_events_total": int(p1.merge_events), "unmerge_events_total": int(p1.unmerge_events),
                         "contacts_last_step": int(sysm.num_contacts())}
    torch.cuda.synchronize()
    if args.profile:
        torch.cuda.profiler.stop()
    clk = clocks.stop()
    barrier(ws)
    t_max = max_over_ranks(ws, total_ms / 1e3, "cuda")
    value = ws * args.steps * n_units / t_max
    e2e_t = max_over_ranks(ws, e2e_s, "cuda")
    e2e = ws * args.steps * n_units / e2e_t
    if rank != 0:
        return
    peak, peak_kind = measured_peak()
    unit = "scene-steps/s" if batch else "steps/s"
    cfg.update({"l2": "flushed between timed steps (256 MB write)",
                "parallelism": "independent scenes per GPU" if batch else "replicas only",
                "timed_window": f"steps {args.warmup + 1}..{args.warmup + args.steps} from the initial state"})
    out = {"metric": METRIC, "value": value, "unit": unit, "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32" if batch else "f64", "data": "synthetic",
           "config": cfg,
           "e2e": {"value": e2e, "unit": unit, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                   "ms_per_step_put_get": [1e3 * x / args.steps for x in split],
                   "note": "same steps as value; wall time of push + step + read back through the C ABI"},
           "gpu_launches": launches, "clocks": clk}
    if batch:
        sm_mhz = clk.get("sm_mhz") or 2070.0
        head = summarise_window(w, args.steps, n_units, args.warmup, "the timed steps")
        cfg.update({k: head[k] for k in ("frac_scene_steps_residual_le_1e-6", "residual_rel_max",
                                         "pgs_sweeps_mean", "contacts_mean")})
        cfg.update(w["last"])
        sweep_ms = pgs_ms / args.steps
        bytes_step = head["contacts_mean"] * SWEEP_HBM_BYTES_PER_CONTACT + cfg["bodies"] * SWEEP_HBM_BYTES_PER_BODY
        achieved = bytes_step / (sweep_ms / 1e3) / 1e9 if sweep_ms > 0 else 0.0
        traffic = traffic_basis = None
        tf = os.path.join(ROOT, "profiles", "k_batch_sweep_traffic.json")
        if os.path.exists(tf):
            with open(tf) as f:
                tj = json.load(f)
            if tj.get("warmup") == args.warmup and tj.get("steps") == args.steps:
                traffic = tj.get("dram_bytes_per_step")
                traffic_basis = tj.get("basis")
        floor_ms = w["floor_cycles"] / (sm_mhz * 1e3) / args.steps
        out["roofline"] = {
            "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if peak else None, "traffic": traffic, "traffic_basis": traffic_basis,
            "peak_source": peak_kind,
            "kernel": "k_batch_sweep + k_batch_sweep_cluster (all sweep launches of a step)",
            "sweep_ms_per_step": sweep_ms,
            "algorithmic_bytes_per_step": bytes_step,
            "note": "compulsory HBM bytes of the sweep launches (records and multipliers in once, results out "
                    "once); every sweep after the first reads shared memory, so the sweep is not HBM-bound: "
                    "see critical_path"}
        out["critical_path"] = {
            "bound": "dependent-chain latency", "unit": "ms per step",
            "floor_ms_per_step": floor_ms, "sweep_ms_per_step": sweep_ms,
            "frac": floor_ms / sweep_ms if sweep_ms > 0 else None,
            "cycles_per_contact": CHAIN_CYCLES_PER_CONTACT, "sm_mhz": sm_mhz,
            "definition": "per step, max over scenes of sweeps x (sum over colours of the longest body-pair group "
                          "in contacts) x cycles of one contact update's arithmetic chain, at the sampled SM clock; "
                          "the scenes run concurrently, so the slowest chain bounds the sweep launches"}
        out["phases_ms_per_step"] = head["phases_ms_per_step"]
        out["phases_note"] = ("device time between consecutive CUDA events on the library stream; the phases add up "
                              "to the step, host waits included")
        sysm.close()
        # the same kernels and scenes, plain projected Gauss-Seidel
        if not args.no_plain:
            pg = _batch_system(sc, P, args.threads, 0, args.stage)
            pstream = torch.cuda.ExternalStream(pg.stream_handle())
            for _ in range(args.warmup):
                pg.step(dt)
            pw = time_batch_window(pg, dt, args.steps, flush, pstream)
            plain = summarise_window(pw, args.steps, n_units, args.warmup, "the timed steps")
            plain["pgs"] = "FP32 projected Gauss-Seidel, no acceleration, previous-frame warm start, same kernels"
            out["plain_gpu_pgs"] = plain
            out["accelerated_over_plain"] = value / plain["value"]
            pg.close()
        # the steady window (steps 21..60) beside the timed one, both arms
        if (args.warmup, args.steps) != STEADY and not args.no_steady and not args.no_plain:
            steady = {}
            for name, acc in (("accelerated", 1), ("plain", 0)):
                g = _batch_system(sc, P, args.threads, acc, args.stage)
                gs = torch.cuda.ExternalStream(g.stream_handle())
                for _ in range(STEADY[0]):
                    g.step(dt)
                sw = time_batch_window(g, dt, STEADY[1], flush, gs)
                steady[name] = summarise_window(sw, STEADY[1], n_units, STEADY[0], "steady window")
                g.close()
            steady["accelerated_over_plain"] = steady["accelerated"]["value"] / steady["plain"]["value"]
            out["steady_window"] = steady
        if not args.no_plain:
            k1 = min(args.steps, 10)
            one = plain_fp32_one_scene_at_a_time(sc, P, dt, args.warmup, k1, flush)
            one["batched_accelerated_over_this"] = value / one["value"]
            out["plain_gpu_pgs_one_scene_at_a_time"] = one
            f64 = fp64_drop_in_one_scene_at_a_time(sc, dt, args.warmup, k1, flush)
            f64["batched_accelerated_over_this"] = value / f64["value"]
            out["fp64_drop_in_one_scene_at_a_time"] = f64
        if args.learned:
            out["learned_warm_start"] = learned_protocol(sc, P, dt)
    else:
        cfg["frac_steps_residual_le_1e-6"] = float(np.mean(np.array(res) <= 1e-6))
        out["pgs_ms_per_step"] = pgs_ms / args.steps
        out["events"] = window_events
        out["solve_form"] = sysm.mixed_form()
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args.workload, warmup=args.warmup,
                                           steps=min(args.steps, 10) if batch else args.steps, n_scenes=args.scenes)
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=None,
                    help="untimed steps before the window (default 20; the funnel 600, by which the pour has "
                         "reached the platform)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch")
    ap.add_argument("--order", default=None, choices=("reference", "coloured", "mixed"),
                    help="full-solve order of the single-scene workloads (tower, wall, wall_nomerge)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the comparison arms (plain batched PGS, one scene at a time; profiling runs only)")
    ap.add_argument("--no-steady", action="store_true", help="skip the steady-window (steps 21..60) figures")
    ap.add_argument("--learned", action="store_true", help="also run the learned warm-start protocol")
    ap.add_argument("--threads", type=int, default=0, help="batched solve: CTA size (0: autotuned)")
    ap.add_argument("--scenes", type=int, default=BATCH_SCENES, help="bins in the batch (profiling runs only)")
    ap.add_argument("--profile", action="store_true",
                    help="bracket the timed steps with cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    ap.add_argument("--stage", type=int, default=0,
                    help="batched solve: staging slots (0: autotuned; with --threads, no tuning launches)")
    args = ap.parse_args()
    if args.warmup is None:
        args.warmup = 600 if args.workload == "funnel" else 20
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
