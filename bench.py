#!/usr/bin/env python3
"""Benchmark of the batched Euler finite-volume update (one JSON line on stdout).

Workload (the batched configuration): 512 independent 2D grids, N x N with N
log-uniform in [64, 512] (SplitMix64 seed 4), each a four-quadrant Riemann
problem with per-quadrant rho, P ~ U(0.1, 2), vx, vy ~ U(-1, 1), gamma 1.4,
freeflow boundaries, "plm cons" reconstruction with the van Leer slope limiter,
Roe flux, Runge-Kutta 2 (midpoint), per-instance CFL dt (0.475), FP32 bulk with
FP64 dt reduction and time.  31.8 M interior cells in total.  A step is one
update of every instance (two fused stage launches plus the per-instance dt
kernel).  Synthetic, seeded inputs stand in for a dataset (the reference has
none for this path).

The van Leer limiter is the reference's own alternate form kept beside its
table entry (hydro/app.lua:631, (r + |r|) / (1 + |r|)): the table form divides
0 by 0 at r = -1, which the reference's own arithmetic reaches within a few
steps on every quadrant problem (see the parity tests); the two are identical
for every other r.

Arms:
  default           the CUDA batched FP32 form through libhydrocuda's C ABI
  --impl reference  the reference's algorithm on the host cores (the C++ CPU
                    restatement of its OpenCL kernels; the reference's own
                    LuaJIT/OpenCL stack cannot run on these machines)
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "hydro-cl-lua_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
for p in (PKG, ORACLE_DIR):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "cell-updates/s (FP32 batched)"
WORKLOAD = ("batched 2D Euler: 512 quadrant Riemann problems, N log-uniform in [64,512] (seed 4), "
            "plm cons + van Leer, Roe, RK2, CFL .475, gamma 1.4, freeflow")
UNIT = "cell-updates/s"
COUNT = 512
E2E_STEPS = 200          # the configuration's 200 steps per instance
STATUS_BYTES_PER_SLOT = 64   # per-slot status head read back after every update
SCHEME = dict(usePLM="plm cons", slopeLimiter="van Leer (abs)", integrator="Runge-Kutta 2")
BYTES_PER_VALUE = 4
FIELDS = 5


def instance_args(n):
    return dict(dim=2, gridSize=[n, n], mins=[-1, -1, -1], maxs=[1, 1, 1], boundary="freeflow",
                cfl=.475, eqnArgs={"heatCapacityRatio": 1.4}, **SCHEME)


def workload(count=COUNT, seed=4, rank=0):
    import hydrocuda as hc
    sizes = hc.batched_quadrant_sizes(count, seed + 7919 * rank)
    out = []
    for i, n in enumerate(sizes):
        args = instance_args(n)
        q = hc.random_quadrants(hc.SplitMix64(100000 * (rank + 1) + i))
        out.append((args, q))
    return out


def aggregate(elapsed, credited, dist):
    """The whole job's clock and work over the ranks: the slowest rank's timed
    region (max) and every rank's credited cell-updates (sum).  `dist` None:
    one rank."""
    if not dist:
        return elapsed, credited
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([elapsed], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([float(credited)], dtype=torch.float64, device=dev)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return float(t.item()), int(c.item())


def soa5_f32(hc, args, q):
    cons = hc.quadrant_state(args, q)
    return np.ascontiguousarray(cons[:, :5].T, dtype=np.float32)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0}, "fallback"


def stage_arrays(integrator_index):
    """Algorithmic state arrays each fused stage moves (reads + writes) for the
    explicit integrators, from the reference's tables: the halo input, the
    other pointwise states and stored derivatives it combines, the output, and
    a stored derivative when a later stage needs it."""
    tables = {1: [2, 3], 7: [2, 3], 9: [2, 3, 3], 0: [2]}
    return tables.get(integrator_index)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), "hc_clocks_%d.csv" % os.getpid())

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
            time.sleep(0.15)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        try:
            rows = [l.strip().split(",") for l in open(self.path) if l.strip()]
        except Exception:
            rows = []
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(nm)
            except Exception:
                pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def traffic_from_profiles(schedule, cells):
    """DRAM bytes per stage launch of `schedule`, from the committed ncu
    summary of the batched workload's stage kernel (profiles/traffic.json:
    dram__bytes_read.sum + dram__bytes_write.sum per interior cell-stage,
    measured per schedule), scaled by this workload's interior cells; None
    when that schedule has no capture."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            t = json.load(f)
        return float(t["schedules"][str(schedule)]["dram_bytes_per_cell_stage"]) * cells
    except Exception:
        return None


def cpu_baseline(work, budget_s=12.0, budget_cells=6_000_000):
    """The oracle (C++ restatement, OpenMP on all host cores) on a bounded
    sample of the workload: the first instances up to `budget_cells` cells
    (their oracle state held in host memory at once), then rounds of one update
    of each of them until the time budget is spent (at least one round)."""
    import hydrocuda as hc
    import oracle
    oracle.build()
    n_thr = oracle.num_threads()
    solvers = []
    held = 0
    for args, q in work:
        s = oracle.OracleSolver(args)
        s.reset_state(hc.quadrant_state(args, q))
        s.update()   # first-touch warm-up of this instance
        n = args["gridSize"][0] * args["gridSize"][1]
        solvers.append((s, n))
        held += n
        if held >= budget_cells:
            break
    cells = 0
    t_total = 0.0
    rounds = 0
    while True:
        for s, n in solvers:
            t0 = time.perf_counter()
            s.update()
            t_total += time.perf_counter() - t0
            cells += n
        rounds += 1
        if t_total >= budget_s:
            break
    return {"value": cells / t_total, "unit": UNIT, "cores": n_thr, "kind": "port",
            "sample": "%d rounds of one Runge-Kutta 2 update of the first %d of %d instances (%d cells; %d cell-updates), "
                      "%.1f s" % (rounds, len(solvers), len(work), held, cells, t_total)}


def run_reference(args):
    """--impl reference: the reference's algorithm (oracle port) on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import hydrocuda as hc
    import oracle
    work = workload()
    oracle.build()
    solvers = []
    # a bounded sample: at most 6 M cells, fewer when --steps is large, so the
    # whole run stays near two minutes at the oracle's ~3e7 cell-updates/s
    budget_cells = int(min(6_000_000, max(250_000, 3e7 * 120 / (args.steps + args.warmup))))
    cells = 0
    for a, q in work:
        s = oracle.OracleSolver(a)
        s.reset_state(hc.quadrant_state(a, q))
        solvers.append(s)
        cells += a["gridSize"][0] * a["gridSize"][1]
        if cells >= budget_cells:
            break
    for _ in range(args.warmup):
        for s in solvers:
            s.update()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for s in solvers:
            s.update()
    dt = time.perf_counter() - t0
    value = cells * args.steps / dt
    sample = "first %d of %d instances (%d cells), %d updates each" % (len(solvers), len(work), cells, args.steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "cells": sum(a["gridSize"][0] * a["gridSize"][1] for a, _ in work),
                   "instances": len(work), "parallelism": "host cores (OpenMP)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--serving-requests", type=int, default=1000,
                    help="requests of the bounded serving run reported in the bench line")
    ap.add_argument("--count", type=int, default=COUNT,
                    help="instances (the configuration has 512; fewer only for profiling a small case)")
    ap.add_argument("--workload", default="c4", choices=["c4", "c1", "c2", "c3", "c5"],
                    help="c4: the batched quadrants (the headline); c1 Sod; c2 Kelvin-Helmholtz 1024^2; "
                         "c3 blast 256^3; c5 serving")
    ap.add_argument("--size", type=int, default=0, help="c2 / c3: grid side (default: the configuration's)")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="c2 / c3: only step the FP32 batch --warmup + this many updates (a case for ncu)")
    ap.add_argument("--schedule", type=int, default=-1,
                    help="c4: pin the 2D stage-kernel schedule (autotuner variant number) instead of tuning")
    ap.add_argument("--requests", type=int, default=1000,
                    help="c5: requests in the stream (the configuration has 20000)")
    ap.add_argument("--host-states", action="store_true",
                    help="c5: build initial states on the host and upload them (default: on the device)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "c4":
        return {"c1": run_c1, "c2": run_c2, "c3": run_c3, "c5": run_c5}[args.workload](args)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        torch.cuda.set_device(local)

    import hydrocuda as hc
    ctx = hc.Context(local)
    work = workload(count=args.count, rank=rank)
    cells = sum(a["gridSize"][0] * a["gridSize"][1] for a, _ in work)
    inputs = [soa5_f32(hc, a, q) for a, q in work]
    b = hc.Batch(ctx, precision="f32", max_slots=len(work), **SCHEME)
    cells_of = {}
    for k, ((a, _), u) in enumerate(zip(work, inputs)):
        slot = b.admit(a, u, t_end=math.inf, tag=k, layout="soa5_f32")
        cells_of[slot] = a["gridSize"][0] * a["gridSize"][1]
    tune_cache = os.path.join(PKG, "_build", "autotune.txt")
    if args.schedule >= 0:
        b.set_schedule(2, args.schedule)
    elif not args.no_autotune:
        b.autotune(tune_cache)
    st = b.stats()
    b.step(args.warmup)

    before = {e["slot"]: e for e in b.list()}
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        stage_ms, total_ms = b.step_timed(args.steps)
    after = {e["slot"]: e for e in b.list()}
    # only the updates every instance actually did are credited: an instance
    # that went non-finite stops stepping and would otherwise count
    credited = 0
    full = 0
    bad = 0
    for slot, e in after.items():
        n = e["steps"] - before[slot]["steps"]
        credited += cells_of[slot] * n
        full += n == args.steps and e["status"] == 0
        bad += e["status"] != 0
    elapsed, credited = aggregate(total_ms / 1e3, credited, dist)
    value = credited / elapsed
    work_check = {"instances": len(after), "stepped_every_update": full, "status_nonzero": bad,
                  "credited_cell_updates": credited}

    # roofline of the stage kernel: algorithmic bytes per launch / mean launch time
    arrays = stage_arrays(1)
    stage_bytes = [cells * FIELDS * BYTES_PER_VALUE * n for n in arrays]
    launches = args.steps * len(arrays)
    achieved = sum(b_ * args.steps for b_ in stage_bytes) / (sum(stage_ms) / 1e3) / 1e9
    peaks, peak_kind = measured_peaks()
    peak = float(peaks.get("hbm_gbs", 6800.0))
    traffic = traffic_from_profiles(st["schedule"][1], cells)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD,
                   "cells": cells, "instances": len(work), "l2": "inputs larger than L2 (%.0f MB per state array)" % (
                       cells * FIELDS * BYTES_PER_VALUE / 1e6),
                   "tile": st["tile"][1], "parallelism": "independent grids per GPU" if world > 1 else "1 GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": traffic,
                     "kernel": ("k_march2 (one warp per strip marching up the rows: PLM + Roe + divergence + RK "
                                "combine + constrainU + dt)" if st["marching"][1] else
                                "k_stage (tile: PLM + Roe + divergence + RK combine + constrainU + dt)"),
                     "bytes_per_launch": sum(stage_bytes) / len(stage_bytes),
                     "ms_per_launch": sum(stage_ms) / launches},
        "gpu_launches": args.steps * (1 + len(arrays)) + 1,
        "clocks": clk.summary(),
        "work_check": work_check,
    }

    if rank == 0 and not args.no_e2e:
        out["e2e"] = e2e_run(hc, ctx, work, inputs, cells, st["schedule"][1])
    if rank == 0:
        # the arithmetic ceilings beside the HBM roofline (the stage kernels
        # are bound by their instruction streams)
        out["alu_peaks"] = {"fp32_tflops": hc.measure_fma("f32"), "fp64_tflops": hc.measure_fma("f64"),
                            "note": "FMA throughput of a kernel of independent FMA chains (hc_measure_fma)"}
        if not args.no_fp64:
            out["fp64"] = fp64_run(hc, ctx, work)
        if not args.no_serving:
            out["serving"] = serving_run(hc, ctx, args.serving_requests)
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(work)
        print(json.dumps(out))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def e2e_run(hc, ctx, work, inputs, cells, schedule, tick=8):
    """The whole job through the public API with host buffers: admit every
    instance from pinned host memory (H2D) in one hc_batch_admit_many call,
    run the configuration's 200 updates, reading every instance's status back
    (D2H) after each call of `tick` updates (the serving loop's tick), fetch
    every final state (D2H) into a second pinned buffer in one
    hc_batch_fetch_many call (the library reads and writes page-locked
    buffers in place over the host link).  The job runs three times and the
    median is reported.  Measured beside it: the same job reading the status
    after every update, and with one admit / fetch call per instance."""
    import ctypes
    nbytes = sum(u.nbytes for u in inputs)
    L = hc.load_library()
    ptr = ctypes.c_void_p()
    hc._check(L.hc_host_alloc(nbytes, ctypes.byref(ptr)))
    optr = ctypes.c_void_p()
    hc._check(L.hc_host_alloc(nbytes, ctypes.byref(optr)))

    def job(views, outs, per_call, many):
        t0 = time.perf_counter()
        b = hc.Batch(ctx, precision="f32", max_slots=len(work), **SCHEME)
        # the schedule the device-timed batch runs (the autotuner's choice for
        # this workload, as a user pins it from the autotuner's cache), set
        # before admission so each instance's tensor maps are encoded once
        b.set_schedule(2, schedule)
        if many:
            b.admit_many([(a, v, math.inf, E2E_STEPS, k) for k, ((a, _), v) in enumerate(zip(work, views))],
                         layout="soa5_f32")
        else:
            for k, ((a, _), v) in enumerate(zip(work, views)):
                b.admit(a, v, t_end=math.inf, max_steps=E2E_STEPS, tag=k, layout="soa5_f32")
        t_admit = time.perf_counter()
        calls = 0
        while b.step(per_call) > 0:
            calls += 1
        t_step = time.perf_counter()
        evs = b.poll()
        if many:
            b.fetch_many([ev["slot"] for ev in evs], "soa5_f32", [outs[ev["tag"]] for ev in evs])
        else:
            for ev in evs:
                b.fetch(ev["slot"], "soa5_f32", out=outs[ev["tag"]])
        t1 = time.perf_counter()
        b.close()
        return t0, t_admit, t_step, t1, evs, calls + 1

    try:
        host = np.frombuffer((ctypes.c_char * nbytes).from_address(ptr.value), dtype=np.float32)
        ohost = np.frombuffer((ctypes.c_char * nbytes).from_address(optr.value), dtype=np.float32)
        views, outs, off = [], [], 0
        for u in inputs:
            views.append(host[off:off + u.size].reshape(u.shape))
            outs.append(ohost[off:off + u.size].reshape(u.shape))
            off += u.size
        for v, u in zip(views, inputs):
            v[...] = u

        def run(per_call, many):
            return job(views, outs, per_call, many)

        # the job three times, the median by its total time reported (the
        # first job of a process also pays the device's first allocations)
        jobs = sorted((run(tick, True) for _ in range(3)), key=lambda j: j[3] - j[0])
        t0, t_admit, t_step, t1, evs, calls = jobs[1]
        job_s = [j[3] - j[0] for j in jobs]
        p0, _, _, p1, _, _ = run(1, True)
        q0, q_admit, q_step, q1, _, _ = run(tick, False)
    finally:
        L.hc_host_free(ptr)
        L.hc_host_free(optr)
    ctl_bytes = STATUS_BYTES_PER_SLOT * len(work)
    # credit the updates each instance reports doing
    credited = sum(work[ev["tag"]][0]["gridSize"][0] * work[ev["tag"]][0]["gridSize"][1] * ev["steps"] for ev in evs)
    got = len(evs)
    check = {"instances": len(work), "finished": got,
             "all_200_updates": sum(1 for ev in evs if ev["steps"] == E2E_STEPS),
             "status_nonzero": sum(1 for ev in evs if ev["status"] != 0), "credited_cell_updates": credited}
    return {"value": credited / (t1 - t0), "unit": UNIT, "work_check": check,
            "h2d_bytes_per_step": nbytes / E2E_STEPS, "d2h_bytes_per_step": nbytes / E2E_STEPS + ctl_bytes * calls / E2E_STEPS,
            "steps": E2E_STEPS, "updates_per_call": tick, "instances_fetched": got, "seconds": t1 - t0,
            "seconds_admit": t_admit - t0, "seconds_steps": t_step - t_admit, "seconds_fetch": t1 - t_step,
            "value_status_every_update": cells * E2E_STEPS / (p1 - p0),
            "value_one_call_per_instance": cells * E2E_STEPS / (q1 - q0),
            "one_call_per_instance_seconds_admit": q_admit - q0, "one_call_per_instance_seconds_fetch": q1 - q_step,
            "jobs_seconds": job_s,
            "note": "median of 3 whole jobs (jobs_seconds: all three, sorted); each job: admission (uploads, one "
                    "admit_many call; page-locked buffers read in place), 200 updates in calls of %d with "
                    "a status read after each call, result fetch (one fetch_many call); value_status_every_update: "
                    "the same job reading the status after every update; value_one_call_per_instance: one admit "
                    "and one fetch call per instance" % tick}


def fp64_run(hc, ctx, work):
    """FP64 reference points on the same workload: the plain FP64 form (one
    solver per grid, kernel-for-kernel, host dt read per update) on a sample,
    and the fused FP64 batch on the whole workload."""
    sample = work[::max(1, len(work) // 64)][:64]
    cells = 0
    t = 0.0
    for a, q in sample:
        s = hc.Solver(ctx, precision="f64 plain", **a)
        s.resetState(hc.quadrant_state(a, q))
        s.update()
        t0 = time.perf_counter()
        for _ in range(3):
            s.update()
        t += time.perf_counter() - t0
        cells += 3 * a["gridSize"][0] * a["gridSize"][1]
        s.close()
    plain = cells / t
    b = hc.Batch(ctx, precision="f64", max_slots=len(work), **SCHEME)
    allcells = 0
    for k, (a, q) in enumerate(work):
        b.admit(a, hc.quadrant_state(a, q), t_end=math.inf, tag=k)
        allcells += a["gridSize"][0] * a["gridSize"][1]
    b.step(1)
    _, ms = b.step_timed(3)
    fused = allcells * 3 / (ms / 1e3)
    b.close()
    # FP32 against FP64 over the configuration's 200 updates, on the first
    # instances of the workload (both batched)
    l1, cells_l1 = [], 0
    got = {}
    for prec in ("f32", "f64"):
        bb = hc.Batch(ctx, precision=prec, max_slots=16, **SCHEME)
        for k, (a, q) in enumerate(work[:16]):
            bb.admit(a, hc.quadrant_state(a, q), t_end=math.inf, max_steps=E2E_STEPS, tag=k)
        out = {}
        while len(out) < min(16, len(work)):
            bb.step(50)
            for ev in bb.poll():
                out[ev["tag"]] = bb.fetch(ev["slot"])
        bb.close()
        got[prec] = out
    for k in got["f32"]:
        l1.append(float(np.mean(np.abs(got["f32"][k][:, 0] - got["f64"][k][:, 0]))))
        cells_l1 += got["f32"][k].shape[0]
    return {"plain_value": plain, "plain_sample": "%d grids (every %dth of the workload, N %d..%d) x 3 updates" % (
                len(sample), max(1, len(work) // 64), min(a["gridSize"][0] for a, _ in sample),
                max(a["gridSize"][0] for a, _ in sample)),
            "fused_batched_value": fused, "unit": UNIT,
            "l1_rho_f32_vs_f64": {"max": max(l1), "mean": float(np.mean(l1)),
                                  "sample": "first %d instances (%d cells), %d updates each, FP64 fused batch as the "
                                            "FP64 reference (bit-identical to the oracle in the parity tests)" % (
                                                len(l1), cells_l1, E2E_STEPS)}}


# ---------------------------------------------------------------------------
# The other configurations: one JSON line each (--workload c1 | c2 | c3 | c5)
# ---------------------------------------------------------------------------

def conf_sod(n=256):
    """1D Sod, x in [-1, 1], gamma 1.4, freeflow, Roe + superbee flux limiter, forward Euler, CFL .5."""
    return dict(dim=1, gridSize=[n], mins=[-1, -1, -1], maxs=[1, 1, 1], boundary="freeflow",
                fluxLimiter="superbee", integrator="forward Euler", cfl=.5, eqnArgs={"heatCapacityRatio": 1.4})


def conf_kh(n=1024):
    """2D Kelvin-Helmholtz on [-.5, .5]^2, periodic, plm cons + MC, Roe, RK3-TVD, CFL .4, gamma 1.4."""
    return dict(dim=2, gridSize=[n, n], mins=[-.5, -.5, -1], maxs=[.5, .5, 1], boundary="periodic",
                usePLM="plm cons", slopeLimiter="monotized central", integrator="Runge-Kutta 3, TVD",
                cfl=.4, eqnArgs={"heatCapacityRatio": 1.4})


def conf_blast(n=256):
    """3D blast on [-1, 1]^3, freeflow, plm cons + minmod, Roe, RK2, CFL .3, gamma 5/3."""
    return dict(dim=3, gridSize=[n, n, n], mins=[-1, -1, -1], maxs=[1, 1, 1], boundary="freeflow",
                usePLM="plm cons", slopeLimiter="minmod", integrator="Runge-Kutta 2",
                cfl=.3, eqnArgs={"heatCapacityRatio": 5. / 3.})


def _cells(args):
    return int(np.prod(args["gridSize"]))


def _scheme(args):
    return {k: args[k] for k in ("usePLM", "slopeLimiter", "fluxLimiter", "integrator", "flux") if k in args}


def l1_density(a, b):
    """Mean |rho_a - rho_b| over the interior cells (AoS-6 states; equal cell volumes)."""
    return float(np.mean(np.abs(a[:, 0] - b[:, 0])))


def batch_solve(hc, ctx, args, cons, precision, t_end=math.inf, max_steps=0, chunk=16, init=None, checkpoints=()):
    """One solve through the batch API, device-timed stage by stage.  Runs
    until the instance reports done (t >= t_end or max_steps updates).
    Returns the final AoS-6 interior state, updates done, device ms and the
    Kahan FP64 sums of the conserved fields before and after; with
    `checkpoints` (update counts) also the state after each of them."""
    tune = None
    if precision == "f32":
        # the schedule is tuned on a throwaway batch of the same grid (tuning
        # advances the solve it times), then read from the cache
        tune = os.path.join(PKG, "_build", "autotune_single.txt")
        tb = hc.Batch(ctx, precision=precision, max_slots=1, **_scheme(args))
        try:
            if init is not None:
                tb.admit_init(args, init[0], t_end=math.inf, tag=0, **init[1])
            else:
                tb.admit(args, cons, t_end=math.inf, tag=0)
            tb.autotune(tune)
        finally:
            tb.close()
    b = hc.Batch(ctx, precision=precision, max_slots=1, **_scheme(args))
    try:
        if init is not None:
            slot = b.admit_init(args, init[0], t_end=t_end, max_steps=max_steps, tag=0, **init[1])
        else:
            slot = b.admit(args, cons, t_end=t_end, max_steps=max_steps, tag=0)
        if tune:
            b.autotune(tune)
        sums0 = b.conservation(slot)
        total_ms = 0.0
        ev = []
        snaps = {}
        done = 0
        for cp in checkpoints:
            if cp > done:
                _, ms = b.step_timed(cp - done)
                total_ms += ms
                done = cp
            snaps[cp] = b.fetch(slot, "aos6")
        while not ev:
            n = chunk if not max_steps else max(1, min(chunk, max_steps))
            _, ms = b.step_timed(n)
            total_ms += ms
            ev = b.poll()
        state = b.fetch(slot, "aos6")
        sums1 = b.conservation(slot)
        return dict(state=state, steps=ev[0]["steps"], t=ev[0]["t"], ms=total_ms, status=ev[0]["status"],
                    sums0=sums0, sums1=sums1, snaps=snaps, schedule=b.stats()["schedule"][args["dim"] - 1])
    finally:
        b.close()


def warm(hc, ctx, args, cons, precision):
    """Loads the kernels of a form (lazy module loading) outside any timed region."""
    batch_solve(hc, ctx, args, cons, precision, max_steps=2, chunk=2)


def plain_rate(hc, ctx, args, cons, updates):
    """The plain FP64 form (kernel per reference kernel, host dt read per update)."""
    s = hc.Solver(ctx, precision="f64 plain", **args)
    try:
        s.resetState(cons)
        s.update()
        t0 = time.perf_counter()
        for _ in range(updates):
            s.update()
        dt = time.perf_counter() - t0
    finally:
        s.close()
    return _cells(args) * updates / dt


def oracle_rate(hc, args, cons, updates):
    """The oracle (the reference's kernels restated in C++, OpenMP on every host core)."""
    import oracle
    oracle.build()
    o = oracle.OracleSolver(args)
    o.reset_state(cons)
    o.update()
    t0 = time.perf_counter()
    for _ in range(updates):
        o.update()
    dt = time.perf_counter() - t0
    return {"value": _cells(args) * updates / dt, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
            "sample": "%d update(s) of the full grid after one untimed update" % updates}


def fp64_first_update_vs_oracle(hc, ctx, args, cons):
    """Max |difference| between the fused FP64 form and the oracle after one
    update of the full-size grid (the parity tests require 0)."""
    import oracle
    oracle.build()
    o = oracle.OracleSolver(args)
    o.reset_state(cons)
    o.update()
    r = batch_solve(hc, ctx, args, cons, "f64", max_steps=1, chunk=1)
    return float(np.max(np.abs(r["state"] - o.get_interior())))


def drift(r):
    s0, s1 = r["sums0"], r["sums1"]
    return {"mass": float((s1[0] - s0[0]) / s0[0]), "energy": float((s1[4] - s0[4]) / s0[4])}


def config_line(name, metric, value, extra):
    out = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": 1, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "data": "synthetic"}
    out.update(extra)
    out["config"] = dict(out.get("config", {}), workload=name)
    print(json.dumps(out))
    return 0


def run_c1(args):
    """1D Sod, 256 cells, to t = 0.2: the plain FP64 form's parity case."""
    import hydrocuda as hc
    import oracle
    from sod_exact import sod_exact
    ctx = hc.Context(0)
    a = conf_sod()
    U0 = hc.sod_state(a)
    oracle.build()
    o = oracle.OracleSolver(a)
    o.reset_state(U0)
    t0 = time.perf_counter()
    o.run_until(0.2)
    t_cpu = time.perf_counter() - t0
    ref = o.get_interior()
    res = {}
    for prec in ("f64 plain", "f64", "f32"):
        s = hc.Solver(ctx, precision=prec, **a)
        s.resetState(U0)
        s.update()          # loads the kernels
        s.resetState(U0)
        s.t = 0.0
        t0 = time.perf_counter()
        n = s.run_until(0.2)
        el = time.perf_counter() - t0
        g = s.getState("aos6")
        res[prec] = {"seconds": el, "updates": n, "max_abs_diff_vs_oracle": float(np.max(np.abs(g - ref))),
                     "l1_rho_vs_oracle": l1_density(g, ref)}
        s.close()
    x = hc.cell_centers(a)[0]
    exact = sod_exact(o.t, x, gamma=1.4)[0]
    plain = res["f64 plain"]
    return config_line("1D Sod 256, Roe + superbee, forward Euler, CFL .5, t = 0.2", "cell-updates/s (FP64 plain)",
                       256 * plain["updates"] / plain["seconds"], {
                           "dtype": "f64", "forms": res,
                           "l1_rho_oracle_vs_exact_sod": float(np.mean(np.abs(ref[:, 0] - exact))),
                           "cpu_baseline": {"value": 256 * plain["updates"] / t_cpu, "unit": UNIT,
                                            "cores": oracle.num_threads(), "kind": "port",
                                            "sample": "the whole run"},
                           "note": "launch-bound at this size; this configuration is the parity case"})


def run_grid_config(name, a, U0, t_end, max_steps, plain_updates, oracle_updates, checkpoints=()):
    import hydrocuda as hc
    ctx = hc.Context(0)
    small = dict(a, gridSize=[min(n, 32) for n in a["gridSize"]])
    U_small = None
    for prec in ("f32", "f64"):
        if U_small is None:
            U_small = initial_for(hc, small)
        warm(hc, ctx, small, U_small, prec)
    r32 = batch_solve(hc, ctx, a, U0, "f32", t_end=t_end, max_steps=max_steps, checkpoints=checkpoints)
    r64 = batch_solve(hc, ctx, a, U0, "f64", t_end=t_end, max_steps=max_steps, checkpoints=checkpoints)
    cells = _cells(a)
    v32 = cells * r32["steps"] / (r32["ms"] / 1e3)
    v64 = cells * r64["steps"] / (r64["ms"] / 1e3)
    n_stages = {"forward Euler": 1, "Runge-Kutta 2": 2, "Runge-Kutta 3, TVD": 3}[a["integrator"]]
    arrays = {1: 2, 2: 5, 3: 8}[n_stages]           # state arrays read + written per update
    gbs = v32 * arrays * FIELDS * BYTES_PER_VALUE / 1e9
    peaks, peak_kind = measured_peaks()
    peak = float(peaks.get("hbm_gbs", 6800.0))
    extra = {
        "dtype": "f32", "steps": r32["steps"], "t_end_reached": r32["t"],
        "ms_total": r32["ms"],
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                     "peak_kind": peak_kind, "traffic": None,
                     "note": "algorithmic bytes: %d state arrays x 5 fields x 4 B per cell-update" % arrays},
        "l1_rho_f32_vs_f64": l1_density(r32["state"], r64["state"]),
        "l1_rho_f32_vs_f64_by_step": {str(k): l1_density(r32["snaps"][k], r64["snaps"][k]) for k in checkpoints},
        "fp64": {"fused_value": v64, "plain_value": plain_rate(hc, ctx, a, U0, plain_updates),
                 "plain_sample": "%d updates" % plain_updates,
                 "fused_first_update_max_abs_diff_vs_oracle": fp64_first_update_vs_oracle(hc, ctx, a, U0)},
        "drift": {"f32": drift(r32), "f64": drift(r64)},
        "status": {"f32": r32["status"], "f64": r64["status"]},
        "cpu_baseline": oracle_rate(hc, a, U0, oracle_updates),
        "config": {"cells": cells, "l2": "inputs %s than L2 (%.0f MB per state array)" % (
            "larger" if cells * 20 > 129e6 else "smaller", cells * 20 / 1e6), "schedule": r32["schedule"]},
    }
    extra["fp64"]["speedup_f32_vs_plain"] = v32 / extra["fp64"]["plain_value"]
    return config_line(name, "cell-updates/s (FP32 fused)", v32, extra)


def initial_for(hc, a):
    if a["dim"] == 2 and a["boundary"] == "periodic":
        return hc.kelvin_helmholtz_state(a, seed=2)
    if a["dim"] == 3:
        return hc.blast_state(a)
    return hc.sod_state(a)


def profile_case(args, a, U0):
    """A short run of the configuration's FP32 stage kernels for an ncu
    capture (not a bench value): one admission, the schedule of --schedule
    (else the autotuner's, from its cache file when the key is there), then
    --warmup + --profile-steps updates.  Prints one line with the device time."""
    import hydrocuda as hc
    ctx = hc.Context(0)
    b = hc.Batch(ctx, precision="f32", max_slots=1, **_scheme(a))
    try:
        b.admit(a, U0, t_end=math.inf, tag=0)
        if args.schedule >= 0:
            b.set_schedule(a["dim"], args.schedule)
        else:
            b.autotune(os.path.join(PKG, "_build", "autotune_single.txt"))
        b.step(args.warmup)
        _, ms = b.step_timed(args.profile_steps)
        print(json.dumps({"profile_case": True, "cells": _cells(a), "steps": args.profile_steps,
                          "schedule": b.stats()["schedule"][a["dim"] - 1], "ms_per_step": ms / args.profile_steps}))
    finally:
        b.close()
    return 0


def run_c2(args):
    import hydrocuda as hc
    a = conf_kh(args.size or 1024)
    if args.profile_steps:
        return profile_case(args, a, hc.kelvin_helmholtz_state(a, seed=2))
    return run_grid_config("2D Kelvin-Helmholtz %d^2, plm cons + MC, Roe, RK3-TVD, CFL .4, periodic, 500 steps"
                           % a["gridSize"][0], a, hc.kelvin_helmholtz_state(a, seed=2), math.inf, 500, 10, 2,
                           checkpoints=(1, 10, 50, 100, 200, 300, 400))


def run_c3(args):
    import hydrocuda as hc
    a = conf_blast(args.size or 256)
    if args.profile_steps:
        return profile_case(args, a, hc.blast_state(a))
    return run_grid_config("3D blast %d^3, plm cons + minmod, Roe, RK2, CFL .3, gamma 5/3, freeflow, t = 0.1"
                           % a["gridSize"][0], a, hc.blast_state(a), 0.1, 0, 3, 1)


class StatePrefetch:
    """Builds request states on worker threads, a bounded number of requests
    ahead of admission, so the serving loop does not wait on host-side set-up
    of inputs (which stands in for clients uploading their states).  Time the
    loop still spends waiting for a state is reported."""

    def __init__(self, reqs, workers=4, ahead=96):
        from concurrent.futures import ThreadPoolExecutor
        self.pool = ThreadPoolExecutor(max_workers=workers)
        self.reqs = reqs
        self.makers = {r.tag: r.cons for r in reqs}
        self.futs = {}
        self.next = 0
        self.taken = 0
        self.ahead = ahead
        self.wait_s = 0.0
        for r in reqs:
            r.cons = (lambda tag: lambda: self.get(tag))(r.tag)
        self._fill()

    def _fill(self):
        while self.next < len(self.reqs) and self.next < self.taken + self.ahead:
            tag = self.reqs[self.next].tag
            self.futs[tag] = self.pool.submit(self.makers.pop(tag))
            self.next += 1

    def get(self, tag):
        t0 = time.perf_counter()
        a = self.futs.pop(tag).result()
        self.wait_s += time.perf_counter() - t0
        self.taken += 1
        self._fill()
        return a

    def close(self):
        self.pool.shutdown(wait=True, cancel_futures=True)


SERVE_SCHEME = dict(usePLM="plm cons", slopeLimiter="minmod", integrator="Runge-Kutta 2")
SERVE_BUDGET = 150 * (1 << 30)


def serving_schedules(hc, ctx):
    """Loads the 1D / 2D / 3D kernels outside any measured run, then tunes the
    stage-kernel schedules once on a calibration batch of requests drawn from
    the serving distribution (another seed): the serving batch starts empty,
    so it has nothing to tune on, and pins these."""
    import serve
    warm_reqs = serve.synthetic_stream(24, rate_hz=1e6, seed=11, scale=0.05)
    wb = hc.Batch(ctx, precision="f32", max_slots=64, hbm_budget=SERVE_BUDGET, **SERVE_SCHEME)
    serve.Server(wb, steps_per_tick=4, keep_results=False).run(warm_reqs)
    wb.close()
    cal = serve.synthetic_stream(48, rate_hz=1e6, seed=13, device_init=True)
    cb = hc.Batch(ctx, precision="f32", max_slots=64, hbm_budget=SERVE_BUDGET, **SERVE_SCHEME)
    for r in cal:
        cb.admit_init(r.args, r.init[0], t_end=math.inf, tag=r.tag, **r.init[1])
    cb.autotune()
    schedules = {d: cb.stats()["schedule"][d - 1] for d in (1, 2, 3)}
    cb.close()
    return schedules


def capacity(reqs, done, wall):
    """The offered load against what was served: the stream's work (cell
    updates of the finished requests) over its arrival span, and over the
    wall time it took to serve."""
    work = sum(r.steps * int(np.prod(r.args["gridSize"])) for r in done)
    span = max(r.arrival for r in reqs) if reqs else 0.0
    offered = work / span if span > 0 else None
    served = work / wall if wall > 0 else None
    return {"cell_updates": work, "arrival_span_s": span, "wall_s": wall,
            "offered_cell_updates_per_s": offered, "served_cell_updates_per_s": served,
            "offered_over_served": offered / served if offered and served else None,
            "note": "offered_over_served > 1: the stream brings more work per second than the GPU completes, "
                    "so requests queue and the latency percentiles are queueing time"}


def serving_run(hc, ctx, requests):
    """A bounded run of the serving configuration's stream (device-built
    initial states) for the bench line: throughput, completed requests per
    second, p50 / p99 time-to-solution, and the capacity arithmetic."""
    import serve
    schedules = serving_schedules(hc, ctx)
    reqs = serve.synthetic_stream(requests, rate_hz=200.0, seed=5, device_init=True)
    b = hc.Batch(ctx, precision="f32", max_slots=1024, hbm_budget=SERVE_BUDGET, **SERVE_SCHEME)
    for d, v in schedules.items():
        b.set_schedule(d, v)
    srv = serve.Server(b, steps_per_tick=8, keep_results=False)
    t0 = time.perf_counter()
    done = srv.run(reqs)
    wall = time.perf_counter() - t0
    b.close()
    return {"requests": len(reqs), "finished": len(done), "wall_s": wall,
            "requests_per_s_completed": len(done) / wall, "arrival_rate_hz": 200.0,
            "cell_updates_per_s": srv.cell_updates / wall, "latency": serve.latency_summary(done),
            "statuses_nonzero": sum(1 for r in done if r.status), "ticks": srv.ticks,
            "host_wait_s": srv.wait_s, "passed_over": srv.passed_over,
            "capacity": capacity(reqs, done, wall),
            "schedules": {str(d): v for d, v in schedules.items()},
            "config": "%d requests of the serving stream (Poisson, mean 200/s, seed 5; 40%% 1D, 45%% 2D, 15%% 3D), "
                      "plm cons + minmod, RK2, CFL .3, 150 GB budget, FP32" % requests}


def run_c5(args):
    """Serving: a Poisson stream (mean 200 requests/s) of 1D / 2D / 3D solves
    through the continuous-batching loop, FP32 bulk, 150 GB HBM budget."""
    import hydrocuda as hc
    import serve
    ctx = hc.Context(0)
    scheme = SERVE_SCHEME
    budget = SERVE_BUDGET
    schedules = serving_schedules(hc, ctx)

    device_init = not args.host_states
    reqs = serve.synthetic_stream(args.requests, rate_hz=200.0, seed=5, lazy=True, layout="soa5_f32",
                                  device_init=device_init)
    # FP64 cross-check sample: the first few requests of each dimension small
    # enough to solve alone in FP64 within seconds, from their FP64 states
    limits = {1: (2, 2048), 2: (4, 200), 3: (2, 72)}
    sample, per = [], {1: 0, 2: 0, 3: 0}
    for r in reqs:
        d = r.args["dim"]
        if per[d] < limits[d][0] and r.args["gridSize"][0] <= limits[d][1]:
            sample.append(r.tag)
            per[d] += 1
    f64_stream = serve.synthetic_stream(args.requests, rate_hz=200.0, seed=5, lazy=True, layout="aos6",
                                        device_init=True)
    sample_in = {r.tag: (r.args, r.init, r.t_end) for r in f64_stream if r.tag in set(sample)}
    pre = StatePrefetch(reqs) if not device_init else None
    b = hc.Batch(ctx, precision="f32", max_slots=1024, hbm_budget=budget, **scheme)
    for d, v in schedules.items():
        b.set_schedule(d, v)
    srv = serve.Server(b, steps_per_tick=8, keep_results=set(sample))
    t0 = time.perf_counter()
    done = srv.run(reqs)
    wall = time.perf_counter() - t0
    if pre:
        pre.close()
    b.close()
    lat = serve.latency_summary(done)
    value = srv.cell_updates / wall
    # served FP32 results against the same requests solved alone in FP64
    l1 = []
    by_tag = {r.tag: r for r in done}
    for tag, (a, init, t_end) in sample_in.items():
        r = by_tag.get(tag)
        if r is None or r.result is None:
            continue
        f64 = batch_solve(hc, ctx, dict(a, **scheme), None, "f64", t_end=t_end, init=init)["state"]
        l1.append(l1_density(r.result, f64))
    # requests that ended non-finite: the same solve alone in FP32 and in FP64
    failed = []
    by_req = {r.tag: r for r in f64_stream}
    for r in done:
        if not r.status:
            continue
        q = by_req[r.tag]
        info = {"tag": r.tag, "dim": q.args["dim"], "n": q.args["gridSize"][0], "init": q.init[0],
                "t_end": q.t_end, "steps": r.steps, "t": r.t}
        for prec in ("f32", "f64"):
            rr = batch_solve(hc, ctx, dict(q.args, **scheme), None, prec, t_end=q.t_end, init=q.init)
            info[prec + "_alone"] = {"status": rr["status"], "steps": rr["steps"]}
        failed.append(info)
    peaks, peak_kind = measured_peaks()
    peak = float(peaks.get("hbm_gbs", 6800.0))
    gbs = value * 5 * FIELDS * BYTES_PER_VALUE / 1e9
    dims = {1: 0, 2: 0, 3: 0}
    for r in reqs:
        dims[r.args["dim"]] += 1
    return config_line(
        "serving: Poisson stream, mean 200 req/s, %d requests (40%% 1D N in [512,65536], 45%% 2D N^2 in "
        "[128^2,1024^2], 15%% 3D N^3 in [64^3,192^3]), t_end ~ U(0.05,0.2), plm cons + minmod, RK2, CFL .3, "
        "150 GB budget" % len(reqs), "cell-updates/s (FP32 served)", value, {
            "dtype": "f32", "requests": len(reqs), "finished": len(done), "wall_s": wall,
            "requests_per_s": len(done) / wall, "latency": lat,
            "statuses_nonzero": sum(1 for r in done if r.status),
            "nonfinite_requests": failed,
            "ticks": srv.ticks, "dims": dims, "host_wait_s": srv.wait_s, "passed_over": srv.passed_over,
            "capacity": capacity(reqs, done, wall),
            "initial_states": "built on the device at admission (hc_batch_admit_init)" if device_init else
                              "built on the host by worker threads, uploaded at admission",
            "host_state_wait_s": pre.wait_s if pre else 0.0,
            "schedules": {"by_dim": {str(d): v for d, v in schedules.items()},
                          "note": "autotuned on a 48-request calibration batch (seed 13), then pinned"},
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "peak_kind": peak_kind, "traffic": None,
                         "note": "algorithmic bytes: RK2, 5 state arrays x 5 fields x 4 B per cell-update"},
            "l1_rho_f32_vs_f64": {"max": max(l1) if l1 else None, "mean": float(np.mean(l1)) if l1 else None,
                                  "sample": "%d requests (1D N <= 2048, 2D N <= 200, 3D N <= 72), each solved "
                                            "alone in FP64 from its FP64 state" % len(l1)},
            "config": {"arrival_rate_hz": 200.0, "seed": 5, "hbm_budget_bytes": budget, "steps_per_tick": 8,
                       "note": "the configuration's stream has 20000 requests; --requests sets the count"}})


if __name__ == "__main__":
    sys.exit(main())
