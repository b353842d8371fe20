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
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "hydro-cl-lua_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
for p in (PKG, ORACLE_DIR):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "cell-updates/s (FP32 batched)"
UNIT = "cell-updates/s"
COUNT = 512
E2E_STEPS = 200          # the configuration's 200 steps per instance
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
        self.path = os.path.join(ROOT, "gpurun_out", "clocks_bench.csv") if os.path.isdir(
            os.path.join(ROOT, "gpurun_out")) else "/tmp/hc_clocks_%d.csv" % os.getpid()

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


def traffic_from_profiles(cells, stage_bytes_list):
    """DRAM bytes per stage launch from the committed ncu summary, scaled to this
    workload by interior cells, or None."""
    path = os.path.join(ROOT, "profiles", "k_stage_2d_plm_f32_c4.md")
    try:
        text = open(path).read()
    except Exception:
        return None
    import re
    m = re.search(r"dram_bytes_per_cell_stage:\s*([0-9.eE+-]+)", text)
    if not m:
        return None
    return float(m.group(1)) * cells


def cpu_baseline(work, budget_s=12.0, threads=None):
    """The oracle (C++ restatement, OpenMP on all host cores) on a bounded
    sample of the workload: whole updates of instances in workload order
    until the time budget is spent."""
    import hydrocuda as hc
    import oracle
    oracle.build()
    n_thr = oracle.num_threads()
    cells = 0
    t_total = 0.0
    used = 0
    for args, q in work:
        s = oracle.OracleSolver(args)
        s.reset_state(hc.quadrant_state(args, q))
        s.update()   # first-touch warm-up of this instance
        t0 = time.perf_counter()
        s.update()
        t_total += time.perf_counter() - t0
        cells += args["gridSize"][0] * args["gridSize"][1]
        used += 1
        if t_total >= budget_s:
            break
    return {"value": cells / t_total, "unit": UNIT, "cores": n_thr, "kind": "port",
            "sample": "%d of %d instances, one Runge-Kutta 2 update each (%d cells), %.1f s" % (used, len(work), cells, t_total)}


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
    budget_cells = 6_000_000   # about one to a few seconds of CPU work per step
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
        "config": {"workload": "batched 2D Euler quadrants, 512 grids N in [64,512], plm cons + van Leer, Roe, RK2, CFL .475",
                   "sample": sample},
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
    ap.add_argument("--count", type=int, default=COUNT,
                    help="instances (the configuration has 512; fewer only for profiling a small case)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)

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
    for k, ((a, _), u) in enumerate(zip(work, inputs)):
        b.admit(a, u, t_end=math.inf, tag=k, layout="soa5_f32")
    if not args.no_autotune:
        b.autotune(os.path.join(PKG, "_build", "autotune.txt"))
    st = b.stats()
    b.step(args.warmup)

    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        stage_ms, total_ms = b.step_timed(args.steps)
    elapsed = total_ms / 1e3
    if dist:
        import torch
        t = torch.tensor([elapsed], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    value = world * cells * args.steps / elapsed

    # roofline of the stage kernel: algorithmic bytes per launch / mean launch time
    arrays = stage_arrays(1)
    stage_bytes = [cells * FIELDS * BYTES_PER_VALUE * n for n in arrays]
    launches = args.steps * len(arrays)
    achieved = sum(b_ * args.steps for b_ in stage_bytes) / (sum(stage_ms) / 1e3) / 1e9
    peaks, peak_kind = measured_peaks()
    peak = float(peaks.get("hbm_gbs", 6800.0))
    traffic = traffic_from_profiles(cells, stage_bytes)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batched 2D Euler: 512 quadrant Riemann problems, N log-uniform in [64,512] (seed 4), "
                               "plm cons + van Leer, Roe, RK2, CFL .475, gamma 1.4, freeflow",
                   "cells": cells, "instances": len(work), "l2": "inputs larger than L2 (%.0f MB per state array)" % (
                       cells * FIELDS * BYTES_PER_VALUE / 1e6),
                   "tile": st["tile"][1], "parallelism": "independent grids per GPU" if world > 1 else "1 GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": traffic,
                     "kernel": "k_stage (fused PLM + Roe + divergence + RK combine + constrainU + dt)",
                     "bytes_per_launch": sum(stage_bytes) / len(stage_bytes),
                     "ms_per_launch": sum(stage_ms) / launches},
        "gpu_launches": args.steps * (1 + len(arrays)) + 1,
        "clocks": clk.summary(),
    }

    if rank == 0 and not args.no_e2e:
        out["e2e"] = e2e_run(hc, ctx, work, inputs, cells)
    if rank == 0:
        if not args.no_fp64:
            out["fp64"] = fp64_run(hc, ctx, work)
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(work)
        print(json.dumps(out))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def e2e_run(hc, ctx, work, inputs, cells):
    """The whole job through the public API with host buffers: admit every
    instance from pinned host memory (H2D), run the configuration's 200
    updates reading each update's per-instance status back (D2H), fetch every
    final state (D2H)."""
    import ctypes
    nbytes = sum(u.nbytes for u in inputs)
    L = hc.load_library()
    ptr = ctypes.c_void_p()
    hc._check(L.hc_host_alloc(nbytes, ctypes.byref(ptr)))
    try:
        host = np.frombuffer((ctypes.c_char * nbytes).from_address(ptr.value), dtype=np.float32)
        views, off = [], 0
        for u in inputs:
            v = host[off:off + u.size].reshape(u.shape)
            v[...] = u
            views.append(v)
            off += u.size
        t0 = time.perf_counter()
        b = hc.Batch(ctx, precision="f32", max_slots=len(work), **SCHEME)
        for k, ((a, _), v) in enumerate(zip(work, views)):
            b.admit(a, v, t_end=math.inf, max_steps=E2E_STEPS, tag=k, layout="soa5_f32")
        steps = 0
        while b.step(1) > 0:
            steps += 1
        got = 0
        for ev in b.poll():
            views[ev["tag"]][...] = b.fetch(ev["slot"], "soa5_f32")
            got += 1
        t1 = time.perf_counter()
        b.close()
    finally:
        L.hc_host_free(ptr)
    ctl_bytes = 48 * len(work)
    return {"value": cells * E2E_STEPS / (t1 - t0), "unit": UNIT,
            "h2d_bytes_per_step": nbytes / E2E_STEPS, "d2h_bytes_per_step": nbytes / E2E_STEPS + ctl_bytes,
            "steps": E2E_STEPS, "instances_fetched": got, "seconds": t1 - t0,
            "note": "whole job per call: admission (uploads), 200 updates with a per-update status read, result fetch"}


def fp64_run(hc, ctx, work):
    """FP64 reference points on the same workload: the plain FP64 form (one
    solver per grid, kernel-for-kernel, host dt read per update) on a sample,
    and the fused FP64 batch on the whole workload."""
    sample = work[:8]
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
    return {"plain_value": plain, "plain_sample": "%d grids x 3 updates" % len(sample),
            "fused_batched_value": fused, "unit": UNIT}


if __name__ == "__main__":
    sys.exit(main())
