"""Continuous-batching request loop over hc_batch (host side).

Requests (Euler solves of any dimension and size, each with its own end time)
arrive over time.  The loop admits arrived requests against the batch's HBM budget and slot
table (in arrival order, passing over one that does not fit unless it has
waited too long), advances all live solves together with
``hc_batch_step_async`` / ``hc_batch_wait`` (each with its own CFL dt, on the
device; admissions are issued while a tick runs), and as solves finish it
fetches their states, retires their slots (returning their bytes to the
budget) and records time-to-solution.  Requests that arrive while others
are on the GPU are admitted as soon as memory and a slot free up, so their
work overlaps on the device with the solves already running.

The reference has no serving layer: each hydro-cl-lua App steps its solvers in
its own loop (hydro/app.lua:1573-1750).  One request here is one App run to
exitTime (the exit test precedes each update, so the last update overshoots).
"""
import collections
import time

import numpy as np

import hydrocuda


class Request:
    """One solve: `cons` is the initial interior state in `layout`, or a
    callable returning it (called once, when the request is first offered for
    admission, so a long stream need not hold every state in host memory), or
    None with `init` = (kind, params) naming an initial condition the library
    builds on the device (hydrocuda.make_init)."""
    __slots__ = ("arrival", "args", "cons", "t_end", "tag", "layout", "init", "admitted", "finished", "steps", "t",
                 "status", "result")

    def __init__(self, arrival, args, cons, t_end, tag, layout="aos6", init=None):
        self.arrival = float(arrival)
        self.args = args
        self.cons = cons
        self.t_end = float(t_end)
        self.tag = int(tag)
        self.layout = layout
        self.init = init
        self.admitted = None
        self.finished = None
        self.steps = 0
        self.t = 0.0
        self.status = None
        self.result = None


class Server:
    """Drives one hc_batch with a stream of requests.

    steps_per_tick: updates per tick between admission / poll passes (larger
    values amortise host round trips, smaller ones admit and retire sooner).
    keep_results: fetch the final state of every solve (True), of none
    (False), or of the requests whose tags are in the given set.

    Admission backfills: the arrived requests are offered in arrival order and
    one that does not fit (HBM budget or slot table) is passed over for now,
    so smaller requests behind it still start.  A request that has waited
    longer than age_cap_s is not passed over: admission stops at it until
    retirements free enough memory, so a large request is not starved.  At
    most max_refusals refusals end the pass (each is a host call).

    async_ticks: each tick's updates are queued first (hc_batch_step_async),
    then the arrived requests are admitted while they run (the admissions'
    set-up launches queue behind them), then the tick is waited for and the
    finished solves are polled, fetched and retired.
    """

    def __init__(self, batch, steps_per_tick=8, keep_results=True, result_layout="aos6", age_cap_s=1.0,
                 max_refusals=8, async_ticks=True):
        self.batch = batch
        self.steps_per_tick = int(steps_per_tick)
        self.keep_results = keep_results
        self.result_layout = result_layout
        self.age_cap_s = float(age_cap_s)
        self.max_refusals = int(max_refusals)
        self.async_ticks = bool(async_ticks)
        self.by_tag = {}
        self.slot_of = {}
        self.ticks = 0
        self.cell_updates = 0
        self.wait_s = 0.0          # host time spent waiting for the device's ticks
        self.passed_over = 0       # admissions that went ahead of an older waiting request

    def _admit(self, waiting, clock, live, cells_of):
        """One admission pass over the waiting requests; returns how many started."""
        i, refused, started = 0, 0, 0
        while i < len(waiting) and refused < self.max_refusals:
            r = waiting[i]
            if r.init is not None:
                slot = self.batch.try_admit_init(r.args, r.init[0], r.t_end, tag=r.tag, **r.init[1])
            else:
                if callable(r.cons):
                    r.cons = r.cons()
                slot = self.batch.try_admit(r.args, r.cons, r.t_end, tag=r.tag, layout=r.layout)
            if slot is None:
                if live + started == 0:
                    raise RuntimeError("request %d does not fit an empty batch" % r.tag)
                refused += 1
                if clock() - r.arrival > self.age_cap_s:
                    break          # the oldest starving request keeps its place
                i += 1
                continue
            del waiting[i]
            if i > 0:
                self.passed_over += 1
            r.admitted = clock()
            r.cons = None
            self.by_tag[r.tag] = r
            self.slot_of[r.tag] = slot
            cells_of[r.tag] = hydrocuda.interior_count(self.batch.slot_desc[slot])
            started += 1
        return started

    def run(self, requests, clock=None, sleep=None, max_wall=None):
        """Serves `requests` (sorted by arrival time, seconds from start).

        clock(): seconds since start; defaults to the wall clock.  Returns the
        list of finished requests with latency fields filled in.
        """
        t0 = time.perf_counter()
        clock = clock or (lambda: time.perf_counter() - t0)
        sleep = sleep or time.sleep
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        waiting = []
        live = 0
        done = []
        cells_of = {}
        while pending or waiting or live:
            now = clock()
            if max_wall is not None and now > max_wall:
                break
            while pending and pending[0].arrival <= now:
                waiting.append(pending.popleft())
            ticking = live > 0
            if ticking and self.async_ticks:
                self.batch.step_async(self.steps_per_tick)
            started = self._admit(waiting, clock, live, cells_of)
            if ticking:
                w0 = time.perf_counter()
                if self.async_ticks:
                    self.batch.wait()
                else:
                    self.batch.step(self.steps_per_tick)
                self.wait_s += time.perf_counter() - w0
                self.ticks += 1
                for ev in self.batch.poll():
                    r = self.by_tag.pop(ev["tag"])
                    slot = self.slot_of.pop(r.tag)
                    r.steps = ev["steps"]
                    r.t = ev["t"]
                    r.status = ev["status"]
                    keep = self.keep_results
                    if keep is True or (keep and not isinstance(keep, bool) and r.tag in keep):
                        r.result = self.batch.fetch(slot, self.result_layout)
                    self.batch.retire(slot)
                    r.finished = clock()
                    self.cell_updates += r.steps * cells_of.pop(r.tag)
                    live -= 1
                    done.append(r)
            live += started
            if not ticking and not started and pending and not waiting:
                sleep(max(0.0, pending[0].arrival - clock()))
        return done


def latency_summary(done):
    lat = np.array([r.finished - r.arrival for r in done])
    return {
        "count": int(lat.size),
        "p50_s": float(np.percentile(lat, 50)) if lat.size else None,
        "p99_s": float(np.percentile(lat, 99)) if lat.size else None,
        "mean_s": float(lat.mean()) if lat.size else None,
    }


def _in_layout(cons, layout):
    if layout == "aos6":
        return cons
    a = np.ascontiguousarray(cons[:, :5].T)
    return a.astype(np.float32) if layout == "soa5_f32" else a


def synthetic_stream(count, rate_hz, seed=5, scale=1.0, gamma=1.4, lazy=False, layout="aos6", device_init=False):
    """Poisson arrivals (mean rate_hz) of 1D / 2D / 3D Euler solves.

    40 % 1D with N ~ logU[512, 65536], 45 % 2D with N ~ logU[128, 1024],
    15 % 3D with N ~ logU[64, 192] (N scaled by `scale` for reduced runs);
    the initial state is uniformly one of Sod (along x), blast, quadrant;
    t_end ~ U(0.05, 0.2).  Scheme: plm cons + minmod, Runge-Kutta 2, CFL 0.3.
    lazy: each request carries a callable that builds its state on demand
    (every random draw is still made here, in stream order).  layout: the
    state layout handed to admission ("aos6", "soa5", "soa5_f32").
    device_init: each request names its initial condition instead, and the
    library builds the (identical) state on the device at admission.
    """
    rng = hydrocuda.SplitMix64(seed)
    t = 0.0
    out = []
    for tag in range(count):
        t += -np.log(1.0 - rng.uniform()) / rate_hz
        u = rng.uniform()
        if u < .40:
            dim, lo, hi = 1, 512, 65536
        elif u < .85:
            dim, lo, hi = 2, 128, 1024
        else:
            dim, lo, hi = 3, 64, 192
        n = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi))) * scale))
        n = max(n, 8)
        kind = int(rng.uniform() * 3)
        t_end = rng.uniform(0.05, 0.2)
        args = dict(dim=dim, gridSize=[n] * dim, mins=[-1, -1, -1], maxs=[1, 1, 1], boundary="freeflow",
                    usePLM="plm cons", slopeLimiter="minmod", integrator="Runge-Kutta 2", cfl=.3,
                    eqnArgs={"heatCapacityRatio": gamma})
        if kind == 0 or dim == 1 and kind == 2:
            make = (lambda a: lambda: hydrocuda.sod_state(a))(args)
            init = ("sod", {})
        elif kind == 1 or dim != 2:
            make = (lambda a: lambda: hydrocuda.blast_state(a))(args)
            init = ("blast", {})
        else:
            q = hydrocuda.random_quadrants(rng)
            make = (lambda a, q: lambda: hydrocuda.quadrant_state(a, q))(args, q)
            init = ("quadrant", {"q": q})
        if device_init:
            out.append(Request(t, args, None, t_end, tag, init=init))
            continue
        build = (lambda m: lambda: _in_layout(m(), layout))(make)
        out.append(Request(t, args, build if lazy else build(), t_end, tag, layout))
    return out
