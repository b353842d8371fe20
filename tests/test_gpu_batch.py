"""Batched and served solves: each result equals the same solve run alone,
admission respects the HBM budget and the slot table, failures are contained
to their own instance."""
import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu


def quad(hc, n, seed, **kw):
    args = cases.c4_quadrant(n, **kw)
    return args, hc.quadrant_state(args, hc.random_quadrants(hc.SplitMix64(seed)))


SCHEME = dict(usePLM="plm cons", slopeLimiter="van Leer (abs)", integrator="Runge-Kutta 2")


def alone(hc, ctx, args, cons, t_end, precision):
    s = hc.Solver(ctx, precision=precision, **args)
    s.resetState(cons)
    n = s.run_until(t_end)
    return s.getState(), n, s.t


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_each_result_same_alone_and_in_the_mix(hc, ctx, precision):
    """Instances of different sizes, admitted at different times, give bit-identical
    results to the same solves run one at a time."""
    specs = [(37, 1, .05), (64, 2, .08), (100, 3, .03), (48, 4, .06), (130, 5, .04)]
    probs = [quad(hc, n, seed) + (t_end,) for n, seed, t_end in specs]
    b = hc.Batch(ctx, precision=precision, max_slots=8, **SCHEME)
    slots = {}
    for k, (args, cons, t_end) in enumerate(probs[:3]):
        slots[k] = b.admit(args, cons, t_end, tag=k)
    b.step(3)                      # the first three are already on the GPU ...
    for k, (args, cons, t_end) in enumerate(probs[3:], start=3):
        slots[k] = b.admit(args, cons, t_end, tag=k)   # ... when these arrive
    results = {}
    for _ in range(10000):
        b.step(4)
        for ev in b.poll():
            results[ev["tag"]] = (b.fetch(ev["slot"]), ev["steps"], ev["t"], ev["status"])
            b.retire(ev["slot"])
        if len(results) == len(probs):
            break
    assert len(results) == len(probs)
    for k, (args, cons, t_end) in enumerate(probs):
        ref, n, t = alone(hc, ctx, args, cons, t_end, precision)
        got, steps, tt, status = results[k]
        assert status == 0
        assert steps == n and tt == t
        np.testing.assert_array_equal(got, ref)


def test_fp64_batch_matches_oracle(hc, ctx):
    b = hc.Batch(ctx, precision="f64", max_slots=4, **SCHEME)
    probs = [quad(hc, n, seed) for n, seed in ((24, 11), (33, 12))]
    for k, (args, cons) in enumerate(probs):
        b.admit(args, cons, t_end=.05, tag=k)
    got = {}
    while len(got) < len(probs):
        b.step(8)
        for ev in b.poll():
            got[ev["tag"]] = (b.fetch(ev["slot"]), ev["t"])
    for k, (args, cons) in enumerate(probs):
        orc = oracle.OracleSolver(args)
        orc.reset_state(cons)
        orc.run_until(.05)
        assert got[k][1] == orc.t
        np.testing.assert_array_equal(got[k][0][:, :5], orc.get_interior()[:, :5])


def test_mixed_dimensions_in_one_batch(hc, ctx):
    scheme = dict(usePLM="plm cons", slopeLimiter="minmod", integrator="Runge-Kutta 2")
    base = dict(mins=[-1, -1, -1], maxs=[1, 1, 1], boundary="freeflow", cfl=.3, **scheme)
    probs = []
    a1 = dict(base, dim=1, gridSize=[300])
    probs.append((a1, hc.sod_state(a1), .05))
    a2 = dict(base, dim=2, gridSize=[70, 50])
    probs.append((a2, hc.quadrant_state(a2, hc.random_quadrants(hc.SplitMix64(3))), .04))
    a3 = dict(base, dim=3, gridSize=[20, 18, 16])
    probs.append((a3, hc.blast_state(a3), .03))
    b = hc.Batch(ctx, precision="f32", max_slots=4, **scheme)
    for k, (args, cons, t_end) in enumerate(probs):
        b.admit(args, cons, t_end, tag=k)
    got = {}
    while len(got) < 3:
        b.step(4)
        for ev in b.poll():
            got[ev["tag"]] = b.fetch(ev["slot"])
    for k, (args, cons, t_end) in enumerate(probs):
        ref, _, _ = alone(hc, ctx, args, cons, t_end, "f32")
        np.testing.assert_array_equal(got[k], ref)


def test_budget_and_slot_admission(hc, ctx):
    args, cons = quad(hc, 64, 1)
    probe = hc.Batch(ctx, precision="f32", max_slots=4, **SCHEME)
    s = probe.admit(args, cons, 1.0)
    one = probe.stats()["bytes_in_use"]
    probe.retire(s)
    assert probe.stats()["bytes_in_use"] == 0
    # budget for two instances: the third is refused, then fits after a retire
    b = hc.Batch(ctx, precision="f32", max_slots=8, hbm_budget=2 * one + one // 2, **SCHEME)
    s0 = b.admit(args, cons, 1.0, tag=0)
    b.admit(args, cons, 1.0, tag=1)
    with pytest.raises(hc.HydroCudaError) as e:
        b.admit(args, cons, 1.0, tag=2)
    assert e.value.code == -4
    assert b.try_admit(args, cons, 1.0, tag=2) is None
    b.retire(s0)
    assert b.try_admit(args, cons, 1.0, tag=2) is not None
    # slot table
    c = hc.Batch(ctx, precision="f32", max_slots=1, **SCHEME)
    c.admit(args, cons, 1.0)
    with pytest.raises(hc.HydroCudaError) as e:
        c.admit(args, cons, 1.0)
    assert e.value.code == -5


def test_nonfinite_request_is_contained(hc, ctx):
    """A request whose host state holds a NaN finishes with HC_ERR_NONFINITE;
    the others in the batch finish normally and match their alone runs."""
    b = hc.Batch(ctx, precision="f32", max_slots=4, **SCHEME)
    good_args, good = quad(hc, 40, 8)
    bad_args, bad = quad(hc, 40, 9)
    bad = bad.copy()
    bad[123, 4] = np.nan
    b.admit(good_args, good, .04, tag=0)
    b.admit(bad_args, bad, .04, tag=1)
    events = {}
    while len(events) < 2:
        b.step(4)
        for ev in b.poll():
            events[ev["tag"]] = ev
            if ev["tag"] == 0:
                events["state"] = b.fetch(ev["slot"])
    assert events[1]["status"] == -6
    assert events[0]["status"] == 0
    ref, _, _ = alone(hc, ctx, good_args, good, .04, "f32")
    np.testing.assert_array_equal(events["state"], ref)


def _variants_from_log(path):
    """(key, [variants]) from an autotune cache file's timing log."""
    key, vs = None, []
    for line in open(path):
        parts = line.split()
        if len(parts) > 3 and parts[0] == "#" and parts[2] == "variant":
            key = parts[1]
            vs.append(int(parts[3]))
    return key, vs


def _solve_all(hc, ctx, probs, scheme, t_end, cache=None):
    b = hc.Batch(ctx, precision="f32", max_slots=4, **scheme)
    try:
        for k, (args, cons) in enumerate(probs):
            b.admit(args, cons, t_end, tag=k)
        if cache:
            b.autotune(cache)
        got = {}
        while len(got) < len(probs):
            b.step(4)
            for ev in b.poll():
                got[ev["tag"]] = b.fetch(ev["slot"])
        return got, b.stats()["tile"]
    finally:
        b.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_every_schedule_same_bits(hc, ctx, tmp_path, dim):
    """Tile shape, segment length and unrolling change the schedule, not the
    arithmetic: every compiled schedule of the FP32 stage kernel gives the same
    bits.  The autotuner times them all once; each is then forced in turn
    through the tuner's cache file."""
    if dim == 2:
        probs = [quad(hc, n, s) for n, s in ((150, 21), (90, 22))]
        scheme, t_end = SCHEME, .03
    else:
        args = cases.c3_blast(28)
        probs = [(args, hc.blast_state(args))]
        scheme = dict(usePLM="plm cons", slopeLimiter="minmod", integrator="Runge-Kutta 2")
        t_end = .02
    base, _ = _solve_all(hc, ctx, probs, scheme, t_end)
    cache = str(tmp_path / "tune.txt")
    tuned, _ = _solve_all(hc, ctx, probs, scheme, t_end, cache)
    key, variants = _variants_from_log(cache)
    assert key and len(variants) >= 2
    for k in range(len(probs)):
        np.testing.assert_array_equal(tuned[k], base[k])
    tiles = set()
    for v in variants:
        with open(cache, "w") as f:
            f.write("%s %d\n" % (key, v))
        got, tile = _solve_all(hc, ctx, probs, scheme, t_end, cache)
        tiles.add(tuple(tile[dim - 1]))
        for k in range(len(probs)):
            np.testing.assert_array_equal(got[k], base[k], err_msg="variant %d" % v)
    assert len(tiles) >= 2       # the cache file did select other tile shapes


def test_served_stream_results_match_alone(hc, ctx):
    """A small Poisson stream through the serving loop: every result equals its alone run."""
    import serve
    reqs = serve.synthetic_stream(12, rate_hz=400.0, seed=5, scale=0.08)
    inputs = {r.tag: (r.args, r.cons.copy(), r.t_end) for r in reqs}
    b = hc.Batch(ctx, precision="f32", max_slots=6, hbm_budget=1 << 30,
                 usePLM="plm cons", slopeLimiter="minmod", integrator="Runge-Kutta 2")
    srv = serve.Server(b, steps_per_tick=4)
    done = srv.run(reqs)
    assert len(done) == len(reqs)
    lat = serve.latency_summary(done)
    assert lat["p99_s"] >= lat["p50_s"] > 0
    for r in done:
        args, cons, t_end = inputs[r.tag]
        ref, n, t = alone(hc, ctx, args, cons, t_end, "f32")
        assert r.status == 0 and r.steps == n
        np.testing.assert_array_equal(r.result, ref)


@pytest.mark.parametrize("layout", ["soa5_f32", "aos6"])
def test_admit_many_and_fetch_many_same_bits_as_one_by_one(hc, ctx, layout):
    """hc_batch_admit_many / hc_batch_fetch_many queue the same uploads,
    set-up launches and copies as the one-at-a-time calls, with one wait:
    the same slots, tags and bits, from pinned and from pageable host memory."""
    import ctypes
    work = [quad(hc, n, 40 + n) for n in (33, 64, 50, 97, 128)]
    conv = (lambda a, c: np.ascontiguousarray(c.reshape(-1, 6)[:, :5].T, dtype=np.float32)) \
        if layout == "soa5_f32" else (lambda a, c: c)
    inputs = [conv(a, c) for a, c in work]
    # pinned copies of the inputs for the batched call
    L = hc.load_library()
    nbytes = sum(u.nbytes for u in inputs)
    ptr = ctypes.c_void_p()
    hc._check(L.hc_host_alloc(nbytes, ctypes.byref(ptr)))
    try:
        host = np.frombuffer((ctypes.c_char * nbytes).from_address(ptr.value), dtype=np.uint8)
        pinned, off = [], 0
        for u in inputs:
            v = host[off:off + u.nbytes].view(u.dtype).reshape(u.shape)
            v[...] = u
            pinned.append(v)
            off += u.nbytes
        got = {}
        for form in ("one", "many"):
            b = hc.Batch(ctx, precision="f32", max_slots=8, **SCHEME)
            if form == "one":
                slots = [b.admit(a, u, 0.02, max_steps=7, tag=10 + k, layout=layout)
                         for k, ((a, _), u) in enumerate(zip(work, inputs))]
            else:
                slots = b.admit_many([(a, u, 0.02, 7, 10 + k) for k, ((a, _), u) in enumerate(zip(work, pinned))],
                                     layout=layout)
            assert slots == list(range(len(work)))
            for _ in range(20):
                if b.step(4) == 0:
                    break
            done = {ev["tag"]: ev["slot"] for ev in b.poll()}
            assert sorted(done) == [10 + k for k in range(len(work))]
            order = [done[10 + k] for k in range(len(work))]
            if form == "one":
                got[form] = [b.fetch(s, layout) for s in order]
            else:
                outs = [np.empty_like(u) for u in inputs]
                got[form] = b.fetch_many(order, layout, outs)
                # the batched fetch into the pinned buffers too
                b.fetch_many(order, layout, pinned)
                for x, y in zip(pinned, outs):
                    np.testing.assert_array_equal(x.reshape(y.shape), y)
            b.close()
        for x, y in zip(got["one"], got["many"]):
            np.testing.assert_array_equal(np.asarray(x).reshape(y.shape), y)
    finally:
        L.hc_host_free(ptr)


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_admit_many_fetch_many_mixed_dims_several_launches(hc, ctx, precision):
    """More instances of one dimension than one batched set-up launch takes
    (120), beside 1D and 3D ones, admitted and fetched in one call each: the
    same bits as one-at-a-time admission and fetch, for each layout."""
    probs = []
    for k in range(125):
        a = cases.c4_quadrant(6 + k % 23)
        probs.append((a, hc.quadrant_state(a, hc.random_quadrants(hc.SplitMix64(300 + k)))))
    for n in (40, 77, 130):
        a = dict(cases.c1_sod(gridSize=n, fluxLimiter="donor cell"), **SCHEME)
        probs.append((a, hc.sod_state(a)))
    for n in (6, 11):
        a = dict(cases.c3_blast(n), **SCHEME)
        probs.append((a, hc.blast_state(a)))
    for layout in ("aos6", "soa5"):
        conv = (lambda c: c) if layout == "aos6" else \
            (lambda c: np.ascontiguousarray(c.reshape(-1, 6)[:, :5].T))
        got = {}
        for form in ("one", "many"):
            b = hc.Batch(ctx, precision=precision, max_slots=len(probs), **SCHEME)
            try:
                if form == "one":
                    slots = [b.admit(a, conv(u), np.inf, max_steps=3, tag=k, layout=layout)
                             for k, (a, u) in enumerate(probs)]
                else:
                    slots = b.admit_many([(a, conv(u), np.inf, 3, k) for k, (a, u) in enumerate(probs)],
                                         layout=layout)
                b.step(3)
                if form == "one":
                    got[form] = [b.fetch(s, layout) for s in slots]
                else:
                    got[form] = b.fetch_many(slots, layout, [np.empty_like(conv(u)) for _, u in probs])
            finally:
                b.close()
        for k, (x, y) in enumerate(zip(got["one"], got["many"])):
            np.testing.assert_array_equal(np.asarray(x).reshape(y.shape), y, err_msg="%s instance %d" % (layout, k))


def test_admit_many_stops_at_the_first_refusal(hc, ctx):
    """A refusal inside admit_many leaves the instances before it admitted
    (reported in the error's .slots) and admits none after it."""
    args, cons = quad(hc, 64, 1)
    probe = hc.Batch(ctx, precision="f32", max_slots=4, **SCHEME)
    probe.admit(args, cons, 1.0)
    one = probe.stats()["bytes_in_use"]
    probe.close()
    b = hc.Batch(ctx, precision="f32", max_slots=8, hbm_budget=2 * one + one // 2, **SCHEME)
    with pytest.raises(hc.HydroCudaError) as e:
        b.admit_many([(args, cons, 1.0, 0, k) for k in range(4)])
    assert e.value.code == -4
    assert e.value.slots == [0, 1]
    assert b.stats()["occupied"] == 2
    assert b.stats()["bytes_in_use"] == 2 * one
    # an unknown slot in fetch_many is refused before anything is copied
    with pytest.raises(hc.HydroCudaError) as e:
        b.fetch_many([0, 5])
    assert e.value.code == -8
    out = b.fetch_many([1, 0])
    np.testing.assert_array_equal(out[0], b.fetch(1))
    b.close()
