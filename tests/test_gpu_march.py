"""The 2D marching stage kernel (one warp per 30-column strip marching up a
segment of rows) against the tile kernel: the same arithmetic, so the same
bits, on grids whose sides cut strips and segments anywhere, on every boundary
kind, every explicit integrator the batch runs (stored derivatives included)
and compiled-in as well as run-time slope limiters; and against the FP64
oracle within the FP32 tolerance."""
import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu

MARCH = 16      # the marching schedule's number
TILE = 10       # a tile schedule with every compiled-in limiter


@pytest.fixture(autouse=True)
def full_segments(monkeypatch):
    """The schedule's own segment length: these small batches would otherwise
    be cut into short balanced segments (tested on their own below)."""
    monkeypatch.setenv("HC_MARCH_SEGMENT", "100000")


def _run(hc, ctx, probs, scheme, schedule, steps):
    b = hc.Batch(ctx, precision="f32", max_slots=len(probs), **scheme)
    try:
        for k, (args, cons) in enumerate(probs):
            b.admit(dict(args, **scheme), cons, t_end=np.inf, max_steps=steps, tag=k)
        b.set_schedule(2, schedule)
        assert b.stats()["schedule"][1] == schedule
        got = {}
        for _ in range(1000):
            b.step(4)
            for ev in b.poll():
                assert ev["status"] == 0, ev
                assert ev["steps"] == steps
                got[ev["tag"]] = b.fetch(ev["slot"])
            if len(got) == len(probs):
                break
        return [got[k] for k in range(len(probs))]
    finally:
        b.close()


def _quad(hc, nx, ny, seed, **kw):
    a = cases.c4_quadrant(nx, **kw)
    a["gridSize"] = [nx, ny]
    return a, hc.quadrant_state(a, hc.random_quadrants(hc.SplitMix64(seed)))


SHAPES = [(2, 2), (3, 5), (29, 31), (30, 64), (31, 65), (61, 63), (62, 130), (97, 7), (150, 129)]


@pytest.mark.parametrize("limiter", ["van Leer (abs)", "minmod", "monotized central", "superbee", "van Albada 1"])
def test_march_equals_tile(hc, ctx, limiter):
    probs = [_quad(hc, nx, ny, 40 + k) for k, (nx, ny) in enumerate(SHAPES)]
    scheme = dict(usePLM="plm cons", slopeLimiter=limiter, integrator="Runge-Kutta 2")
    tile = TILE if limiter != "van Albada 1" else 0
    a = _run(hc, ctx, probs, scheme, MARCH, 6)
    b = _run(hc, ctx, probs, scheme, tile, 6)
    for k, (x, y) in enumerate(zip(a, b)):
        np.testing.assert_array_equal(x, y, err_msg="shape %s" % (SHAPES[k],))


@pytest.mark.parametrize("integrator", ["forward Euler", "Runge-Kutta 3, TVD", "Runge-Kutta 4",
                                        "Runge-Kutta 2 Heun", "Runge-Kutta 4, TVD"])
def test_march_equals_tile_integrators(hc, ctx, integrator):
    probs = [_quad(hc, nx, ny, 60 + k) for k, (nx, ny) in enumerate([(45, 70), (64, 33), (5, 90)])]
    scheme = dict(usePLM="plm cons", slopeLimiter="van Leer (abs)", integrator=integrator)
    a = _run(hc, ctx, probs, scheme, MARCH, 5)
    b = _run(hc, ctx, probs, scheme, TILE, 5)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


BOUNDARIES = [
    "periodic",
    "mirror",
    "linear",
    "quadratic",
    {"xmin": "mirror", "xmax": "freeflow", "ymin": "linear", "ymax": "periodic"},
]


@pytest.mark.parametrize("bi", range(len(BOUNDARIES)))
def test_march_equals_tile_boundaries(hc, ctx, bi):
    bc = BOUNDARIES[bi]
    if isinstance(bc, dict):
        # periodic on one side needs periodic on the other
        bc = dict(bc, ymin="periodic")
    probs = []
    for k, (nx, ny) in enumerate([(33, 40), (70, 66), (4, 6)]):
        a, u = _quad(hc, nx, ny, 80 + k)
        a["boundary"] = bc
        probs.append((a, u))
    scheme = dict(usePLM="plm cons", slopeLimiter="monotized central", integrator="Runge-Kutta 2")
    a = _run(hc, ctx, probs, scheme, MARCH, 5)
    b = _run(hc, ctx, probs, scheme, TILE, 5)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("schedule", [17, 18, 19, 20, 21])
def test_march_occupancy_variants(hc, ctx, schedule):
    """The same kernel compiled for 3 and 2 CTAs per SM, and with segments of 16, 32 and 128 rows."""
    probs = [_quad(hc, nx, ny, 90 + k) for k, (nx, ny) in enumerate([(61, 63), (150, 129)])]
    scheme = dict(usePLM="plm cons", slopeLimiter="van Leer (abs)", integrator="Runge-Kutta 2")
    a = _run(hc, ctx, probs, scheme, schedule, 6)
    b = _run(hc, ctx, probs, scheme, TILE, 6)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_march_against_oracle(hc, ctx):
    """FP32 marching kernel against the FP64 oracle: density L1 <= 1e-5 after 20 updates."""
    a, u = _quad(hc, 123, 77, 5)
    scheme = dict(usePLM="plm cons", slopeLimiter="van Leer (abs)", integrator="Runge-Kutta 2")
    got = _run(hc, ctx, [(a, u)], scheme, MARCH, 20)[0]
    o = oracle.OracleSolver(a)
    o.reset_state(u)
    for _ in range(20):
        o.update()
    ref = o.get_interior()
    l1 = float(np.mean(np.abs(got[:, 0] - ref[:, 0])))
    assert l1 <= 1e-5, l1


@pytest.mark.parametrize("seg", ["0", "1", "5", "23"])
def test_march_segment_lengths(hc, ctx, monkeypatch, seg):
    """Segments shorter than the schedule's (0: the balanced length the batch
    picks for a launch that would leave warps idle, here a few rows) give the
    same bits as the tile kernel."""
    monkeypatch.setenv("HC_MARCH_SEGMENT", seg)
    probs = [_quad(hc, nx, ny, 95 + k) for k, (nx, ny) in enumerate([(61, 63), (150, 129), (31, 5), (2, 2)])]
    scheme = dict(usePLM="plm cons", slopeLimiter="van Leer (abs)", integrator="Runge-Kutta 3, TVD")
    a = _run(hc, ctx, probs, scheme, 17, 5)
    b = _run(hc, ctx, probs, scheme, TILE, 5)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
