"""The 3D marching stage kernel (one CTA per 30-column x-y tile marching up a
segment of planes along z) against the 3D tile kernel: the same arithmetic,
so the same bits, on grids whose sides cut strips, tiles and segments
anywhere, on every boundary kind, every explicit integrator the batch runs
(stored derivatives included), compiled-in and run-time slope limiters, and
each compiled tile shape; and against the FP64 oracle within the FP32
tolerance."""
import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu

MARCH = 7       # 12 warps, segments of 32 planes
TILE = 0        # the 3D tile schedule with every compiled-in limiter


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
        b.set_schedule(3, schedule)
        assert b.stats()["schedule"][2] == schedule
        got = {}
        for _ in range(1000):
            b.step(4)
            for ev in b.poll():
                # a solve that turns non-finite stops with its status (the
                # same update in both kernels); the others run every update
                st = b.fetch(ev["slot"]) if ev["status"] == 0 else None
                got[ev["tag"]] = (ev["status"], ev["steps"], st)
            if len(got) == len(probs):
                break
        return [got[k] for k in range(len(probs))]
    finally:
        b.close()


def _same(a, b, what=""):
    assert a[:2] == b[:2], (what, a[:2], b[:2])
    if a[2] is not None:
        np.testing.assert_array_equal(a[2], b[2], err_msg=str(what))


def _blast(hc, nx, ny, nz, **kw):
    a = cases.c3_blast(nx, **kw)
    a["gridSize"] = [nx, ny, nz]
    return a, hc.blast_state(a)


SHAPES = [(2, 2, 2), (3, 5, 4), (12, 10, 14), (29, 11, 33), (30, 20, 32), (31, 21, 65), (61, 9, 40), (5, 37, 3)]


@pytest.mark.parametrize("limiter", ["minmod", "van Leer (abs)", "monotized central", "superbee", "van Albada 1"])
def test_march3_equals_tile(hc, ctx, limiter):
    probs = [_blast(hc, *s) for s in SHAPES]
    scheme = dict(usePLM="plm cons", slopeLimiter=limiter, integrator="Runge-Kutta 2")
    a = _run(hc, ctx, probs, scheme, MARCH, 4)
    b = _run(hc, ctx, probs, scheme, TILE, 4)
    for k, (x, y) in enumerate(zip(a, b)):
        _same(x, y, "shape %s" % (SHAPES[k],))
    if limiter != "van Albada 1":
        # (r^2 + r) / (r^2 + 1) is inf / inf where the left difference is
        # zero: most of these blasts turn non-finite under it, in both kernels
        assert all(x[0] == 0 for x in a)


@pytest.mark.parametrize("integrator", ["forward Euler", "Runge-Kutta 3, TVD", "Runge-Kutta 4",
                                        "Runge-Kutta 2 Heun", "Runge-Kutta 2, TVD"])
def test_march3_equals_tile_integrators(hc, ctx, integrator):
    probs = [_blast(hc, *s) for s in [(33, 14, 35), (8, 24, 9)]]
    scheme = dict(usePLM="plm cons", slopeLimiter="minmod", integrator=integrator)
    a = _run(hc, ctx, probs, scheme, MARCH, 4)
    b = _run(hc, ctx, probs, scheme, TILE, 4)
    for x, y in zip(a, b):
        _same(x, y)
        assert x[0] == 0


BOUNDARIES = [
    "periodic",
    "mirror",
    "linear",
    "quadratic",
    {"xmin": "mirror", "xmax": "freeflow", "ymin": "periodic", "ymax": "periodic", "zmin": "linear",
     "zmax": "mirror"},
]


@pytest.mark.parametrize("bi", range(len(BOUNDARIES)))
def test_march3_equals_tile_boundaries(hc, ctx, bi):
    probs = []
    for s in [(31, 12, 34), (4, 6, 5)]:
        a, u = _blast(hc, *s)
        a["boundary"] = BOUNDARIES[bi]
        probs.append((a, u))
    scheme = dict(usePLM="plm cons", slopeLimiter="monotized central", integrator="Runge-Kutta 2")
    a = _run(hc, ctx, probs, scheme, MARCH, 4)
    b = _run(hc, ctx, probs, scheme, TILE, 4)
    for x, y in zip(a, b):
        _same(x, y)
        assert x[0] == 0


@pytest.mark.parametrize("schedule", [8, 9, 10, 11])
def test_march3_shape_variants(hc, ctx, schedule):
    """Segments of 64 planes; 16-warp tiles; 8-warp tiles at 2 CTAs per SM; 14-warp tiles."""
    probs = [_blast(hc, *s) for s in [(61, 29, 70), (30, 15, 130), (7, 6, 5)]]
    scheme = dict(usePLM="plm cons", slopeLimiter="minmod", integrator="Runge-Kutta 2")
    a = _run(hc, ctx, probs, scheme, schedule, 4)
    b = _run(hc, ctx, probs, scheme, TILE, 4)
    for x, y in zip(a, b):
        _same(x, y)
        assert x[0] == 0


def test_march3_against_oracle(hc, ctx):
    """FP32 marching kernel against the FP64 oracle: density L1 <= 1e-5 after 8 updates."""
    a, u = _blast(hc, 40, 33, 36)
    scheme = dict(usePLM="plm cons", slopeLimiter="minmod", integrator="Runge-Kutta 2")
    status, steps, got = _run(hc, ctx, [(a, u)], scheme, MARCH, 8)[0]
    assert status == 0 and steps == 8
    o = oracle.OracleSolver(a)
    o.reset_state(u)
    for _ in range(8):
        o.update()
    l1 = float(np.mean(np.abs(got[:, 0] - o.get_interior()[:, 0])))
    assert l1 <= 1e-5, l1


@pytest.mark.parametrize("seg", ["0", "1", "6", "19"])
def test_march3_segment_lengths(hc, ctx, monkeypatch, seg):
    """Segments shorter than the schedule's (0: the balanced length the batch
    picks for a launch that would leave CTAs idle, here a few planes) give
    the same bits as the tile kernel."""
    monkeypatch.setenv("HC_MARCH_SEGMENT", seg)
    probs = [_blast(hc, *s) for s in [(31, 21, 65), (12, 10, 14), (2, 2, 2)]]
    scheme = dict(usePLM="plm cons", slopeLimiter="minmod", integrator="Runge-Kutta 3, TVD")
    a = _run(hc, ctx, probs, scheme, 10, 4)
    b = _run(hc, ctx, probs, scheme, TILE, 4)
    for k, (x, y) in enumerate(zip(a, b)):
        _same(x, y, k)
