"""The bounded-wait failure path of the stage kernels, made to run out on
purpose without a fault: with HC_TEST_FORCE_TIMEOUT=1 set when a batch is
created, the first wait for each tile's TMA copy counts as run out; the kernel
records the timeout, waits (bounded again) for its copy to land so its shared
memory is not released under it, and returns.  The step reports
HC_ERR_TIMEOUT, the slot is marked, and the same context then steps a fresh
batch normally."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

SCHEME = dict(usePLM="plm cons", slopeLimiter="van Leer (abs)", integrator="Runge-Kutta 2")


def _prob(hc, dim, seed):
    if dim == 3:
        a = cases.c3_blast(20, slopeLimiter="van Leer (abs)")
        a["gridSize"] = [33, 20, 40]
        return a, hc.blast_state(a)
    a = cases.c4_quadrant(70)
    return a, hc.quadrant_state(a, hc.random_quadrants(hc.SplitMix64(seed)))


# the 2D tile and marching kernels, the 3D marching kernel
@pytest.mark.parametrize("dim,schedule", [(2, 0), (2, 17), (3, 7)])
def test_forced_timeout_is_reported_and_the_context_stays_usable(hc, ctx, monkeypatch, dim, schedule):
    a, u = _prob(hc, dim, 3)
    monkeypatch.setenv("HC_TEST_FORCE_TIMEOUT", "1")
    b = hc.Batch(ctx, precision="f32", max_slots=2, **SCHEME)
    monkeypatch.delenv("HC_TEST_FORCE_TIMEOUT")
    try:
        b.admit(a, u, t_end=np.inf, max_steps=3, tag=7)
        b.set_schedule(dim, schedule)
        with pytest.raises(hc.HydroCudaError) as e:
            b.step(1)
        assert e.value.code == -7              # HC_ERR_TIMEOUT
        assert b.list()[0]["status"] == -7
    finally:
        b.close()
    # a batch created without the knob, in the same context, steps and matches
    # the same solve run alone
    b = hc.Batch(ctx, precision="f32", max_slots=2, **SCHEME)
    try:
        b.admit(a, u, t_end=np.inf, max_steps=3, tag=7)
        b.set_schedule(dim, schedule)
        b.step(4)
        ev = b.poll()
        assert len(ev) == 1 and ev[0]["status"] == 0 and ev[0]["steps"] == 3
        got = b.fetch(ev[0]["slot"])
    finally:
        b.close()
    s = hc.Solver(ctx, precision="f32", **a)
    s.resetState(u)
    for _ in range(3):
        s.update()
    np.testing.assert_array_equal(got, s.getState())
