"""Parity at the configurations' real sizes.

* The batched quadrant workload (512 grids, N 64..512): its first instances in
  FP64 bit-equal to the oracle over 10 updates; the instances that reach a
  non-finite state within 30 updates, and the update at which they do, the
  same in the FP64 batch as in the oracle (tests/golden/c4_nonfinite.json,
  written by make_c4_nonfinite.py), and the same instances in the FP32 batch.
* The 3D blast at its full 256^3: the fused FP64 form bit-equal to the oracle
  after two Runge-Kutta 2 updates, and the FP32 form within density L1 1e-5 of
  it."""
import json
import os

import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
SCHEME4 = dict(usePLM="plm cons", slopeLimiter="van Leer (abs)", integrator="Runge-Kutta 2")


def _batch_run(hc, ctx, precision, probs, steps, scheme):
    """Every problem through one batch for up to `steps` updates; returns
    {index: (state or None, status, steps)}."""
    b = hc.Batch(ctx, precision=precision, max_slots=len(probs), **scheme)
    try:
        for k, (a, cons) in enumerate(probs):
            b.admit(a, cons, t_end=np.inf, max_steps=steps, tag=k)
        out = {}
        for _ in range(10000):
            b.step(8)
            for ev in b.poll():
                st = b.fetch(ev["slot"]) if ev["status"] == 0 else None
                out[ev["tag"]] = (st, ev["status"], ev["steps"])
                b.retire(ev["slot"])
            if len(out) == len(probs):
                break
        return out
    finally:
        b.close()


def test_c4_first_instances_fp64_bit_equal(hc, ctx):
    work = cases.c4_workload()[:12]
    probs = [(a, hc.quadrant_state(a, q)) for a, q in work]
    got = _batch_run(hc, ctx, "f64", probs, 10, SCHEME4)
    sizes = []
    for k, (a, cons) in enumerate(probs):
        o = oracle.OracleSolver(a)
        o.reset_state(cons)
        for _ in range(10):
            o.update()
        st, status, steps = got[k]
        assert status == 0 and steps == 10
        np.testing.assert_array_equal(st[:, :5], o.get_interior()[:, :5], err_msg="instance %d" % k)
        sizes.append(a["gridSize"][0])
    assert max(sizes) >= 256 and min(sizes) <= 128     # the size range of the workload


def test_c4_nonfinite_instances_match_the_oracle(hc, ctx):
    gold = json.load(open(os.path.join(HERE, "golden", "c4_nonfinite.json")))
    expect = {k: upd for k, n, upd in gold["nonfinite"]}
    work = cases.c4_workload()
    probs = [(a, hc.quadrant_state(a, q)) for a, q in work]
    f64 = _batch_run(hc, ctx, "f64", probs, gold["updates"], SCHEME4)
    got = {k: steps for k, (_, status, steps) in f64.items() if status != 0}
    assert got == expect
    f32 = _batch_run(hc, ctx, "f32", probs, gold["updates"], SCHEME4)
    assert {k for k, (_, status, _) in f32.items() if status != 0} == set(expect)
    assert all(steps == gold["updates"] for k, (_, status, steps) in f32.items() if status == 0)


def test_c3_full_size(hc, ctx):
    a = cases.c3_blast(256)
    cons = hc.blast_state(a)
    scheme = dict(usePLM="plm cons", slopeLimiter="minmod", integrator="Runge-Kutta 2")
    f64 = _batch_run(hc, ctx, "f64", [(a, cons)], 2, scheme)[0]
    f32 = _batch_run(hc, ctx, "f32", [(a, cons)], 2, scheme)[0]
    assert f64[1] == 0 and f32[1] == 0
    o = oracle.OracleSolver(a)
    o.reset_state(cons)
    for _ in range(2):
        o.update()
    np.testing.assert_array_equal(f64[0][:, :5], o.get_interior()[:, :5])
    l1 = float(np.mean(np.abs(f32[0][:, 0] - f64[0][:, 0])))
    assert l1 <= 1e-5, l1
