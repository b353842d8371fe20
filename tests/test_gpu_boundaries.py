"""The linear and quadratic boundaries (gridsolver.lua:783-858) in every form:
the FP64 forms bit-identical to the oracle per step (state and ghosts), the
FP32 form within the density L1 bound, batched solves equal to their alone
runs."""
import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu

L1_RHO_F32 = 1e-5

MIXED = dict(xmin="linear", xmax="quadratic", ymin="freeflow", ymax="linear", zmin="quadratic", zmax="mirror")

BC_CASES = [
    ("sod1d", cases.c1_sod(gridSize=64, fluxLimiter="superbee"), "sod", 6),
    ("sod1d_plm_rk2", cases.c1_sod(gridSize=48, fluxLimiter="donor cell", usePLM="plm cons",
                                   slopeLimiter="minmod", integrator="Runge-Kutta 2"), "sod", 5),
    ("quadrant2d", cases.c4_quadrant(32), "quadrant", 5),
    ("blast3d", cases.c3_blast(12), "blast", 3),
]


def _state(hc, args, kind):
    if kind == "sod":
        return hc.sod_state(args)
    if kind == "blast":
        return hc.blast_state(args)
    return hc.quadrant_state(args, hc.random_quadrants(hc.SplitMix64(9)))


@pytest.mark.parametrize("bc", ["linear", "quadratic", "mixed"])
@pytest.mark.parametrize("name,args,kind,steps", BC_CASES, ids=[c[0] for c in BC_CASES])
def test_boundaries_match_oracle(hc, ctx, bc, name, args, kind, steps):
    a = dict(args, boundary=MIXED if bc == "mixed" else bc)
    U0 = _state(hc, a, kind)
    orc = oracle.OracleSolver(a)
    orc.reset_state(U0)
    gpus = {p: hc.Solver(ctx, precision=p, **a) for p in ("f64 plain", "f64", "f32")}
    for g in gpus.values():
        g.resetState(U0)
    np.testing.assert_array_equal(gpus["f64 plain"].getState(withGhosts=True), orc.get_full())
    for k in range(steps):
        dt_o = orc.calcDT()
        for p in ("f64 plain", "f64"):
            assert gpus[p].calcDT() == dt_o, (p, k)
        orc.update()
        for g in gpus.values():
            g.update()
        o = orc.get_interior()[:, :5]
        for p in ("f64 plain", "f64"):
            np.testing.assert_array_equal(gpus[p].getState()[:, :5], o, err_msg="%s %s step %d" % (p, name, k))
    np.testing.assert_array_equal(gpus["f64 plain"].getState(withGhosts=True), orc.get_full())
    np.testing.assert_array_equal(gpus["f64"].getState(withGhosts=True)[:, :5], orc.get_full()[:, :5])
    g32 = gpus["f32"].getState()
    assert float(np.mean(np.abs(g32[:, 0] - orc.get_interior()[:, 0]))) <= L1_RHO_F32


def test_boundaries_batch_equals_alone(hc, ctx):
    scheme = dict(usePLM="plm cons", slopeLimiter="minmod", integrator="Runge-Kutta 2")
    probs = [(cases.c4_quadrant(n, boundary=b, **scheme), s)
             for n, s, b in ((40, 3, "linear"), (36, 4, "quadratic"), (28, 5, "freeflow"))]
    b = hc.Batch(ctx, precision="f32", max_slots=4, **scheme)
    for k, (a, s) in enumerate(probs):
        b.admit(a, hc.quadrant_state(a, hc.random_quadrants(hc.SplitMix64(s))), .03, tag=k)
    got = {}
    while len(got) < len(probs):
        b.step(4)
        for ev in b.poll():
            got[ev["tag"]] = (b.fetch(ev["slot"]), ev["status"])
    b.close()
    for k, (a, s) in enumerate(probs):
        alone = hc.Solver(ctx, precision="f32", **a)
        alone.resetState(hc.quadrant_state(a, hc.random_quadrants(hc.SplitMix64(s))))
        alone.run_until(.03)
        np.testing.assert_array_equal(got[k][0], alone.getState())


def test_quadratic_needs_three_cells(hc, ctx):
    with pytest.raises(hc.HydroCudaError):
        hc.Solver(ctx, precision="f64 plain", **cases.c1_sod(gridSize=2, boundary="quadratic"))
