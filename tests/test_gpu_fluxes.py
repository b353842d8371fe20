"""The HLL, Rusanov and HLLC interface fluxes (hydro/flux/hll.cl, rusanov.cl,
euler-hllc.cl) in every form: the FP64 forms bit-identical to the oracle per step, the FP32
form within the density L1 bound, batched solves equal to their alone runs."""
import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu

L1_RHO_F32 = 1e-5

FLUX_CASES = [
    ("sod1d", cases.c1_sod(gridSize=64, fluxLimiter="donor cell"), "sod", 8),
    ("sod1d_plm", cases.c1_sod(gridSize=64, fluxLimiter="donor cell", usePLM="plm cons", slopeLimiter="minmod",
                               integrator="Runge-Kutta 2"), "sod", 8),
    ("quadrant2d_plm", cases.c4_quadrant(36), "quadrant", 6),
    ("kh2d", cases.c2_kh(32, usePLM=None, slopeLimiter="donor cell"), "kh", 5),
    ("blast3d_plm", cases.c3_blast(12), "blast", 4),
    # a flux limiter is ignored by every flux but Roe (fvsolver.lua:62-64)
    ("sod1d_limiter_ignored", cases.c1_sod(gridSize=48, fluxLimiter="superbee"), "sod", 6),
]


def _state(hc, args, kind):
    if kind == "sod":
        return hc.sod_state(args)
    if kind == "kh":
        return hc.kelvin_helmholtz_state(args, seed=2)
    if kind == "blast":
        return hc.blast_state(args)
    return hc.quadrant_state(args, hc.random_quadrants(hc.SplitMix64(7)))


FLUXES = [("hll", None), ("rusanov", None), ("euler-hllc", None), ("euler-hllc", 0), ("euler-hllc", 1)]


@pytest.mark.parametrize("flux,method", FLUXES, ids=["%s%s" % (f, "" if m is None else m) for f, m in FLUXES])
@pytest.mark.parametrize("name,args,kind,steps", FLUX_CASES, ids=[c[0] for c in FLUX_CASES])
def test_fluxes_match_oracle(hc, ctx, flux, method, name, args, kind, steps):
    a = dict(args, flux=flux)
    if method is not None:
        a["hllcMethod"] = method
    U0 = _state(hc, a, kind)
    orc = oracle.OracleSolver(a)
    orc.reset_state(U0)
    gpus = {}
    for prec in ("f64 plain", "f64", "f32"):
        gpus[prec] = hc.Solver(ctx, precision=prec, **a)
        gpus[prec].resetState(U0)
    for k in range(steps):
        dt_o = orc.calcDT()
        for prec in ("f64 plain", "f64"):
            assert gpus[prec].calcDT() == dt_o, (prec, k)
        orc.update()
        for g in gpus.values():
            g.update()
        o = orc.get_interior()[:, :5]
        for prec in ("f64 plain", "f64"):
            np.testing.assert_array_equal(gpus[prec].getState()[:, :5], o, err_msg="%s %s step %d" % (prec, name, k))
    g32 = gpus["f32"].getState()
    assert float(np.mean(np.abs(g32[:, 0] - orc.get_interior()[:, 0]))) <= L1_RHO_F32


@pytest.mark.parametrize("flux", ["hll", "rusanov", "euler-hllc"])
def test_flux_batch_equals_alone(hc, ctx, flux):
    scheme = dict(usePLM="plm cons", slopeLimiter="minmod", integrator="Runge-Kutta 2", flux=flux)
    probs = [(cases.c4_quadrant(n, **scheme), s) for n, s in ((40, 3), (56, 4))]
    b = hc.Batch(ctx, precision="f32", max_slots=4, **scheme)
    for k, (a, s) in enumerate(probs):
        b.admit(a, hc.quadrant_state(a, hc.random_quadrants(hc.SplitMix64(s))), .03, tag=k)
    got = {}
    while len(got) < 2:
        b.step(4)
        for ev in b.poll():
            got[ev["tag"]] = b.fetch(ev["slot"])
    b.close()
    for k, (a, s) in enumerate(probs):
        alone = hc.Solver(ctx, precision="f32", **a)
        alone.resetState(hc.quadrant_state(a, hc.random_quadrants(hc.SplitMix64(s))))
        alone.run_until(.03)
        np.testing.assert_array_equal(got[k], alone.getState())
