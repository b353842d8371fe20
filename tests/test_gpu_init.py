"""Initial conditions built on the device equal the host generators bit for bit.

hydro-cl-lua builds initial states with its initCond kernel; the library does
the same (hc_solver_init_state, hc_batch_admit_init).  Each case resets one
solver from the host generator's array and one from the device-built state,
and requires identical states after the reset and after two updates, in every
precision form, and the same for batched admission.
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def _cases(hc):
    q = hc.random_quadrants(hc.SplitMix64(17))
    return [
        ("sod 1D", cases.c1_sod(gridSize=96, fluxLimiter="donor cell", usePLM="plm cons", slopeLimiter="minmod",
                                integrator="Runge-Kutta 2"),
         "sod", {}, hc.sod_state),
        ("sod 2D", cases.c4_quadrant(40), "sod", dict(rhoL=1.5, PR=.2), lambda a: hc.sod_state(a, rhoL=1.5, PR=.2)),
        ("blast 3D", cases.c3_blast(18), "blast", {}, hc.blast_state),
        ("blast 2D", cases.c4_quadrant(36), "blast", dict(radius=.3), lambda a: hc.blast_state(a, radius=.3)),
        ("quadrant", cases.c4_quadrant(44), "quadrant", dict(q=q), lambda a: hc.quadrant_state(a, q)),
        ("kelvin-helmholtz", cases.c2_kh(48), "kelvin-helmholtz", dict(seed=9, noise=.02),
         lambda a: hc.kelvin_helmholtz_state(a, seed=9, noise=.02)),
    ]


@pytest.mark.parametrize("precision", ["f64 plain", "f64", "f32"])
def test_solver_init_state_matches_host(hc, ctx, precision):
    for name, args, kind, params, host in _cases(hc):
        a = dict(args, precision=precision)
        s_host = hc.Solver(ctx, **a)
        s_dev = hc.Solver(ctx, **a)
        s_host.resetState(host(args))
        s_dev.initState(kind, **params)
        np.testing.assert_array_equal(s_dev.getState(), s_host.getState(), err_msg=name)
        for _ in range(2):
            s_host.update()
            s_dev.update()
        np.testing.assert_array_equal(s_dev.getState(), s_host.getState(), err_msg=name)
        assert s_dev.t == s_host.t


def test_batch_admit_init_matches_host(hc, ctx):
    scheme = dict(usePLM="plm cons", slopeLimiter="van Leer (abs)", integrator="Runge-Kutta 2")
    got = {}
    for mode in ("host", "device"):
        b = hc.Batch(ctx, precision="f32", max_slots=8, **scheme)
        for k, (name, args, kind, params, host) in enumerate(_cases(hc)):
            a = dict(args, **scheme)
            a.pop("fluxLimiter", None)
            if mode == "host":
                b.admit(a, host(a), .02, tag=k)
            else:
                b.admit_init(a, kind, .02, tag=k, **params)
        out = {}
        while len(out) < len(_cases(hc)):
            b.step(4)
            for ev in b.poll():
                out[ev["tag"]] = (b.fetch(ev["slot"]), ev["steps"])
        got[mode] = out
        b.close()
    for k in got["host"]:
        np.testing.assert_array_equal(got["device"][k][0], got["host"][k][0])
        assert got["device"][k][1] == got["host"][k][1]


def test_init_rejects_bad_requests(hc, ctx):
    s = hc.Solver(ctx, precision="f32", **cases.c1_sod(gridSize=32))
    with pytest.raises(hc.HydroCudaError):
        s.initState("quadrant")          # two-dimensional only
    with pytest.raises(ValueError):
        hc.make_init("sod", radius=1.0)   # not a Sod parameter


def test_served_stream_with_device_states_matches_host_states(hc, ctx):
    """The serving loop admitting requests by initial-condition name gives the
    results it gives when the same states are built on the host and uploaded."""
    import serve
    scheme = dict(usePLM="plm cons", slopeLimiter="minmod", integrator="Runge-Kutta 2")
    out = {}
    for device in (False, True):
        reqs = serve.synthetic_stream(10, rate_hz=500.0, seed=8, scale=0.08, device_init=device)
        b = hc.Batch(ctx, precision="f32", max_slots=4, hbm_budget=1 << 30, **scheme)
        done = serve.Server(b, steps_per_tick=4).run(reqs)
        b.close()
        out[device] = {r.tag: (r.result, r.steps) for r in done}
    assert len(out[True]) == 10
    for tag, (res, steps) in out[False].items():
        np.testing.assert_array_equal(out[True][tag][0], res)
        assert out[True][tag][1] == steps
