"""Headless views on the GPU against the numpy restatement (oracle/viz.py):
display variables bit for bit (the power in S within an ulp), their range,
mean and deviation, and the heat-map, volume and LIC images."""
import os
import sys

import numpy as np
import pytest

import cases

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import viz  # noqa: E402

pytestmark = pytest.mark.gpu

CASES = [
    ("sod1d", cases.c1_sod(gridSize=40, fluxLimiter="donor cell", usePLM="plm cons", slopeLimiter="minmod",
                           integrator="Runge-Kutta 2"), "sod"),
    ("quadrant2d", cases.c4_quadrant(24), "quadrant"),
    ("blast3d", cases.c3_blast(10), "blast"),
]


def _state(hc, args, kind):
    if kind == "sod":
        return hc.sod_state(args)
    if kind == "blast":
        return hc.blast_state(args)
    return hc.quadrant_state(args, hc.random_quadrants(hc.SplitMix64(5)))


def _solver(hc, ctx, args, kind, precision, steps=3):
    s = hc.Solver(ctx, precision=precision, **args)
    s.resetState(_state(hc, args, kind))
    for _ in range(steps):
        s.update()
    return s


def _grid(s):
    n = list(s.gridSize) + [1] * (3 - s.dim)
    return s.getState().reshape(n[2], n[1], n[0], 6)


def _gamma(args):
    return args["eqnArgs"]["heatCapacityRatio"]


@pytest.mark.parametrize("precision", ["f64 plain", "f64", "f32"])
@pytest.mark.parametrize("name,args,kind", CASES, ids=[c[0] for c in CASES])
def test_display_variables(hc, ctx, precision, name, args, kind):
    s = _solver(hc, ctx, args, kind, precision)
    U = _grid(s)
    for var in viz.DISPLAY_VARS:
        for zb in (False, True):
            got = s.display(var, zeroBorder=zb)
            want = viz.display_buffer(U, var, _gamma(args), zero_border=zb).reshape(got.shape)
            if var == "S":
                np.testing.assert_allclose(got, want, rtol=4e-16, atol=0, err_msg=var)
            else:
                np.testing.assert_array_equal(got, want, err_msg="%s zeroBorder=%s" % (var, zb))


@pytest.mark.parametrize("name,args,kind", CASES, ids=[c[0] for c in CASES])
def test_display_range(hc, ctx, name, args, kind):
    s = _solver(hc, ctx, args, kind, "f64")
    U = _grid(s)
    for var in ("rho", "P", "v mag", "Mach number", "eInt"):
        mn, mx, mean, dev = s.displayRange(var)
        wmn, wmx, wmean, wdev = viz.display_range(U, var, _gamma(args))
        assert (mn, mx) == (wmn, wmx), var
        np.testing.assert_allclose([mean, dev], [wmean, wdev], rtol=1e-12, err_msg=var)


def _close_images(got, want, frac=.995, tol=2):
    assert got.shape == want.shape
    d = np.abs(got.astype(int) - want.astype(int))
    assert (d <= tol).mean() >= frac, (d.max(), (d > tol).mean())
    assert (d <= 1).mean() >= .98


@pytest.mark.parametrize("palette", [0, 3])
def test_heatmap(hc, ctx, palette):
    args = cases.c4_quadrant(24)
    s = _solver(hc, ctx, args, "quadrant", "f32")
    U = _grid(s)
    tex = viz.display_buffer(U, "rho", _gamma(args)).astype(np.float32)
    mn, mx = s.displayRange("rho")[:2]
    got = s.render("heatmap", var="rho", width=72, height=60, palette=palette)
    want = viz.heatmap(tex, 2, s.gridSize, args["mins"], args["maxs"], 72, 60,
                       [args["mins"][0], args["mins"][1], args["maxs"][0], args["maxs"][1]], mn, mx, palette=palette)
    _close_images(got, want)
    # a wider view leaves the outside transparent, a log mapping differs
    got2 = s.render("heatmap", var="P", width=40, height=40, bbox=[-2, -2, 2, 2], use_log=True, value_min=.05,
                    value_max=3.)
    tex2 = viz.display_buffer(U, "P", _gamma(args)).astype(np.float32)
    want2 = viz.heatmap(tex2, 2, s.gridSize, args["mins"], args["maxs"], 40, 40, [-2, -2, 2, 2], .05, 3.,
                        use_log=True)
    _close_images(got2, want2)
    assert (got2[0, 0] == 0).all()


def test_heatmap_slice_of_3d(hc, ctx):
    args = cases.c3_blast(10)
    s = _solver(hc, ctx, args, "blast", "f32", steps=2)
    U = _grid(s)
    tex = viz.display_buffer(U, "P", _gamma(args)).astype(np.float32)
    q = (np.sin(np.pi / 8), 0., 0., np.cos(np.pi / 8))   # 45 degrees about x
    got = s.render("heatmap", var="P", width=48, height=48, slice_angle=q, fixed_z=.1, value_min=.1, value_max=1.)
    want = viz.heatmap(tex, 3, s.gridSize, args["mins"], args["maxs"], 48, 48, [-1, -1, 1, 1], .1, 1., q=q,
                       fixed_z=.1)
    _close_images(got, want)


def test_lic(hc, ctx):
    args = cases.c2_kh(32)
    s = hc.Solver(ctx, precision="f32", **args)
    s.resetState(hc.kelvin_helmholtz_state(args, seed=3, noise=.05))
    for _ in range(4):
        s.update()
    U = _grid(s)
    vel = np.stack([viz.display_buffer(U, v, _gamma(args)) for v in ("v x", "v y", "v z")], -1)
    vel = np.concatenate([vel, np.zeros(vel.shape[:-1] + (1,))], -1).astype(np.float32)
    noise = viz.splitmix_uniforms(7, 64 * 64).reshape(64, 64)
    mn, mx = s.displayRange("v mag")[:2]
    got = s.render("lic", width=64, height=64, noise_size=64, noise_seed=7)
    want = viz.lic(vel, noise, 2, s.gridSize, args["mins"], args["maxs"], 64, 64,
                   [args["mins"][0], args["mins"][1], args["maxs"][0], args["maxs"][1]], mn, mx)
    _close_images(got, want)


@pytest.mark.parametrize("isobars,lighting", [(False, False), (True, False), (False, True)])
def test_volume(hc, ctx, isobars, lighting):
    args = cases.c3_blast(12)
    s = _solver(hc, ctx, args, "blast", "f32", steps=3)
    U = _grid(s)
    tex = viz.display_buffer(U, "P", _gamma(args)).astype(np.float32)
    eye = (2.5, 1.5, 3.5)
    got = s.render("volume", var="P", width=40, height=32, eye=eye, max_iter=48, value_min=.1, value_max=1.,
                   use_isobars=isobars, use_lighting=lighting)
    want = viz.volume(tex, s.gridSize, args["mins"], args["maxs"], 40, 32, .1, 1., eye, max_iter=48,
                      use_isobars=isobars, use_lighting=lighting)
    _close_images(got, want)
    assert got[..., 3].max() > 0


@pytest.mark.parametrize("axis,isobars", [(2, True), (3, False), (1, True)])
def test_slices(hc, ctx, axis, isobars):
    args = cases.c3_blast(12)
    s = _solver(hc, ctx, args, "blast", "f32", steps=3)
    U = _grid(s)
    tex = viz.display_buffer(U, "P", _gamma(args)).astype(np.float32)
    got = s.render("slices", var="P", width=36, height=30, slice_axis=axis, num_slices=40, use_isobars=isobars,
                   value_min=.1, value_max=1.)
    want = viz.slices(tex, s.gridSize, 36, 30, .1, 1., axis=axis, num_slices=40, use_isobars=isobars)
    _close_images(got, want, frac=.99, tol=3)
    assert got[..., 3].max() > 0


def test_render_rejects_bad_views(hc, ctx):
    s = _solver(hc, ctx, cases.c4_quadrant(16), "quadrant", "f32", steps=0)
    with pytest.raises(hc.HydroCudaError):
        s.render("volume")                 # 2D grid
    with pytest.raises(hc.HydroCudaError):
        s.render("slices")                 # 2D grid
    with pytest.raises(hc.HydroCudaError):
        s.render("heatmap", width=0)
    with pytest.raises(hc.HydroCudaError):
        s.render("heatmap", slice_angle=[0, 0, 0, 0])
