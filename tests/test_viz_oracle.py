"""The numpy restatement of the views (oracle/viz.py) on cases with known
answers (CPU)."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import viz  # noqa: E402


def _cons(rho, v, P, g):
    v = np.asarray(v, dtype=float)
    return np.array([rho, rho * v[0], rho * v[1], rho * v[2], rho * .5 * (v @ v) + P / (g - 1), 0.])


def test_display_values_of_a_known_state():
    g = 1.4
    U = _cons(2., [3., 4., 0.], 1.5, g)
    val = lambda n: float(viz.display_values(U[None], n, g)[0])
    assert abs(val("P") - 1.5) < 1e-14
    assert abs(val("v mag") - 5.) < 1e-15
    cs = np.sqrt(g * 1.5 / 2.)
    assert abs(val("speed of sound") - cs) < 1e-15
    assert abs(val("Mach number") - 5. / cs) < 1e-14
    assert abs(val("eInt") - 1.5 / (g - 1) / 2.) < 1e-14
    assert abs(val("hTotal") - (1.5 + U[4]) / 2.) < 1e-14
    assert abs(val("S") - 1.5 / 2. ** g) < 1e-15


def test_display_buffer_clamps_or_zeroes_ghosts():
    U = np.zeros((1, 3, 4, 6))
    U[..., 0] = np.arange(12).reshape(1, 3, 4) + 1.
    U[..., 4] = 10.
    b = viz.display_buffer(U, "rho", 1.4)
    assert b.shape == (1, 7, 8)
    assert b[0, 0, 0] == 1. and b[0, -1, -1] == 12. and b[0, 3, 0] == b[0, 3, 2] == 5.
    z = viz.display_buffer(U, "rho", 1.4, zero_border=True)
    assert z[0, 0].sum() == 0 and z[0, 2:5, 2:6].sum() == 78.


def test_gradient_texture_ends_are_the_palette_ends():
    for p, cols in viz.PALETTES.items():
        g = viz.gradient_texture(p)
        np.testing.assert_allclose(g[0], cols[0], atol=1e-7)
        np.testing.assert_allclose(g[-1], cols[-1], atol=1e-7)


def test_linear_sampling_hits_texels_at_their_centres():
    tex = np.arange(24, dtype=np.float32).reshape(1, 4, 6, 1)
    u = (np.arange(6) + .5) / 6
    for j in range(4):
        got = viz.sample_linear(tex, u.astype(np.float32), np.full(6, (j + .5) / 4, dtype=np.float32))[..., 0]
        np.testing.assert_allclose(got, tex[0, j, :, 0], atol=1e-5)
    # half way between two texels: their mean; past the edge: wraps around
    got = viz.sample_linear(tex, np.float32([1. / 6, 0.]), np.float32([.125, .125]))[..., 0]
    np.testing.assert_allclose(got, [.5, (0. + 5.) / 2], atol=1e-5)


def test_heatmap_of_a_ramp_follows_the_palette():
    tex = np.tile(np.linspace(0., 1., 14, dtype=np.float32), (14, 1))[None]   # 10 interior + ghosts
    img = viz.heatmap(tex, 2, [10, 10], [0, 0, -1], [1, 1, 1], 10, 4, [0, 0, 1, 1], 0., 1.)
    # from the blue end (left) through the rainbow to red (right); alpha .8
    assert img[0, 0, 2] > 200 and img[0, 0, 0] < 60
    assert img[0, -1, 0] > 200 and img[0, -1, 2] < 60
    assert (img[..., 3] == 204).all()
