"""The oracle's linear and quadratic boundaries (gridsolver.lua:783-858) on
states they must reproduce exactly: linear extrapolation continues a linear
profile into the ghosts, quadratic extrapolation a quadratic one (CPU)."""
import numpy as np
import pytest

import oracle


@pytest.mark.parametrize("kind,degree", [("linear", 1), ("quadratic", 2)])
def test_extrapolation_is_exact_on_its_polynomials(kind, degree):
    n = 12
    s = oracle.OracleSolver(dict(dim=2, gridSize=[n, n], boundary=kind, eqnArgs={"heatCapacityRatio": 1.4}))
    # every component a polynomial of the cell indices (exact in double)
    j, i = np.mgrid[0:n + 4, 0:n + 4].astype(float)
    poly = (lambda x: 3. + 2. * x) if degree == 1 else (lambda x: 1. + x + .5 * x * x)
    want = np.stack([poly(i) + k * poly(j) for k in range(6)], -1)
    full = np.zeros_like(want)
    full[2:-2, 2:-2] = want[2:-2, 2:-2]
    s.set_full(full)
    s.boundary()
    got = s.get_full().reshape(n + 4, n + 4, 6)
    # ghosts along x of interior rows and along y of interior columns
    np.testing.assert_array_equal(got[2:-2, :], want[2:-2, :])
    np.testing.assert_array_equal(got[:, 2:-2], want[:, 2:-2])


def test_mixed_sides():
    """Each side follows its own rule: linear on x min, quadratic on x max,
    freeflow on y."""
    n = 10
    bnd = dict(xmin="linear", xmax="quadratic", ymin="freeflow", ymax="freeflow")
    s = oracle.OracleSolver(dict(dim=2, gridSize=[n, n], boundary=bnd, eqnArgs={"heatCapacityRatio": 1.4}))
    rng = np.random.default_rng(1)
    U = rng.uniform(1., 2., size=(n * n, 6))
    full = np.zeros((n + 4, n + 4, 6))
    full[2:-2, 2:-2] = U.reshape(n, n, 6)
    s.set_full(full)
    s.boundary()
    g = s.get_full().reshape(n + 4, n + 4, 6)
    u = U.reshape(n, n, 6)
    np.testing.assert_array_equal(g[2:-2, 1], 2. * u[:, 0] - u[:, 1])
    np.testing.assert_array_equal(g[2:-2, 0], 2. * g[2:-2, 1] - u[:, 0])
    np.testing.assert_array_equal(g[2:-2, n + 2], 3. * u[:, -1] - 3. * u[:, -2] + u[:, -3])
    np.testing.assert_array_equal(g[2:-2, n + 3], 3. * g[2:-2, n + 2] - 3. * u[:, -1] + u[:, -2])
    np.testing.assert_array_equal(g[0, 2:-2], u[0])
    np.testing.assert_array_equal(g[-1, 2:-2], u[-1])


def test_fixed_side_holds_its_state():
    """gridsolver.lua:746-765: both ghost layers of a fixed side take the
    side's constant state (ePot 0) across the whole face, whatever the
    interior does; the other sides follow their own rules."""
    n = 10
    top = {"name": "fixed", "prim": {"rho": 1.0, "v": [2.0, 0.0, 0.0], "P": 1.0}}
    args = dict(dim=2, gridSize=[n, n], boundary={"xmin": "mirror", "xmax": "mirror", "ymin": "freeflow",
                                                  "ymax": top}, eqnArgs={"heatCapacityRatio": 1.4})
    s = oracle.OracleSolver(args)
    want = oracle.fixed_cons(top, 1.4)
    assert want == [1.0, 2.0, 0.0, 0.0, 1.0 * (.5 * 4.0) + 1.0 / 0.4]
    rng = np.random.default_rng(3)
    u = np.zeros((n * n, 6))
    u[:, 0] = 1 + rng.random(n * n)
    u[:, 4] = 3 + rng.random(n * n)
    s.reset_state(u)
    for _ in range(3):
        s.update()
        g = s.get_full().reshape(n + 4, n + 4, 6)
        for j in (n + 2, n + 3):
            np.testing.assert_array_equal(g[j, :, :5], np.tile(want, (n + 4, 1)))
            np.testing.assert_array_equal(g[j, :, 5], 0.0)
        np.testing.assert_array_equal(g[1, 2:-2], g[2, 2:-2])       # freeflow below


def test_entropy_fix_factor_zero_is_no_fix():
    """With a zero factor no wave speed is below dws = 0: the fix changes
    nothing; with the reference's .2 it changes the Sod solution, a little."""
    base = dict(dim=1, gridSize=128, boundary="freeflow", fluxLimiter="superbee", cfl=.5,
                eqnArgs={"heatCapacityRatio": 1.4})
    from oracle import OracleSolver
    import hydrocuda
    u = hydrocuda.sod_state(base)
    out = []
    for extra in ({}, dict(useEntropyFluxFix=True, entropyFluxFixLimitingFactor=0.0),
                  dict(useEntropyFluxFix=True)):
        s = OracleSolver(dict(base, **extra))
        s.reset_state(u)
        s.run_until(0.1)
        out.append(s.get_interior())
    np.testing.assert_array_equal(out[0], out[1])
    d = float(np.mean(np.abs(out[2][:, 0] - out[0][:, 0])))
    assert 0 < d < 1e-2, d
