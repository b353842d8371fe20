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
