"""Shared solver configurations for the parity tests (reference args-table vocabulary)."""


def c1_sod(**kw):
    """1D Sod, 256 cells on [-1,1], gamma 1.4, freeflow, Roe + superbee flux limiter, FE, CFL .5."""
    a = dict(dim=1, gridSize=256, mins=[-1, -1, -1], maxs=[1, 1, 1], boundary="freeflow",
             flux="roe", fluxLimiter="superbee", integrator="forward Euler", cfl=.5,
             eqnArgs={"heatCapacityRatio": 1.4})
    a.update(kw)
    return a


def c2_kh(n=1024, **kw):
    """2D Kelvin-Helmholtz on [-.5,.5]^2, periodic, plm cons + MC, Roe, RK3-TVD, CFL .4, gamma 1.4."""
    a = dict(dim=2, gridSize=[n, n], mins=[-.5, -.5, -1], maxs=[.5, .5, 1], boundary="periodic",
             flux="roe", usePLM="plm cons", slopeLimiter="monotized central", integrator="Runge-Kutta 3, TVD",
             cfl=.4, eqnArgs={"heatCapacityRatio": 1.4})
    a.update(kw)
    return a


def c3_blast(n=256, **kw):
    """3D blast on [-1,1]^3, freeflow, plm cons + minmod, Roe, RK2 (midpoint), CFL .3, gamma 5/3."""
    a = dict(dim=3, gridSize=[n, n, n], mins=[-1, -1, -1], maxs=[1, 1, 1], boundary="freeflow",
             flux="roe", usePLM="plm cons", slopeLimiter="minmod", integrator="Runge-Kutta 2",
             cfl=.3, eqnArgs={"heatCapacityRatio": 5. / 3.})
    a.update(kw)
    return a


def c4_quadrant(n, **kw):
    """One instance of the batched quadrant problem: [-1,1]^2, freeflow, plm cons + van Leer, RK2, CFL .475.

    The reference's table form of van Leer, max(0, r) * 2 / (1 + r), is 0/0 at
    r = -1 and turns these problems non-finite within a few steps (the oracle
    shows it); the default here is the form the reference keeps beside it in a
    comment, (r + |r|) / (1 + |r|), identical for every other r."""
    a = dict(dim=2, gridSize=[n, n], mins=[-1, -1, -1], maxs=[1, 1, 1], boundary="freeflow",
             flux="roe", usePLM="plm cons", slopeLimiter="van Leer (abs)", integrator="Runge-Kutta 2",
             cfl=.475, eqnArgs={"heatCapacityRatio": 1.4})
    a.update(kw)
    return a


def c4_workload(count=512, seed=4):
    """The batched quadrant workload as the benchmark builds it: `count` grids
    with N log-uniform in [64, 512] (SplitMix64 seed 4), instance i's quadrant
    states from SplitMix64(100000 + i).  Returns [(args, quadrants)]."""
    import hydrocuda as hc
    sizes = hc.batched_quadrant_sizes(count, seed)
    return [(c4_quadrant(n), hc.random_quadrants(hc.SplitMix64(100000 + i))) for i, n in enumerate(sizes)]
