"""The "plm prim" and "plm athena" reconstructions (hydro/solver/plm.cl:191-253,
782-879) in every form, with the Roe, HLL and HLLC fluxes: the FP64 forms
bit-identical to the oracle per step, the FP32 form within the density L1
bound, batched solves equal to their alone runs."""
import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu

L1_RHO_F32 = 1e-5

RECON_CASES = [
    ("sod1d", cases.c1_sod(gridSize=64, fluxLimiter="donor cell", slopeLimiter="minmod"), "sod", 8),
    ("sod1d_rk3", cases.c1_sod(gridSize=48, fluxLimiter="donor cell", slopeLimiter="superbee",
                               integrator="Runge-Kutta 3, TVD"), "sod", 5),
    ("quadrant2d", cases.c4_quadrant(36), "quadrant", 6),
    ("kh2d", cases.c2_kh(32), "kh", 5),
    ("blast3d", cases.c3_blast(12), "blast", 4),
]


def _state(hc, args, kind):
    if kind == "sod":
        return hc.sod_state(args)
    if kind == "kh":
        return hc.kelvin_helmholtz_state(args, seed=2)
    if kind == "blast":
        return hc.blast_state(args)
    return hc.quadrant_state(args, hc.random_quadrants(hc.SplitMix64(7)))


RECONS = [("plm prim", "roe"), ("plm athena", "roe"), ("plm prim", "euler-hllc"), ("plm athena", "hll")]


@pytest.mark.parametrize("recon,flux", RECONS, ids=["%s-%s" % (r.replace(" ", "_"), f) for r, f in RECONS])
@pytest.mark.parametrize("name,args,kind,steps", RECON_CASES, ids=[c[0] for c in RECON_CASES])
def test_reconstructions_match_oracle(hc, ctx, recon, flux, name, args, kind, steps):
    a = dict(args, usePLM=recon, flux=flux)
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
    assert np.all(np.isfinite(g32))
    assert float(np.mean(np.abs(g32[:, 0] - orc.get_interior()[:, 0]))) <= L1_RHO_F32


def test_reconstructions_differ(hc, ctx):
    """The three PLM kinds are different schemes (a mix-up in the kernel
    registry would make two of them equal)."""
    a0 = cases.c4_quadrant(40)
    U0 = hc.quadrant_state(a0, hc.random_quadrants(hc.SplitMix64(3)))
    out = {}
    for recon in ("plm cons", "plm prim", "plm athena"):
        s = hc.Solver(ctx, precision="f32", **dict(a0, usePLM=recon))
        s.resetState(U0)
        for _ in range(3):
            s.update()
        out[recon] = s.getState()
    assert not np.array_equal(out["plm cons"], out["plm prim"])
    assert not np.array_equal(out["plm cons"], out["plm athena"])
    assert not np.array_equal(out["plm prim"], out["plm athena"])


@pytest.mark.parametrize("recon", ["plm prim", "plm athena"])
def test_reconstruction_batch_equals_alone(hc, ctx, recon):
    scheme = dict(usePLM=recon, slopeLimiter="minmod", integrator="Runge-Kutta 2")
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
