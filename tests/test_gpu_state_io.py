"""The reference's whole UBuf (ghosts included) from every form.

The plain form holds the UBuf itself; the fused forms expand their interior
with the reference's boundary rules.  The FP64 forms are bit-identical to the
oracle, so their ghost-inclusive states must be identical too, corners
included, and writing a UBuf back must reproduce the solve.
"""
import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,args", [
    ("kh periodic", cases.c2_kh(40)),
    ("blast freeflow", cases.c3_blast(14)),
    ("quadrant mirror", cases.c4_quadrant(36, boundary="mirror")),
])
def test_fused_ubuf_equals_plain_and_oracle(hc, ctx, name, args):
    U0 = hc.kelvin_helmholtz_state(args) if "kh" in name else (
        hc.blast_state(args) if "blast" in name else hc.quadrant_state(args, hc.random_quadrants(hc.SplitMix64(3))))
    plain = hc.Solver(ctx, precision="f64 plain", **args)
    fused = hc.Solver(ctx, precision="f64", **args)
    orc = oracle.OracleSolver(args)
    for s in (plain, fused):
        s.resetState(U0)
    orc.reset_state(U0)
    for _ in range(3):
        full_p = plain.getState(withGhosts=True)
        full_f = fused.getState(withGhosts=True)
        np.testing.assert_array_equal(full_f, full_p, err_msg=name)
        np.testing.assert_array_equal(full_p, orc.get_full(), err_msg=name)
        plain.update()
        fused.update()
        orc.update()


def test_ubuf_round_trip_restarts_the_solve(hc, ctx):
    args = cases.c4_quadrant(48)
    U0 = hc.quadrant_state(args, hc.random_quadrants(hc.SplitMix64(5)))
    for prec in ("f64 plain", "f64", "f32"):
        a = hc.Solver(ctx, precision=prec, **args)
        a.resetState(U0)
        for _ in range(3):
            a.update()
        full = a.getState(withGhosts=True)
        b = hc.Solver(ctx, precision=prec, **args)
        b.setState(full, withGhosts=True)
        b.t = a.t
        for s in (a, b):
            s.update()
            s.update()
        np.testing.assert_array_equal(b.getState(), a.getState(), err_msg=prec)
        assert b.t == a.t


def test_snapshot_restart_from_fits(hc, ctx, tmp_path):
    """GridSolver:save's UBuf image written as FITS, read back into a fresh
    solver: the restarted solve continues bit for bit."""
    import snapshot
    args = cases.c2_kh(32)
    for prec in ("f64 plain", "f32"):
        a = hc.Solver(ctx, precision=prec, **args)
        a.resetState(hc.kelvin_helmholtz_state(args))
        a.update()
        a.update()
        path = snapshot.save(a, str(tmp_path / prec.replace(" ", "_")))
        b = hc.Solver(ctx, precision=prec, **args)
        hdr = snapshot.restore(b, path)
        assert hdr["HCTIME"] == a.t == b.t
        np.testing.assert_array_equal(b.getState(withGhosts=True), a.getState(withGhosts=True))
        a.update()
        b.update()
        np.testing.assert_array_equal(b.getState(), a.getState(), err_msg=prec)


@pytest.mark.parametrize("dim", [2, 3])
def test_solver_autotune_keeps_the_solve(hc, ctx, dim):
    """hc_solver_autotune times the schedules on the solver's own grid and puts
    its state and time back: the solve goes on exactly as an untuned one."""
    import cases
    if dim == 2:
        a = cases.c4_quadrant(96)
        u = hc.quadrant_state(a, hc.random_quadrants(hc.SplitMix64(12)))
    else:
        a = cases.c3_blast(24)
        u = hc.blast_state(a)
    tuned = hc.Solver(ctx, precision="f32", **a)
    plain = hc.Solver(ctx, precision="f32", **a)
    for s in (tuned, plain):
        s.resetState(u)
        s.update()
    before = tuned.getState(withGhosts=True)
    t0 = tuned.t
    tuned.autotune()
    np.testing.assert_array_equal(tuned.getState(withGhosts=True), before)
    assert tuned.t == t0
    for _ in range(3):
        tuned.update()
        plain.update()
    np.testing.assert_array_equal(tuned.getState(), plain.getState())
    assert tuned.t == plain.t
