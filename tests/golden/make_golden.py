"""Writes the golden vectors in this folder: for a handful of small solves,
the initial interior state, the dt of every update and the final interior
state, computed by the oracle (the C++ CPU restatement of the reference,
pinned to the reference's recorded errors by tests/test_oracle_pins.py).

    python tests/golden/make_golden.py

The tests compare the oracle and every FP64 form of the library with these
files bit for bit, so any later change of the arithmetic shows up against a
frozen record."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests"), os.path.join(ROOT, "hydro-cl-lua_gb300")]

import cases  # noqa: E402
import hydrocuda as hc  # noqa: E402   (host-side generators only; no device needed)
import oracle  # noqa: E402

GOLDEN = [
    ("sod1d_superbee_fe", cases.c1_sod(gridSize=64), "sod", 12),
    ("sod1d_hllc_plm_prim_rk3tvd", cases.c1_sod(gridSize=48, fluxLimiter="donor cell", flux="euler-hllc",
                                               usePLM="plm prim", slopeLimiter="minmod",
                                               integrator="Runge-Kutta 3, TVD"), "sod", 8),
    ("quadrant2d_plm_vanleer_rk2", cases.c4_quadrant(24), "quadrant", 6),
    ("kh2d_plm_mc_rk3tvd", cases.c2_kh(20), "kh", 5),
    ("blast3d_plm_minmod_rk2", cases.c3_blast(10), "blast", 3),
    ("quadrant2d_athena_hll_linear", cases.c4_quadrant(20, usePLM="plm athena", flux="hll", boundary="linear"),
     "quadrant", 4),
]


def initial(args, kind):
    if kind == "sod":
        return hc.sod_state(args)
    if kind == "kh":
        return hc.kelvin_helmholtz_state(args, seed=2)
    if kind == "blast":
        return hc.blast_state(args)
    return hc.quadrant_state(args, hc.random_quadrants(hc.SplitMix64(7)))


def run(args, kind, steps):
    U0 = initial(args, kind)
    s = oracle.OracleSolver(args)
    s.reset_state(U0)
    dts = []
    for _ in range(steps):
        dts.append(s.calcDT())
        s.update()
    return U0, np.array(dts), s.get_interior(), s.t


def main():
    for name, args, kind, steps in GOLDEN:
        U0, dts, U, t = run(args, kind, steps)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), initial=U0, dts=dts, final=U, t=t)
        print(name, U.shape, "t = %.17g" % t)


if __name__ == "__main__":
    main()
