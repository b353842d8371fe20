"""How far an FMA-contracting build of the reference's arithmetic can drift
from the oracle's contraction-free reading.

OpenCL compiles with FP_CONTRACT ON, so the reference's kernels may fuse
multiply-adds where the compiler chooses; the oracle (and the FP64 forms,
bit-equal to it) evaluate every expression as written.  A second build of the
oracle with -ffp-contract=fast (FMA instructions enabled) stands in for such a
build: from identical states, one update of each differs by at most 1e-12 of
each field's largest magnitude (the per-step parity tolerance), and after the
1D Sod configuration's whole run their densities differ by at most 1e-10 in
L1 (the full-run tolerance) -- so the contraction-free reading is the
reference's result to within the stated tolerances, whichever way its
compiler contracted."""
import numpy as np
import pytest

import cases
import hydrocuda as hc
import oracle


def _configs():
    sod = cases.c1_sod()
    quad = cases.c4_quadrant(48)
    kh = cases.c2_kh(32)
    blast = cases.c3_blast(16)
    return [
        ("sod", sod, hc.sod_state(sod)),
        ("quadrant", quad, hc.quadrant_state(quad, hc.random_quadrants(hc.SplitMix64(3)))),
        ("kh", kh, hc.kelvin_helmholtz_state(kh, seed=2)),
        ("blast", blast, hc.blast_state(blast)),
    ]


@pytest.mark.parametrize("name,args,init", _configs(), ids=[c[0] for c in _configs()])
def test_one_update_from_the_same_state(name, args, init):
    ref = oracle.OracleSolver(args)
    ref.reset_state(init)
    fused = oracle.OracleSolver(args, contract=True)
    worst = 0.0
    for k in range(12):
        state, t = ref.get_full(), ref.t
        fused.set_full(state)
        fused.t = t
        ref.update()
        fused.update()
        a, b = ref.get_interior()[:, :5], fused.get_interior()[:, :5]
        scale = np.max(np.abs(a), axis=0)
        rel = np.max(np.abs(a - b), axis=0) / np.where(scale > 0, scale, 1.0)
        worst = max(worst, float(rel.max()))
        assert ref.t == fused.t or abs(ref.t - fused.t) <= 1e-12 * abs(ref.t)
    assert worst <= 1e-12, worst


def test_sod_full_run():
    args = cases.c1_sod()
    out = []
    for contract in (False, True):
        o = oracle.OracleSolver(args, contract=contract)
        o.reset_state(hc.sod_state(args))
        o.run_until(0.2)
        out.append(o.get_interior())
    assert float(np.mean(np.abs(out[0][:, 0] - out[1][:, 0]))) <= 1e-10
