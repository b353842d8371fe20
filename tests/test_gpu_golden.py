"""Every form of the library against the golden vectors in tests/golden: the
FP64 forms reproduce every dt and the final state bit for bit, the FP32 form
within the density L1 bound."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,args,kind,steps", make_golden.GOLDEN, ids=[g[0] for g in make_golden.GOLDEN])
def test_forms_reproduce_golden(hc, ctx, name, args, kind, steps):
    g = np.load(os.path.join(os.path.dirname(make_golden.__file__), name + ".npz"))
    for prec in ("f64 plain", "f64", "f32"):
        s = hc.Solver(ctx, precision=prec, **args)
        s.resetState(g["initial"])
        dts = np.array([s.update() for _ in range(steps)])
        U = s.getState()
        if prec == "f32":
            assert float(np.mean(np.abs(U[:, 0] - g["final"][:, 0]))) <= 1e-5, name
        else:
            np.testing.assert_array_equal(dts, g["dts"], err_msg="%s %s" % (name, prec))
            np.testing.assert_array_equal(U[:, :5], g["final"][:, :5], err_msg="%s %s" % (name, prec))
            assert s.t == float(g["t"])
