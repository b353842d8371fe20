"""The oracle against the golden vectors in tests/golden (written by
tests/golden/make_golden.py): initial states, every update's dt and the final
states, bit for bit (CPU)."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden  # noqa: E402


@pytest.mark.parametrize("name,args,kind,steps", make_golden.GOLDEN, ids=[g[0] for g in make_golden.GOLDEN])
def test_oracle_reproduces_golden(name, args, kind, steps):
    g = np.load(os.path.join(os.path.dirname(make_golden.__file__), name + ".npz"))
    U0, dts, U, t = make_golden.run(args, kind, steps)
    np.testing.assert_array_equal(U0, g["initial"])
    np.testing.assert_array_equal(dts, g["dts"])
    np.testing.assert_array_equal(U, g["final"])
    assert t == float(g["t"])
