"""Writes c4_nonfinite.json: which instances of the batched quadrant workload
(512 grids, plm cons + van Leer (abs), Roe, RK2, CFL .475) reach a non-finite
state within their first 30 updates, and at which update, computed by the
oracle (the C++ CPU restatement of the reference, in FP64).

    python tests/golden/make_c4_nonfinite.py

The GPU tests require the FP64 batch to stop the same instances at the same
updates, and the FP32 batch to stop the same instances; the benchmark credits
only the updates the other instances do."""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests"), os.path.join(ROOT, "hydro-cl-lua_gb300")]

import cases  # noqa: E402
import hydrocuda as hc  # noqa: E402   (host-side generators only; no device needed)
import oracle  # noqa: E402

UPDATES = 30


def main():
    oracle.build()
    bad = []
    for k, (a, q) in enumerate(cases.c4_workload()):
        o = oracle.OracleSolver(a)
        o.reset_state(hc.quadrant_state(a, q))
        for s in range(UPDATES):
            o.update()
            if not np.isfinite(o.get_interior()).all():
                bad.append([k, a["gridSize"][0], s + 1])
                break
    with open(os.path.join(HERE, "c4_nonfinite.json"), "w") as f:
        json.dump({"updates": UPDATES, "instances": 512,
                   "nonfinite": bad, "columns": ["instance", "N", "first non-finite update"]}, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
