"""hc_calc_dt_noalloc: the time step for callers that cannot allocate device memory.

Such a caller -- one recording a CUDA graph, one whose device memory belongs
to an outside allocator, one in a loop that cannot afford cudaMalloc's
implicit synchronisation -- hands the library a state and an output it
already owns and gets the CFL dt back without the library allocating
anything.  These tests call that entry point through the C ABI on device
buffers the test itself owns, twice in a row, and compare each result with
the allocating entry point (hc_solver_calc_dt of the plain FP64 form) on the
same state; the plain form's tolerance is equality.  The file sorts last so a
run that stops at the first failure has run everything else already.
"""
import ctypes

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def _device_copy(torch, host):
    t = torch.from_numpy(np.ascontiguousarray(host)).to("cuda")
    torch.cuda.synchronize()
    return t


def test_noalloc_dt_matches_solver_twice(hc, ctx):
    torch = pytest.importorskip("torch")
    L = hc.load_library()
    states = []
    for args, U0 in ((cases.c2_kh(96), None), (cases.c3_blast(20), None)):
        s = hc.Solver(ctx, precision="f64 plain", **args)
        s.resetState(hc.kelvin_helmholtz_state(args, seed=2) if args["dim"] == 2 else hc.blast_state(args))
        s.update()
        states.append((args, s))
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    for args, s in states + states[:1]:
        want = s.calcDT()
        full = s.getState(withGhosts=True)
        d_state = _device_copy(torch, full)
        desc = hc.make_desc(dict(args, precision="f64 plain"))
        for _ in range(2):
            out.fill_(-1.0)
            torch.cuda.synchronize()
            code = L.hc_calc_dt_noalloc(ctypes.byref(desc), ctypes.c_void_p(d_state.data_ptr()),
                                        ctypes.c_void_p(out.data_ptr()), None)
            assert code == 0, L.hc_last_error().decode()
            torch.cuda.synchronize()
            assert float(out.item()) == want


def test_noalloc_fixed_dt_and_limits(hc, ctx):
    torch = pytest.importorskip("torch")
    L = hc.load_library()
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    state = torch.zeros(6 * 20, dtype=torch.float64, device="cuda")
    desc = hc.make_desc(dict(cases.c1_sod(gridSize=16), fixedDT=0.125))
    assert L.hc_calc_dt_noalloc(ctypes.byref(desc), ctypes.c_void_p(state.data_ptr()),
                                ctypes.c_void_p(out.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert float(out.item()) == 0.125
    # beyond the fixed scratch array: refused before any launch
    big = hc.make_desc(dict(cases.c3_blast(300)))
    assert L.hc_calc_dt_noalloc(ctypes.byref(big), ctypes.c_void_p(state.data_ptr()),
                                ctypes.c_void_p(out.data_ptr()), None) == -1
    assert b"HC_NOALLOC_MAX_CELLS" in L.hc_last_error()
