"""One grid cut into slabs across two ranks, each rank stepping its slab with
a libhydrocuda solver (fused forms) on the one GPU, the ranks exchanging the
two-layer slabs next to their internal faces through the host over gloo
before every Runge-Kutta stage (hc_solver_get_slab / hc_solver_set_slab /
hc_solver_stage) and agreeing on the minimum dt: the FP64 result is bit-equal
to the single-domain oracle run, the FP32 result bit-equal to the single-domain
FP32 solver.  The ranks' kernels never wait on one another (the exchange is
host-side between stages), so two ranks on one device are only two contexts."""
import os

import numpy as np
import pytest

import cases
from test_multirank import free_port

pytestmark = pytest.mark.gpu


def _state(hc, args):
    if args["dim"] == 1:
        return hc.sod_state(args)
    if args["dim"] == 2:
        return hc.kelvin_helmholtz_state(args, seed=2)
    return hc.blast_state(args)


def _grid(U, args):
    n = list(args["gridSize"])[:args["dim"]]
    return U.reshape(tuple(reversed(n)) + (6,))


def _rank_main(rank, world, port, args, precision, steps, out_dir):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "hydro-cl-lua_gb300"))
    import torch.distributed as dist
    import decomp
    import hydrocuda as hc
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    hc.load_library()
    sargs, lo, hi = decomp.slab_args(args, rank, world)
    mine = _grid(_state(hc, args), args)[lo:hi].reshape(-1, 6)
    s = hc.Solver(hc.default_context(), precision=precision, **decomp.solver_args(sargs))
    s.resetState(mine)
    dts = []
    for _ in range(steps):
        dts.append(decomp.update(s, sargs, rank, world, dist))
    np.save(os.path.join(out_dir, "rank%d.npy" % rank), s.getState())
    np.save(os.path.join(out_dir, "dt%d.npy" % rank), np.array(dts + [s.t]))
    dist.barrier()
    dist.destroy_process_group()


def _run_ranks(args, precision, steps, tmp_path, world=2):
    import torch.multiprocessing as mp
    mp.start_processes(_rank_main, args=(world, free_port(), args, precision, steps, str(tmp_path)),
                       nprocs=world, join=True, start_method="spawn")
    parts = [np.load(tmp_path / ("rank%d.npy" % r)) for r in range(world)]
    dts = [np.load(tmp_path / ("dt%d.npy" % r)) for r in range(world)]
    return parts, dts


def _joined(parts, args):
    n = list(args["gridSize"])[:args["dim"]]
    inner = tuple(reversed(n[:-1])) + (6,)
    return np.concatenate([p.reshape((-1,) + inner) for p in parts], axis=0).reshape(-1, 6)


CASES = {
    "kh-periodic-rk3tvd": cases.c2_kh(32, integrator="Runge-Kutta 3, TVD", gridSize=[32, 30]),
    "kh-freeflow-rk3tvd": cases.c2_kh(32, integrator="Runge-Kutta 3, TVD", gridSize=[32, 30], boundary="freeflow"),
    "sod-freeflow-rk4": cases.c1_sod(integrator="Runge-Kutta 4", gridSize=[256]),
    # forward Euler alternates the state between two buffers (the slab calls
    # follow the rotation)
    "kh-periodic-fe": cases.c2_kh(32, integrator="forward Euler", gridSize=[32, 30]),
    "blast-freeflow-rk2": cases.c3_blast(12, gridSize=[12, 10, 14]),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_slabs_fp64_bit_equal_to_the_single_domain_oracle(hc, tmp_path, name):
    import oracle
    args = CASES[name]
    steps = 5
    parts, dts = _run_ranks(args, "f64", steps, tmp_path)
    whole = oracle.OracleSolver(args)
    whole.reset_state(_state(hc, args))
    ref_dts = [whole.update() for _ in range(steps)]
    np.testing.assert_array_equal(dts[0], dts[1])
    got = _joined(parts, args)
    np.testing.assert_array_equal(got[:, :5], whole.get_interior()[:, :5])
    np.testing.assert_array_equal(dts[0][:steps], np.array(ref_dts))
    assert dts[0][steps] == whole.t


@pytest.mark.parametrize("name", ["kh-periodic-rk3tvd", "blast-freeflow-rk2"])
def test_slabs_fp32_bit_equal_to_the_single_domain_solver(hc, ctx, tmp_path, name):
    args = CASES[name]
    steps = 5
    parts, _ = _run_ranks(args, "f32", steps, tmp_path)
    s = hc.Solver(ctx, precision="f32", **args)
    s.resetState(_state(hc, args))
    for _ in range(steps):
        s.update()
    np.testing.assert_array_equal(_joined(parts, args), s.getState())


def test_stage_calls_guard_whole_updates(hc, ctx):
    args = CASES["kh-periodic-rk3tvd"]
    s = hc.Solver(ctx, precision="f64", **args)
    s.resetState(_state(hc, args))
    assert s.num_stages == 3
    dt = s.calcDT()
    s.stage(dt)
    with pytest.raises(hc.HydroCudaError) as e:
        s.update()
    assert e.value.code == -8          # HC_ERR_STATE: an update is part done
    s.stage(dt)
    s.stage(dt)
    s.update()                         # the staged update is complete
    p = hc.Solver(ctx, precision="f64 plain", **args)
    with pytest.raises(hc.HydroCudaError):
        p.stage(dt)
