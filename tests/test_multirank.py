"""Multi-rank host logic on CPU (gloo, two ranks): the slab decomposition of one
grid with ghost exchange and a min-allreduce of dt reproduces the
single-domain oracle run bit for bit; instances shard without exchange."""
import os
import socket

import numpy as np
import pytest

import cases


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, args, steps, out_dir):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (os.path.join(root, "hydro-cl-lua_gb300"), os.path.join(root, "oracle")):
        sys.path.insert(0, p)
    import torch.distributed as dist
    import decomp
    import hydrocuda
    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # the whole initial state, cut to this rank's slab
    U0 = hydrocuda.kelvin_helmholtz_state(args, seed=2) if args["dim"] == 2 else hydrocuda.sod_state(args)
    sargs, lo, hi = decomp.slab_args(args, rank, world)
    dim = args["dim"]
    n = args["gridSize"]
    grid = U0.reshape(n[1], n[0], 6) if dim == 2 else U0.reshape(n[0], 6)
    mine = grid[lo:hi] if dim == 2 else grid[lo:hi]
    s = oracle.OracleSolver(sargs)
    s.reset_state(mine.reshape(-1, 6))
    # resetState filled the internal faces' ghosts with nothing: exchange, then
    # constrain as the single-domain resetState does (constrainU is per cell)
    full = s.get_full()
    decomp.exchange_ghosts(full, sargs, rank, world, dist)
    s.set_full(full)
    for _ in range(steps):
        dt = decomp.allreduce_min(s.calcDT(), dist)
        full = s.get_full()
        decomp.exchange_ghosts(full, sargs, rank, world, dist)
        s.set_full(full)
        s.step(dt)
        s.t = s.t + dt
    np.save(os.path.join(out_dir, "rank%d.npy" % rank), s.get_interior())
    dist.barrier()
    dist.destroy_process_group()


def run_ranks(args, steps, tmp_path, world=2):
    import torch.multiprocessing as mp
    port = free_port()
    mp.start_processes(_rank_main, args=(world, port, args, steps, str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    return [np.load(tmp_path / ("rank%d.npy" % r)) for r in range(world)]


@pytest.mark.parametrize("boundary", ["freeflow", "periodic"])
def test_slab_decomposition_matches_single_domain(tmp_path, boundary):
    import oracle
    import hydrocuda
    args = cases.c2_kh(24, boundary=boundary, integrator="forward Euler", usePLM="plm cons",
                       slopeLimiter="monotized central")
    args["gridSize"] = [24, 20]
    parts = run_ranks(args, 6, tmp_path)
    whole = oracle.OracleSolver(args)
    whole.reset_state(hydrocuda.kelvin_helmholtz_state(args, seed=2))
    for _ in range(6):
        whole.update()
    ref = whole.get_interior().reshape(20, 24, 6)
    got = np.concatenate([p.reshape(-1, 24, 6) for p in parts], axis=0)
    np.testing.assert_array_equal(got, ref)


def test_slab_bounds_cover_the_axis():
    import decomp
    for n in (7, 8, 1024):
        for world in (1, 2, 3, 8):
            spans = [decomp.slab_bounds(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[k][1] == spans[k + 1][0] for k in range(world - 1))
            assert max(h - l for l, h in spans) - min(h - l for l, h in spans) <= 1


def test_instances_shard_without_overlap():
    import decomp
    items = list(range(37))
    parts = [decomp.shard_instances(items, r, 4) for r in range(4)]
    assert sorted(sum(parts, [])) == items
