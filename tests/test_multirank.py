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


def _bench_rank(rank, world, port, out_dir):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "hydro-cl-lua_gb300")):
        sys.path.insert(0, p)
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    work = bench.workload(count=6, rank=rank)
    sizes = [a["gridSize"][0] for a, _ in work]
    # each rank's own clock and credited work, as bench.py's main has them
    elapsed, credited = bench.aggregate(1.0 + rank, 1000 * (rank + 1), dist)
    np.save(os.path.join(out_dir, "bench%d.npy" % rank),
            np.array([elapsed, credited] + sizes, dtype=np.float64))
    quads = [q for _, q in work]
    import pickle
    with open(os.path.join(out_dir, "quads%d.pkl" % rank), "wb") as f:
        pickle.dump(quads, f)
    dist.barrier()
    dist.destroy_process_group()


def test_bench_replicas_aggregate_over_ranks(tmp_path):
    """bench.py's WORLD_SIZE=2 path on gloo ranks: every rank holds its own
    instances (weak scaling: the same count, different seeds), and the job's
    value is every rank's credited work over the slowest rank's clock."""
    import pickle
    import torch.multiprocessing as mp
    port = free_port()
    mp.start_processes(_bench_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r0, r1 = (np.load(tmp_path / ("bench%d.npy" % r)) for r in range(2))
    for r in (r0, r1):
        assert r[0] == 2.0                      # max of the ranks' 1.0 and 2.0 s
        assert r[1] == 3000                     # 1000 + 2000 cell-updates
    assert len(r0) == len(r1) == 2 + 6
    q0, q1 = (pickle.load(open(tmp_path / ("quads%d.pkl" % r), "rb")) for r in range(2))
    assert all(repr(a) != repr(b) for a, b in zip(q0, q1))   # different instances per rank


def test_bench_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the reference arm's ranks other than 0 exit 0 without work or output."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""
