"""Slab decomposition of one grid across ranks (host logic).

hydro-cl-lua's only multi-device mode, ``choppedup`` (hydro/solver/choppedup.lua),
splits a grid into blocks, takes the minimum of the blocks' dt on the host
(choppedup.lua:344-400) and copies the ghost layers between neighbouring
blocks once per update with clEnqueueCopyBufferRect (choppedup.lua:193-230).

Here a grid is cut into slabs along its last active axis.  Per update every
rank computes the CFL dt of its slab, the ranks agree on the minimum with one
FP64 min-allreduce, and every rank sends the numGhost = 2 layers next to each
internal face to its neighbour before each derivative evaluation.  With one
exchange per derivative evaluation the decomposed run reproduces the
single-domain run exactly; with one exchange per update (the reference's
choice) that holds for forward Euler only.

Two forms of the exchange: ``exchange_ghosts`` on a whole host array in the
reference's layout (AoS-6 cons_t, x-fastest, ghosts included), for the
oracle; and ``exchange_slabs`` / ``update`` on a libhydrocuda solver, through
hc_solver_get_slab / hc_solver_set_slab / hc_solver_stage, so each rank's slab
lives on its device and only the two-layer slabs next to the internal faces
cross to the host and over ``torch.distributed`` point-to-point messages
(gloo here; the slabs are small, host-staged).
"""
import numpy as np

NUM_GHOST = 2


def slab_bounds(n, rank, world):
    """[lo, hi) interior cells of `rank` along an axis of n cells (balanced, contiguous)."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def slab_args(args, rank, world):
    """The solver args of one slab: its share of the last active axis, its
    domain extent, and boundary 'none' on internal faces (their ghosts come from
    the neighbours)."""
    dim = int(args["dim"])
    ax = dim - 1
    gs = list(args["gridSize"]) if not isinstance(args["gridSize"], int) else [args["gridSize"]]
    mins = list(args.get("mins", [-1, -1, -1]))
    maxs = list(args.get("maxs", [1, 1, 1]))
    n = gs[ax]
    lo, hi = slab_bounds(n, rank, world)
    dx = (maxs[ax] - mins[ax]) / n
    out = dict(args)
    out["gridSize"] = gs[:ax] + [hi - lo] + gs[ax + 1:]
    m, M = list(mins), list(maxs)
    m[ax] = mins[ax] + lo * dx
    M[ax] = mins[ax] + hi * dx
    out["mins"], out["maxs"] = m, M
    bnd = args.get("boundary", {}) or {}
    if isinstance(bnd, str):
        bnd = {k: bnd for k in ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")}
    bnd = dict(bnd)
    names = ("x", "y", "z")
    periodic = bnd.get(names[ax] + "min", "freeflow") == "periodic"
    if rank > 0 or periodic:
        bnd[names[ax] + "min"] = "none"
    if rank < world - 1 or periodic:
        bnd[names[ax] + "max"] = "none"
    out["boundary"] = bnd
    out["_periodic_split"] = periodic
    return out, lo, hi


def _full_shape(args):
    dim = int(args["dim"])
    gs = list(args["gridSize"]) if not isinstance(args["gridSize"], int) else [args["gridSize"]]
    shape = [gs[k] + 2 * NUM_GHOST if k < dim else 1 for k in range(3)]
    return shape  # x, y, z


def as_grid(full, args):
    """View a (numCells, 6) x-fastest array as [z][y][x][6]."""
    sx, sy, sz = _full_shape(args)
    return full.reshape(sz, sy, sx, 6)


def exchange_ghosts(full, args, rank, world, dist):
    """Fills the ghost layers on the internal faces of this rank's slab from its
    neighbours' edge layers (last active axis).  `full` is the slab's whole
    AoS-6 state, ghosts included; modified in place."""
    import torch
    dim = int(args["dim"])
    g = as_grid(full, args)
    G = NUM_GHOST
    # numpy axis of the last active axis in [z][y][x] order
    npax = {1: 2, 2: 1, 3: 0}[dim]

    def take(sl):
        idx = [slice(None)] * 4
        idx[npax] = sl
        return tuple(idx)

    reqs = []
    bufs = []
    n = g.shape[npax]
    periodic = bool(args.get("_periodic_split", False))
    down = rank - 1 if rank > 0 else (world - 1 if periodic else None)
    up = rank + 1 if rank < world - 1 else (0 if periodic else None)
    # my first interior layers go down (tag 1), my last interior layers go up
    # (tag 2); the tags keep the two messages apart when both neighbours are
    # the same rank (two ranks, periodic)
    if down is not None:
        send = torch.from_numpy(np.ascontiguousarray(g[take(slice(G, 2 * G))]))
        recv = torch.empty_like(send)
        reqs.append(dist.isend(send, down, tag=1))
        reqs.append(dist.irecv(recv, down, tag=2))
        bufs.append((slice(0, G), recv, send))
    if up is not None:
        send = torch.from_numpy(np.ascontiguousarray(g[take(slice(n - 2 * G, n - G))]))
        recv = torch.empty_like(send)
        reqs.append(dist.isend(send, up, tag=2))
        reqs.append(dist.irecv(recv, up, tag=1))
        bufs.append((slice(n - G, n), recv, send))
    for r in reqs:
        r.wait()
    for sl, recv, _ in bufs:
        g[take(sl)] = recv.numpy()


def _neighbours(args, rank, world):
    periodic = bool(args.get("_periodic_split", False))
    down = rank - 1 if rank > 0 else (world - 1 if periodic else None)
    up = rank + 1 if rank < world - 1 else (0 if periodic else None)
    return down, up


def exchange_slabs(solver, args, rank, world, dist):
    """Before a stage: this slab's two layers next to each internal face go to
    the neighbour across it, and the neighbour's become this slab's ghosts, in
    the state the solver's next stage reads (tags as in exchange_ghosts)."""
    import torch
    ax = int(args["dim"]) - 1
    down, up = _neighbours(args, rank, world)
    reqs, recvs = [], []
    if down is not None:
        send = torch.from_numpy(solver.get_slab(ax, 0))
        recv = torch.empty_like(send)
        reqs.append(dist.isend(send, down, tag=1))
        reqs.append(dist.irecv(recv, down, tag=2))
        recvs.append((0, recv, send))
    if up is not None:
        send = torch.from_numpy(solver.get_slab(ax, 1))
        recv = torch.empty_like(send)
        reqs.append(dist.isend(send, up, tag=2))
        reqs.append(dist.irecv(recv, up, tag=1))
        recvs.append((1, recv, send))
    for r in reqs:
        r.wait()
    for side, recv, _ in recvs:
        solver.set_slab(ax, side, recv.numpy())


def update(solver, args, rank, world, dist):
    """One update of the decomposed grid on a libhydrocuda solver (fused form):
    the ranks' minimum dt, then for every Runge-Kutta stage the slab exchange
    and the stage; t advances by dt.  Returns dt."""
    dt = allreduce_min(solver.calcDT(), dist)
    for _ in range(solver.num_stages):
        exchange_slabs(solver, args, rank, world, dist)
        solver.stage(dt)
    solver.t = solver.t + dt
    return dt


def solver_args(sargs):
    """slab_args without the decomposition's own keys (for hydrocuda.Solver)."""
    return {k: v for k, v in sargs.items() if not k.startswith("_")}


def allreduce_min(value, dist):
    """The ranks' common dt: FP64 min-allreduce."""
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MIN)
    return float(t.item())


def shard_instances(items, rank, world):
    """Independent instances spread over ranks round-robin (no data exchange)."""
    return [it for k, it in enumerate(items) if k % world == rank]
