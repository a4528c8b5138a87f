"""Work split across ranks, host logic on CPU ranks (gloo).

Batches: every grid on exactly one rank, loads balanced to within the largest grid, and the same assignment
computed independently on world_size-2 ranks. One grid in Morton ranges: the ghost lists cover every stencil,
and two ranks that sweep their ranges (with the oracle's node-range functions) and exchange ghosts after every
sweep give the single-rank result bit for bit."""
import os
import socket

import numpy as np
import pytest

from casl_p4est_gb300.sharding import assign_by_size, rank_share


def test_assignment_covers_and_balances():
    rng = np.random.default_rng(3)
    sizes = rng.integers(4000, 130000, 256)
    for world in (1, 2, 3, 8):
        parts = assign_by_size(sizes, world)
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(len(sizes)))
        loads = [int(sizes[p].sum()) for p in parts]
        assert max(loads) - min(loads) <= int(sizes.max())
    with pytest.raises(ValueError):
        assign_by_size(sizes, 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, sizes, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = rank_share(sizes, rank, world)
    # each rank reports its grids; the gathered view must partition the batch
    t = torch.zeros(len(sizes), dtype=torch.int64)
    t[mine] = rank + 1
    dist.all_reduce(t)
    load = torch.tensor([int(np.asarray(sizes)[mine].sum())], dtype=torch.int64)
    loads = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(loads, load)
    q.put((rank, t.tolist(), [int(x) for x in loads]))
    dist.destroy_process_group()


def test_gloo_world2_ranks_agree():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    sizes = list(np.random.default_rng(4).integers(4000, 130000, 64))
    port = _free_port()
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    owners = res[0][1]
    assert res[1][1] == owners
    assert sorted(set(owners)) == [1, 2]  # every grid owned by rank 0 or rank 1, none by both
    assert sum(res[0][2]) == sum(sizes)


# ---- one grid split into Morton ranges --------------------------------------------------------------
from casl_p4est_gb300.sharding import MortonPartition, band_linf_sharded, reinit_schedule, reinitialize_sharded, run_schedule  # noqa: E402

POISON = 1.0e30  # entries a rank neither owns nor receives: any read of them would spoil its results


class OracleBackend:
    """A rank's sweeps on the CPU with the oracle's node-range functions (test infrastructure only)."""

    def __init__(self, og):
        self.og = og
        self.dim = og.dim
        self.N = og.N

    def dd(self, f, out, first, count):
        self.og.compute_derivatives_range(f.numpy(), out.numpy(), first, count)

    def prep(self, phi0, dd0, order_space, limit_high, limit_low, first, count):
        self.dd0 = None if dd0 is None else dd0.numpy()
        self.limits = (limit_high, limit_low)

    def stage(self, order_space, phi0, phin, dd, out, avg_with, first, count):
        hi, lo = self.limits
        ddc = None if (order_space < 2 or dd is None) else dd.numpy()
        dd0 = self.dd0 if order_space > 1 else None
        if avg_with is None:
            self.og.reinit_stage_range(out.numpy(), phi0.numpy(), phin.numpy(), hi, lo, dd0, ddc, first, count)
        else:
            tmp = np.empty(self.N)
            self.og.reinit_stage_range(tmp, phi0.numpy(), phin.numpy(), hi, lo, dd0, ddc, first, count)
            a = avg_with.numpy()
            out.numpy()[first:first + count] = .5 * (a[first:first + count] + tmp[first:first + count])

    def copy(self, src, dst, first, count):
        dst[first:first + count] = src[first:first + count]

    def advect_stage(self, phin, ddq, ddm, vn, dt, out, avg_with, first, count):
        # the oracle computes the quadratic neighbour values inline (ddq is what the GPU sweep reads for them)
        if avg_with is None:
            self.og.advect_stage_range(vn.numpy(), dt, ddm.numpy(), phin.numpy(), out.numpy(), first, count)
        else:
            tmp = np.empty(self.N)
            self.og.advect_stage_range(vn.numpy(), dt, ddm.numpy(), phin.numpy(), tmp, first, count)
            a = avg_with.numpy()
            out.numpy()[first:first + count] = .5 * (a[first:first + count] + tmp[first:first + count])


def _grid(name):
    import grids
    import casl_p4est_gb300 as G
    if name == "circle2d":
        f = grids.circle_2d(3, 7)
        return f, grids.phi0_circle_2d(f)
    if name == "brick2d":
        f = grids.brick_2d(1, 6)
        return f, f.sample(G.shapes.sphere_scaled([0.3, 0.1], 0.6, 0.2, [0.5, 0.5]))
    if name == "flower3d":
        f = grids.flower_3d(3, 5)
        return f, grids.phi0_flower_3d(f)
    f = grids.brick_3d(1, 4)
    return f, f.sample(G.shapes.sphere_scaled([0.7, 0.5, 0.9], 0.3, 0.1, [1, 0.5, 1]))


def test_morton_partition_ghosts_cover_every_stencil():
    import casl_p4est_gb300 as G
    import oracle as O
    f, _ = _grid("flower3d")
    og = O.OracleGrid.from_forest(f)
    rec = og.qnnn(G.qnnn_dtype(3))
    for world in (1, 2, 3, 5):
        part = MortonPartition(rec, world)
        assert part.bounds[0] == 0 and part.bounds[-1] == og.N
        nb = rec["nb"].reshape(og.N, -1)
        for r in range(world):
            b, e = part.bounds[r], part.bounds[r + 1]
            need = set(np.unique(nb[b:e].ravel()).tolist()) - {-1}
            have = set(range(b, e)) | set(part.ghosts[r].tolist())
            assert need <= have
            assert sorted(np.concatenate([v for v in part.recv[r].values()]).tolist() if part.recv[r] else []) == part.ghosts[r].tolist()
            for s, idx in part.send[r].items():  # what r sends s is exactly what s expects from r
                assert np.array_equal(idx, part.recv[s][r])
                assert np.all((idx >= b) & (idx < e))
        if world > 1:
            assert max(len(g) for g in part.ghosts) < 0.25 * og.N  # a halo, not a copy of the grid


def _split_worker(rank, world, port, name, orders, iters, limits, q):
    import torch
    import torch.distributed as dist
    import casl_p4est_gb300 as G
    import oracle as O
    from casl_p4est_gb300.sharding import HaloExchange
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        f, phi0 = _grid(name)
        og = O.OracleGrid.from_forest(f)
        part = MortonPartition(og.qnnn(G.qnnn_dtype(f.dim)), world)
        first, count = part.range_of(rank)
        phi = torch.full((og.N,), POISON, dtype=torch.float64)
        phi[first:first + count] = torch.from_numpy(phi0[first:first + count])
        hi, lo = limits
        reinitialize_sharded(part, rank, phi, OracleBackend(og), HaloExchange(part, rank), iterations=iters, order_space=orders[0],
                             order_pseudotime=orders[1], limit_high=hi, limit_low=lo)
        sizes = [part.range_of(r)[1] for r in range(world)]
        width = max(sizes)
        mine = torch.zeros(width, dtype=torch.float64)
        mine[:count] = phi[first:first + count]
        pieces = [torch.empty(width, dtype=torch.float64) for _ in range(world)]
        dist.all_gather(pieces, mine)
        whole = torch.cat([pieces[r][:sizes[r]] for r in range(world)])
        ref = torch.from_numpy(phi0.copy())
        og.reinitialize(ref.numpy(), orders[0], orders[1], hi, lo, iterations=iters)
        band = band_linf_sharded(part, rank, whole, ref, 0.1)
        q.put((rank, bool(torch.equal(whole, ref)), float((whole - ref).abs().max()), band))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name,orders,limits", [("circle2d", (2, 2), (np.finfo(np.float64).max, -np.finfo(np.float64).max)),
                                                ("brick2d", (1, 2), (0.3, -0.2)),
                                                ("flower3d", (2, 2), (np.finfo(np.float64).max, -np.finfo(np.float64).max)),
                                                ("brick3d", (2, 1), (0.25, -0.15))])
def test_morton_split_on_gloo_world2_equals_one_rank(name, orders, limits):
    """Two CPU ranks, each sweeping its Morton range with the oracle and exchanging the ghosts of phi and of the
    second derivatives after every sweep: bit-identical to the single-rank result; the band check is one
    all-reduce and equals zero."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    port = _free_port()
    q = ctx.Queue()
    procs = [ctx.Process(target=_split_worker, args=(r, 2, port, name, orders, 6, limits, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, equal, diff, band in res:
        assert equal, (rank, diff)
        assert band == 0.0


def test_schedule_matches_the_reference_sweeps():
    ops = reinit_schedule(2, 2, 1)
    kinds = [o[0] for o in ops]
    # phi_0's derivatives and the preparation once, then per iteration dd, stage, dd, stage (+ average), each
    # followed by its ghost update
    assert kinds == ["dd", "exchange", "prep", "dd", "exchange", "stage", "exchange", "dd", "exchange", "stage", "exchange"]
    assert ops[-2] == ("stage", "phi1", "phi", "phi")
    # first order in space: the node's own second derivatives are still swept (the quadratic neighbour
    # values read them) but their ghosts are not exchanged
    assert [o[0] for o in reinit_schedule(1, 1, 2)] == ["dd", "prep", "dd", "stage", "exchange", "dd", "stage", "exchange"]


# ---- interpolation at arbitrary points across a Morton split --------------------------------------
from casl_p4est_gb300.sharding import LeafPartition, interpolate_sharded, sl_advect_sharded  # noqa: E402


class OracleInterp:
    """A rank's point location and interpolation on the CPU with the oracle (test infrastructure only)."""

    def __init__(self, og):
        self.og = og

    def locate(self, xyz):
        import torch
        return torch.from_numpy(self.og.locate(xyz.numpy()).astype(np.int64))

    def interpolate(self, method, F, Fdd, xyz):
        import torch
        if method != 0 and Fdd is None:
            raise ValueError("second derivatives required")
        out = self.og.interpolate(method, F.numpy(), xyz.numpy(), None if Fdd is None else Fdd.numpy())
        return torch.from_numpy(np.ascontiguousarray(out).reshape(F.shape[0], -1))


def _fields(f, og):
    xyz = f.node_xyz()
    d = f.dim
    phi = np.sqrt(((xyz - 0.1) ** 2).sum(1)) - 0.45
    v = np.stack([np.sin(3 * xyz[:, (a + 1) % d]) * (1.0 + 0.3 * a) for a in range(d)])
    vdd = np.stack([og.compute_derivatives(v[a]) for a in range(d)])
    return phi, og.compute_derivatives(phi), v, vdd


def _query_points(f, n, seed):
    rng = np.random.default_rng(seed)
    lo, hi = np.array(f.xyz_min[:f.dim]), np.array(f.xyz_max[:f.dim])
    pts = lo + (hi - lo) * rng.random((n, f.dim))
    pts[: n // 8] = f.node_xyz()[rng.integers(0, f.num_nodes, n // 8)]  # points on nodes, faces and edges
    pts[n // 8: n // 4] = lo - 0.05 + (hi - lo + 0.1) * rng.random((n // 4 - n // 8, f.dim))  # some outside: clipped
    return pts


def _interp_worker(rank, world, port, name, q):
    import torch
    import torch.distributed as dist
    import casl_p4est_gb300 as G
    import oracle as O
    from casl_p4est_gb300.sharding import HaloExchange
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        f, _ = _grid(name)
        og = O.OracleGrid.from_forest(f)
        N, d = og.N, f.dim
        npart = MortonPartition(og.qnnn(G.qnnn_dtype(d)), world)
        lpart = LeafPartition(f.local_nodes(), npart.bounds, world)
        b, e = npart.bounds[rank], npart.bounds[rank + 1]
        phi, phi_dd, v, vdd = _fields(f, og)

        def mine(a):  # this rank's copy: its node range, POISON elsewhere until the exchange fills its ghosts
            t = torch.full(a.shape, POISON, dtype=torch.float64)
            t[..., b:e] = torch.from_numpy(np.ascontiguousarray(a[..., b:e]))
            return t
        F = mine(np.stack([phi, v[0]]))
        Fdd = mine(np.stack([phi_dd, vdd[0]]))
        V, Vdd, P, Pdd = mine(v), mine(vdd), mine(phi), mine(phi_dd)
        ex = HaloExchange(lpart, rank)
        for t, planes in ((F, 2), (Fdd, 2 * d), (V, d), (Vdd, d * d), (P, 1), (Pdd, d)):
            ex(t.view(-1), planes)
        # every rank asks for its own share of the query points
        pts_all = _query_points(f, 3000, 11)
        share = np.array_split(np.arange(len(pts_all)), world)[rank]
        pts = torch.from_numpy(pts_all[share])
        res = {}
        for method in (0, 2, 4):
            got = interpolate_sharded(lpart, rank, pts, OracleInterp(og), method, F, None if method == 0 else Fdd)
            ref = og.interpolate(method, np.stack([phi, v[0]]), pts_all[share], None if method == 0 else np.stack([phi_dd, vdd[0]]))
            res[method] = bool(np.array_equal(got.numpy(), ref))
        # the semi-Lagrangian step for this rank's nodes of the same grid (the grid at n+1 equal to the grid at n)
        xyz = torch.from_numpy(f.node_xyz()[b:e])
        dt = 0.7 * float(f.dxyz_min()[1])
        got = sl_advect_sharded(lpart, rank, xyz, dt, V, Vdd, P, Pdd, OracleInterp(og), f.xyz_min[:d], f.xyz_max[:d])
        ref = og.sl_advect(f.node_xyz()[b:e], dt, v, phi, vdd=vdd, phi_dd=phi_dd)
        res["sl"] = bool(np.array_equal(got.numpy(), ref))
        res["forwarded"] = int(sum(len(x) for x in lpart.recv[rank].values()))
        q.put((rank, res))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name,world", [("circle2d", 2), ("flower3d", 2), ("brick3d", 3)])
def test_forwarded_interpolation_on_gloo_equals_one_rank(name, world):
    """Points located in another rank's leaves are forwarded to it and the values sent back (the query/reply
    exchange of my_p4est_interpolation_t): linear, quadratic non-oscillatory and continuous-v2 interpolation and
    the semi-Lagrangian step on CPU ranks give the single-rank results bit for bit; each rank's copies of the
    fields hold only its node range and the corner ghosts of its leaves."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    port = _free_port()
    q = ctx.Queue()
    procs = [ctx.Process(target=_interp_worker, args=(r, world, port, name, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, r in res:
        assert r[0] and r[2] and r[4] and r["sl"], (rank, r)
        assert r["forwarded"] > 0


def test_leaf_partition_ghosts_cover_every_leaf_corner():
    import oracle as O
    f, _ = _grid("flower3d")
    og = O.OracleGrid.from_forest(f)
    ln = f.local_nodes()
    for world in (1, 2, 5):
        nb = [(og.N * r) // world for r in range(world + 1)]
        lp = LeafPartition(ln, nb, world)
        assert lp.bounds[0] == 0 and lp.bounds[-1] == len(ln)
        for r in range(world):
            need = set(np.unique(ln[lp.bounds[r]:lp.bounds[r + 1]]).tolist())
            have = set(range(nb[r], nb[r + 1])) | set(lp.ghosts[r].tolist())
            assert need <= have
            for s, idx in lp.send[r].items():
                assert np.array_equal(idx, lp.recv[s][r])
        owners = lp.owner_of_leaves(np.arange(len(ln)))
        assert np.all(np.diff(owners) >= 0) and owners[0] == 0 and owners[-1] == world - 1


# ---- normal advection across a Morton split ---------------------------------------------------------
from casl_p4est_gb300.sharding import advect_normal_sharded  # noqa: E402


def _advect_worker(rank, world, port, name, given_dd, two_velocities, q):
    import torch
    import torch.distributed as dist
    import casl_p4est_gb300 as G
    import oracle as O
    from casl_p4est_gb300.sharding import HaloExchange
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        f, phi0 = _grid(name)
        og = O.OracleGrid.from_forest(f)
        N, d = og.N, f.dim
        part = MortonPartition(og.qnnn(G.qnnn_dtype(d)), world)
        first, count = part.range_of(rank)
        xyz = f.node_xyz()
        vn = 0.8 * np.sin(4 * xyz[:, 0] + 1.0) * np.cos(3 * xyz[:, 1])
        vn1 = vn + 0.3 * np.cos(2 * xyz[:, 0]) if two_velocities else None
        dt = 0.5 * og.advect_cfl_dt(np.abs(vn) if vn1 is None else np.maximum(np.abs(vn), np.abs(vn1)))
        dd0 = og.compute_derivatives(phi0)

        def mine(a):
            t = torch.full(a.shape, POISON, dtype=torch.float64)
            t[..., first:first + count] = torch.from_numpy(np.ascontiguousarray(a[..., first:first + count]))
            return t
        phi = mine(phi0)
        pdd = mine(dd0).reshape(-1) if given_dd else None
        advect_normal_sharded(part, rank, phi, mine(vn), dt, OracleBackend(og), HaloExchange(part, rank),
                              vn_np1=None if vn1 is None else mine(vn1), phi_dd=pdd)
        ref = phi0.copy()
        ref_dd = dd0.copy()
        og.advect_in_normal_direction(vn, ref, dt, vn_np1=vn1, phi_dd=ref_dd if given_dd else None)
        ok = bool(np.array_equal(phi.numpy()[first:first + count], ref[first:first + count]))
        if given_dd:
            ok = ok and bool(np.array_equal(pdd.view(d, N).numpy()[:, first:first + count], ref_dd[:, first:first + count]))
        q.put((rank, ok, float(np.max(np.abs(phi.numpy()[first:first + count] - ref[first:first + count])))))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name,given_dd,two", [("circle2d", False, False), ("flower3d", True, True), ("brick3d", False, True),
                                               ("brick2d", True, False)])
def test_advection_split_on_gloo_world2_equals_one_rank(name, given_dd, two):
    """advect_in_normal_direction split into Morton ranges on two CPU ranks (the oracle's node-range sweeps, ghosts of
    phi and of the second derivatives exchanged after every sweep): the owned values, and the caller's second
    derivatives when given, equal the single-rank result bit for bit."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    port = _free_port()
    q = ctx.Queue()
    procs = [ctx.Process(target=_advect_worker, args=(r, 2, port, name, given_dd, two, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ok, diff in res:
        assert ok, (rank, diff)


def test_advect_schedule_follows_the_reference():
    kinds = [o[0] for o in __import__("casl_p4est_gb300.sharding", fromlist=["advect_schedule"]).advect_schedule(False)]
    assert kinds == ["dd", "exchange", "clone", "astage", "exchange", "dd", "exchange", "astage", "copy", "exchange"]


def test_two_ring_partition_covers_second_neighbours():
    import casl_p4est_gb300 as G
    import oracle as O
    f, _ = _grid("flower3d")
    og = O.OracleGrid.from_forest(f)
    rec = og.qnnn(G.qnnn_dtype(3))
    nb = rec["nb"].reshape(og.N, -1)
    for world in (2, 3):
        p1 = MortonPartition(rec, world)
        p2 = MortonPartition(rec, world, rings=2)
        for r in range(world):
            b, e = p2.bounds[r], p2.bounds[r + 1]
            ring1 = np.unique(nb[b:e].ravel())
            ring1 = ring1[ring1 >= 0]
            ring2 = np.unique(nb[ring1].ravel())
            need = set(ring2[ring2 >= 0].tolist()) - set(range(b, e))
            assert need == set(p2.ghosts[r].tolist())
            assert set(p1.ghosts[r].tolist()) <= set(p2.ghosts[r].tolist())
            for s, idx in p2.send[r].items():
                assert np.array_equal(idx, p2.recv[s][r])


def _slots_worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    import casl_p4est_gb300 as G
    import oracle as O
    from casl_p4est_gb300.sharding import HaloExchange
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        f, _ = _grid("flower3d")
        og = O.OracleGrid.from_forest(f)
        part = MortonPartition(og.qnnn(G.qnnn_dtype(3)), world, rings=2)
        N = part.N
        slots = np.random.default_rng(9).permutation(N).astype(np.int32)  # node -> slot, the same on every rank
        truth = np.arange(N, dtype=np.float32) * 0.5 + 1.0  # a value per node
        first, count = part.range_of(rank)
        arr = torch.full((N,), -7.0, dtype=torch.float32)  # slot order; only this rank's nodes known
        owned = np.arange(first, first + count)
        arr[torch.as_tensor(slots[owned], dtype=torch.int64)] = torch.from_numpy(truth[owned])
        HaloExchange(part, rank, slots=slots)(arr, 1)
        g = part.ghosts[rank]
        ok = bool(np.array_equal(arr.numpy()[slots[g]], truth[g])) and bool(np.array_equal(arr.numpy()[slots[owned]], truth[owned]))
        q.put((rank, ok))
    finally:
        dist.destroy_process_group()


def test_slot_ordered_ghost_exchange_on_gloo_world2():
    """The mixed split's ghost update runs on arrays in the level set's slot order (HaloExchange(..., slots=)): on two
    CPU ranks every ghost slot receives its owner's value and no owned slot changes."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    port = _free_port()
    q = ctx.Queue()
    procs = [ctx.Process(target=_slots_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(ok for _, ok in res), res


def _empty_share_worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    import casl_p4est_gb300 as G
    import oracle as O
    from casl_p4est_gb300.sharding import HaloExchange
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        f, _ = _grid("circle2d")
        og = O.OracleGrid.from_forest(f)
        npart = MortonPartition(og.qnnn(G.qnnn_dtype(2)), world)
        lpart = LeafPartition(f.local_nodes(), npart.bounds, world)
        b, e = npart.bounds[rank], npart.bounds[rank + 1]
        phi, phi_dd, _, _ = _fields(f, og)
        F = torch.full((1, og.N), POISON, dtype=torch.float64)
        F[0, b:e] = torch.from_numpy(phi[b:e])
        Fdd = torch.full((1, 2, og.N), POISON, dtype=torch.float64)
        Fdd[0, :, b:e] = torch.from_numpy(phi_dd[:, b:e])
        ex = HaloExchange(lpart, rank)
        ex(F.view(-1), 1)
        ex(Fdd.view(-1), 2)
        pts_all = _query_points(f, 500, 3)
        mine = pts_all if rank == 0 else pts_all[:0]  # rank 1 asks for nothing but serves rank 0's remote points
        got = interpolate_sharded(lpart, rank, torch.from_numpy(mine), OracleInterp(og), 4, F, Fdd)
        ref = og.interpolate(4, phi.reshape(1, -1), mine, phi_dd.reshape(1, 2, -1)) if len(mine) else np.empty((1, 0))
        q.put((rank, tuple(got.shape), bool(np.array_equal(got.numpy(), ref))))
    finally:
        dist.destroy_process_group()


def test_forwarded_interpolation_with_a_rank_asking_nothing():
    """A rank with no points of its own still answers the points forwarded to it, and gets a (nf, 0) result."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    port = _free_port()
    q = ctx.Queue()
    procs = [ctx.Process(target=_empty_share_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] == (1, 500) and res[0][2], res
    assert res[1][1] == (1, 0) and res[1][2], res
