"""The per-rank GPU sweeps of a Morton-range split, on the one GPU of this machine.

Every run here has one GPU, so the ranks of a split are emulated in one process: each rank has its own
full-length arrays and sweeps only its Morton range with the node-range kernels (ShardBackend), and the ghost
update between two sweeps copies, for every rank, the values its ghosts take from their owners. The ranks'
kernels never wait on one another (each launch finishes before the next starts). The result must equal the
single-rank FP64 reinitialisation bit for bit. The distributed exchange itself (HaloExchange over
torch.distributed) is covered on CPU ranks in test_sharding.py."""
import numpy as np
import pytest

import casl_p4est_gb300 as G
from casl_p4est_gb300.sharding import MortonPartition, ShardBackend, reinit_schedule, run_schedule

from grids import brick_2d, brick_3d, circle_2d, flower_3d, phi0_circle_2d, phi0_flower_3d

pytestmark = pytest.mark.gpu

POISON = 1.0e30

GRIDS = {
    "circle2d": (lambda: circle_2d(3, 8), phi0_circle_2d),
    "brick2d": (lambda: brick_2d(1, 7), lambda f: f.sample(G.shapes.sphere_scaled([0.3, 0.1], 0.6, 0.2, [0.5, 0.5]))),
    "flower3d": (lambda: flower_3d(3, 6), phi0_flower_3d),
    "brick3d": (lambda: brick_3d(1, 5), lambda f: f.sample(G.shapes.sphere_scaled([0.7, 0.5, 0.9], 0.3, 0.1, [1, 0.5, 1]))),
}


def lockstep(part, backend, phi0, order_space, order_pseudotime, iterations, limit_high, limit_low):
    """All ranks' schedules in lockstep on one device; returns the owned values put together."""
    import torch
    N, D, W = part.N, backend.dim, part.world
    ranks = []
    for r in range(W):
        first, count = part.range_of(r)
        phi = torch.full((N,), POISON, dtype=torch.float64, device="cuda")
        phi[first:first + count] = phi0[first:first + count]
        arrays = {"phi": phi, "phi1": torch.empty_like(phi),
                  "dd0": torch.full((D * N,), POISON, dtype=torch.float64, device="cuda"),
                  "ddc": torch.full((D * N,), POISON, dtype=torch.float64, device="cuda")}
        ranks.append((first, count, arrays))

    def exchange_all(name, planes):
        for r in range(W):
            dst = ranks[r][2][name].view(planes, N)
            for s, idx in part.recv[r].items():
                i = torch.as_tensor(idx, dtype=torch.int64, device="cuda")
                dst[:, i] = ranks[s][2][name].view(planes, N)[:, i]

    exchange_all("phi", 1)
    for r in range(W):
        ranks[r][2]["phi0"] = ranks[r][2]["phi"].clone()
    for op in reinit_schedule(order_space, order_pseudotime, iterations):
        if op[0] == "exchange":
            exchange_all(op[1], D if op[2] else 1)
            continue
        for first, count, arrays in ranks:
            run_schedule([op], backend, arrays, first, count, None, D, order_space, limit_high, limit_low)
    torch.cuda.synchronize()
    return torch.cat([arrays["phi"][first:first + count] for first, count, arrays in ranks]).cpu().numpy()


@pytest.mark.parametrize("name", sorted(GRIDS))
@pytest.mark.parametrize("world", [1, 3])
def test_morton_split_equals_one_rank(name, world):
    import torch
    build, phi0_of = GRIDS[name]
    f = build()
    phi0 = phi0_of(f)
    ngbd = G.my_p4est_node_neighbors_t(f)
    ls = G.my_p4est_level_set_t(ngbd)
    part = MortonPartition(ngbd.get_neighbors(), world)
    big = np.finfo(np.float64).max
    for (os_, ot), (hi, lo) in [((2, 2), (big, -big)), ((1, 2), (0.3, -0.2)), ((2, 1), (big, -big))]:
        ref = phi0.copy()
        ls.reinitialize_within_range_of_phi_0(ref, os_, ot, hi, lo, 7)
        got = lockstep(part, ShardBackend(ls), torch.from_numpy(phi0).cuda(), os_, ot, 7, hi, lo)
        assert np.array_equal(got, ref), (name, world, os_, ot, np.max(np.abs(got - ref)))


@pytest.mark.parametrize("name", ["circle2d", "flower3d", "brick3d"])
def test_forwarded_interpolation_lockstep_equals_one_rank(name):
    """Interpolation across a Morton split of the leaves on the GPU (ShardInterpBackend), ranks emulated in one
    process: every rank locates its points, each point is interpolated by the rank owning its leaf from that
    rank's own copies of the fields (its node range plus the corner ghosts of its leaves, POISON elsewhere),
    and the values equal the single-rank interpolation bit for bit. The message exchange itself
    (interpolate_sharded over torch.distributed) is covered on CPU ranks in test_sharding.py."""
    import torch
    from casl_p4est_gb300.interpolation import my_p4est_interpolation_nodes_t
    from casl_p4est_gb300.sharding import LeafPartition, ShardInterpBackend
    build, phi0_of = GRIDS[name]
    f = build()
    ngbd = G.my_p4est_node_neighbors_t(f)
    ls = G.my_p4est_level_set_t(ngbd)
    N, d, W = f.num_nodes, f.dim, 3
    phi = phi0_of(f)
    xyz = f.node_xyz()
    v0 = np.sin(3 * xyz[:, 1]) * np.cos(2 * xyz[:, 0])
    F = np.stack([phi, v0])
    Fdd = np.stack([ls.compute_derivatives(phi), ls.compute_derivatives(v0)]).reshape(2, d, N)
    rng = np.random.default_rng(5)
    lo, hi = np.array(f.xyz_min[:d]), np.array(f.xyz_max[:d])
    pts = lo - 0.02 + (hi - lo + 0.04) * rng.random((4000, d))
    pts[:500] = xyz[rng.integers(0, N, 500)]
    nb = [(N * r) // W for r in range(W + 1)]
    lp = LeafPartition(f.local_nodes(), nb, W)
    be = ShardInterpBackend(ls)
    interp = my_p4est_interpolation_nodes_t(ls)
    for method in (0, 2, 4):
        ref = interp.interpolate_points(pts, F, method, None if method == 0 else Fdd)
        copies = []
        for r in range(W):
            keep = np.zeros(N, bool)
            keep[nb[r]:nb[r + 1]] = True
            keep[lp.ghosts[r]] = True
            Fr = np.where(keep, F, 1e30)
            Fddr = np.where(keep, Fdd, 1e30)
            copies.append((torch.from_numpy(Fr).cuda(), torch.from_numpy(np.ascontiguousarray(Fddr)).cuda()))
        P = torch.from_numpy(pts).cuda()
        owner = lp.owner_of_leaves(be.locate(P))
        got = torch.empty((2, len(pts)), dtype=torch.float64, device="cuda")
        for r in range(W):
            sel = torch.nonzero(owner == r).flatten()
            if len(sel):
                got[:, sel] = be.interpolate(method, copies[r][0], None if method == 0 else copies[r][1], P[sel])
        torch.cuda.synchronize()
        assert np.array_equal(got.cpu().numpy(), ref), (name, method)
        assert len(torch.unique(owner)) == W


@pytest.mark.parametrize("name", sorted(GRIDS))
@pytest.mark.parametrize("world", [1, 3])
def test_advection_split_lockstep_equals_one_rank(name, world):
    """advect_in_normal_direction over Morton ranges on the GPU (ShardBackend's node-range sweeps, lsg_advect_stage_
    range_device), the ranks in lockstep in one process with their ghosts copied between sweeps: the same bits as the
    single-GPU FP64 advection, with and without the caller's second derivatives and a second velocity."""
    import torch
    from casl_p4est_gb300.sharding import advect_schedule, run_advect_schedule
    build, phi0_of = GRIDS[name]
    f = build()
    phi0 = phi0_of(f)
    ngbd = G.my_p4est_node_neighbors_t(f)
    ls = G.my_p4est_level_set_t(ngbd)
    part = MortonPartition(ngbd.get_neighbors(), world)
    N, D = part.N, f.dim
    xyz = f.node_xyz()
    vn = 0.8 * np.sin(4 * xyz[:, 0] + 1.0) * np.cos(3 * xyz[:, 1])
    vn1 = vn + 0.3 * np.cos(2 * xyz[:, 0])
    backend = ShardBackend(ls)
    for given_dd, two in ((False, False), (True, True)):
        dt = 0.3 * float(f.dxyz_min()[1]) / float(np.max(np.maximum(np.abs(vn), np.abs(vn1))))
        dd0 = ls.compute_derivatives(phi0).reshape(D, N)
        ref = phi0.copy()
        ref_dd = dd0.copy()
        ls.advect_in_normal_direction(vn, ref, dt, phi_xx=ref_dd if given_dd else None, vn_np1=vn1 if two else None, precision="fp64")
        ranks = []
        for r in range(world):
            first, count = part.range_of(r)

            def mine(a):
                t = torch.full(a.shape, POISON, dtype=torch.float64)
                t[..., first:first + count] = torch.from_numpy(np.ascontiguousarray(a[..., first:first + count]))
                return t.cuda().reshape(-1) if a.ndim > 1 else t.cuda()
            arrays = {"phi": mine(phi0), "vn": mine(vn), "vn1": mine(vn1 if two else vn),
                      "tmp": torch.empty(N, dtype=torch.float64, device="cuda"),
                      "ddq": torch.full((D * N,), POISON, dtype=torch.float64, device="cuda")}
            if given_dd:
                arrays["phi_dd"] = mine(dd0)
            ranks.append((first, count, arrays))

        def exchange_all(name_, planes):
            for r in range(world):
                dst = ranks[r][2][name_].view(planes, N)
                for s, idx in part.recv[r].items():
                    i = torch.as_tensor(idx, dtype=torch.int64, device="cuda")
                    dst[:, i] = ranks[s][2][name_].view(planes, N)[:, i]

        exchange_all("phi", 1)
        for op in advect_schedule(given_dd):
            if op[0] == "exchange":
                exchange_all(op[1], D if op[2] else 1)
                continue
            for first, count, arrays in ranks:
                run_advect_schedule([op], backend, arrays, first, count, None, D, dt)
        torch.cuda.synchronize()
        got = torch.cat([arrays["phi"][first:first + count] for first, count, arrays in ranks]).cpu().numpy()
        assert np.array_equal(got, ref), (name, world, given_dd, np.max(np.abs(got - ref)))
        if given_dd:
            got_dd = torch.cat([arrays["phi_dd"].view(D, N)[:, first:first + count] for first, count, arrays in ranks], dim=1).cpu().numpy()
            assert np.array_equal(got_dd, ref_dd), (name, world)


@pytest.mark.parametrize("name", sorted(GRIDS))
@pytest.mark.parametrize("world", [1, 3])
def test_mixed_split_lockstep_equals_one_rank(name, world):
    """The mixed-precision reinitialisation over Morton ranges (two rings of ghosts; ShardMixedBackend: each rank's
    level set prepares every node, leaves the ones it does not own out of the updates, and runs stage by stage), the
    ranks in lockstep in one process with the FP32 field's ghosts copied after every stage: the owned values equal
    the single-GPU mixed result bit for bit."""
    import torch
    from casl_p4est_gb300.sharding import ShardMixedBackend
    build, phi0_of = GRIDS[name]
    f = build()
    phi0 = phi0_of(f)
    ngbd = G.my_p4est_node_neighbors_t(f)
    part = MortonPartition(ngbd.get_neighbors(), world, rings=2)
    N = part.N
    iters = 6
    ref = phi0.copy()
    G.my_p4est_level_set_t(ngbd, precision="mixed").reinitialize_2nd_order(ref, iters)
    backends, phis = [], []
    for r in range(world):
        first, count = part.range_of(r)
        keep = np.zeros(N, bool)
        keep[first:first + count] = True
        keep[part.ghosts[r]] = True
        phi = torch.from_numpy(np.where(keep, phi0, POISON)).cuda()
        mask = torch.zeros(N, dtype=torch.float64, device="cuda")
        mask[first:first + count] = 1.0
        b = ShardMixedBackend(G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f), precision="mixed"))
        b.begin(phi, mask, 2, np.finfo(np.float64).max, -np.finfo(np.float64).max)
        backends.append(b)
        phis.append(phi)
    fields = [(b.field(0), b.field(1)) for b in backends]
    slots = backends[0].slots().long().cpu().numpy()

    def exchange_all(which):
        for r in range(world):
            for s, idx in part.recv[r].items():
                sl = torch.as_tensor(slots[idx], dtype=torch.int64, device="cuda")
                fields[r][which][sl] = fields[s][which][sl]

    for _ in range(iters):
        for b in backends:
            b.stage(2, 0)
        exchange_all(1)
        for b in backends:
            b.stage(2, 1)
        exchange_all(0)
    for b, phi in zip(backends, phis):
        b.end(phi)
    torch.cuda.synchronize()
    got = np.concatenate([phis[r].cpu().numpy()[part.bounds[r]:part.bounds[r + 1]] for r in range(world)])
    assert np.array_equal(got, ref), (name, world, np.max(np.abs(got - ref)))
