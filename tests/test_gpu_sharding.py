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
