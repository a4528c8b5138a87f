"""Batch sharding across ranks (host logic): every grid on exactly one rank, loads balanced to within
the largest grid, and the same assignment computed independently on world_size-2 gloo ranks."""
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
