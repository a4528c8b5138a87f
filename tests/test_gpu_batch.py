"""Batched reinitialisation: many grids in one set of launches (optionally one CUDA graph) give, grid by
grid, exactly the result of reinitialising each grid alone with the mixed path (the stages are Jacobi
updates and every node's arithmetic is the same in the union), including per-grid iteration counts,
and regardless of the launch shape chosen by the autotuner."""
import numpy as np
import pytest

import casl_p4est_gb300 as G
from casl_p4est_gb300 import shapes

pytestmark = pytest.mark.gpu


def ellipse_grid(seed, lmax):
    rng = np.random.default_rng(seed)
    k = int(rng.integers(1, 5))
    items = [(rng.uniform(-0.6, 0.6), rng.uniform(-0.6, 0.6), rng.uniform(0.05, 0.4), rng.uniform(0.05, 0.4),
              rng.uniform(0, np.pi)) for _ in range(k)]
    f = G.my_p4est_brick_new([1, 1], [-1, -1], [1, 1])
    f.refine_levelset(shapes.ellipses(items), 3, lmax, lip=1.2)
    f.build_nodes()
    phi = f.sample(shapes.ellipses(items, scale=(0.1, (rng.uniform(-0.5, 0.5), rng.uniform(-0.5, 0.5)), 1.0)))
    return f, phi


@pytest.fixture(scope="module")
def batch2d():
    grids = [ellipse_grid(s, l) for s, l in [(1, 6), (2, 8), (3, 7), (4, 9), (5, 6), (6, 8)]]
    forests = [g[0] for g in grids]
    b = G.my_p4est_level_set_batch_t(forests)
    return grids, b


def alone(f, phi, iters):
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f), precision="mixed")
    out = phi.copy()
    ls.reinitialize_2nd_order(out, iters)
    return out


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_equals_each_grid_alone(batch2d, use_graph):
    grids, b = batch2d
    phi = b.concat([g[1] for g in grids])
    b.reinitialize_2nd_order(phi, 12, use_graph=use_graph)
    for k, (f, p0) in enumerate(grids):
        assert np.array_equal(b.split(phi)[k], alone(f, p0, 12)), k


def test_per_grid_iteration_counts_and_graph_replay(batch2d):
    grids, b = batch2d
    its = [0, 3, 12, 7, 3, 1]
    want = [alone(f, p0, n) for (f, p0), n in zip(grids, its)]
    for _ in range(2):  # capture, then replay
        phi = b.concat([g[1] for g in grids])
        b.reinitialize_2nd_order(phi, its, use_graph=True)
        for k in range(len(grids)):
            assert np.array_equal(b.split(phi)[k], want[k]), k


def test_autotuned_shape_keeps_results(batch2d):
    grids, b = batch2d
    phi0 = b.concat([g[1] for g in grids])
    cfg = b.autotune(phi0, trials=2)
    assert cfg["threads_per_block"] in (128, 256) and cfg["uniform_blocks"] >= 0 and cfg["regular_blocks"] >= 0
    assert b.stage_config == cfg
    phi = phi0.copy()
    b.reinitialize_2nd_order(phi, 6)
    b.stage_config = {"threads_per_block": 64, "uniform_blocks": 152, "regular_blocks": 304,
                      "uniform_depth": 3 if cfg["uniform_depth"] != 3 else 1}
    phi2 = phi0.copy()
    b.reinitialize_2nd_order(phi2, 6)
    assert np.array_equal(phi, phi2)


def test_batch_3d_and_device_tensors():
    import torch
    from grids import flower_3d, phi0_flower_3d
    fs = [flower_3d(2, 5), flower_3d(3, 6)]
    phis = [phi0_flower_3d(f) for f in fs]
    b = G.my_p4est_level_set_batch_t(fs)
    b.set_stream(torch.cuda.current_stream().cuda_stream)
    t = torch.from_numpy(b.concat(phis)).cuda()
    b.reinitialize_2nd_order(t, [5, 9])
    torch.cuda.synchronize()
    got = b.split(t.cpu().numpy())
    assert np.array_equal(got[0], alone(fs[0], phis[0], 5))
    assert np.array_equal(got[1], alone(fs[1], phis[1], 9))


def test_batch_rejects_mixed_tree_sizes():
    a = G.my_p4est_brick_new([1, 1], [-1, -1], [1, 1])
    a.refine_levelset(shapes.sphere([0, 0], 0.5), 2, 5)
    a.build_nodes()
    c = G.my_p4est_brick_new([1, 1], [0, 0], [1, 1])
    c.refine_levelset(shapes.sphere([0.5, 0.5], 0.2), 2, 5)
    c.build_nodes()
    with pytest.raises(G.LsgInvalidArgument):
        G.my_p4est_level_set_batch_t([a, c])


@pytest.mark.parametrize("dim", [2, 3])
def test_device_built_batch_equals_host_built(batch2d, dim):
    """Tables built on the GPU (each grid's, concatenated there, then the union's mixed tables) give the
    host-built batch's results bit for bit, with per-grid iteration counts; the grids' nodes are
    numbered on the host for one half of them and on the device for the other."""
    if dim == 2:
        grids = batch2d[0]
        forests = [g[0] for g in grids]
        phis = [g[1] for g in grids]
    else:
        from grids import flower_3d, phi0_flower_3d
        forests = [flower_3d(2, 5), flower_3d(3, 6), flower_3d(2, 4)]
        phis = [phi0_flower_3d(f) for f in forests]
    copies = [f.copy() for f in forests]
    for k, f in enumerate(copies):
        if k % 2:
            f.build_nodes(device=True)
    host = G.my_p4est_level_set_batch_t(forests)
    dev = G.my_p4est_level_set_batch_t(copies, device_build=True)
    assert np.array_equal(dev.offsets, host.offsets)
    its = [int(i) for i in np.arange(len(forests)) % 4 + 3]
    a = host.concat(phis)
    b = dev.concat(phis)
    host.reinitialize_2nd_order(a, its)
    dev.reinitialize_2nd_order(b, its)
    assert np.array_equal(a, b)


def test_every_grid_of_a_batch_within_the_fp64_band_tolerance():
    """Each grid of a batch (sizes from 4k to about 400k nodes, refined in a wide band as the batch workload
    is) against its own FP64 reinitialisation: band L-infinity within 1e-4 dx_min in |phi| < 3 dx_min, and the
    interface zero crossings along the cut grid edges within the same bound."""
    import torch
    rng = np.random.default_rng(17)
    grids = []
    for lmax in (6, 8, 9, 11):
        items = [(rng.uniform(-0.6, 0.6), rng.uniform(-0.6, 0.6), rng.uniform(0.05, 0.4), rng.uniform(0.05, 0.4),
                  rng.uniform(0, np.pi)) for _ in range(int(rng.integers(1, 9)))]
        scale = (0.1, (rng.uniform(-0.5, 0.5), rng.uniform(-0.5, 0.5)), rng.uniform(0.5, 1.5))
        f = G.my_p4est_brick_new([1, 1], [-1, -1], [1, 1])
        f.refine_levelset(shapes.ellipses(items), 6, lmax, lip=14.4)
        f.build_nodes()
        grids.append((f, f.sample(shapes.ellipses(items, scale=scale)), lmax))
    assert grids[-1][0].num_nodes > 200000
    b = G.my_p4est_level_set_batch_t([g[0] for g in grids])
    phi = b.concat([g[1] for g in grids])
    b.reinitialize_2nd_order(phi, 30)
    for k, (f, p0, lmax) in enumerate(grids):
        ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
        ref = p0.copy()
        ls.reinitialize_2nd_order(ref, 30, precision="fp64")
        got = b.split(phi)[k]
        dmin = 2.0 / (1 << lmax)
        band = np.abs(ref) < 3 * dmin
        assert float(np.max(np.abs(got[band] - ref[band]))) <= 1e-4 * dmin, k
        loc, edges, mismatched = ls.interface_location_error(torch.from_numpy(got).cuda(), torch.from_numpy(ref).cuda())
        assert edges > 0 and mismatched == 0 and loc <= 1e-4 * dmin, (k, loc, edges, mismatched)
