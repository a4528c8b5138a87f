"""The regrid path on the device: node numbering (my_p4est_nodes_new), node coordinates and refinement
tags (splitting_criteria_tag_t, the device side of update_p4est's regrid) computed on the GPU equal the
host's exactly, and update_p4est run with device fields gives the host run's grid and values bit for
bit, for the analytic (vortex) and node-sampled velocity forms."""
import math

import numpy as np
import pytest

import casl_p4est_gb300 as G
from grids import brick_2d, brick_3d, circle_2d, flower_3d

pytestmark = pytest.mark.gpu

GRIDS = {
    "circle2d": lambda: circle_2d(3, 8),
    "brick2d": lambda: brick_2d(1, 6),
    "flower3d": lambda: flower_3d(3, 6),
    "brick3d": lambda: brick_3d(1, 5),
}


@pytest.mark.parametrize("name", sorted(GRIDS))
def test_device_node_numbering_and_coordinates(name):
    import torch
    host = GRIDS[name]()
    dev = host.copy()
    dev.build_nodes(device=True)
    assert dev.num_nodes == host.num_nodes
    assert np.array_equal(dev.local_nodes(), host.local_nodes())
    th, xh = host.nodes()
    td, xd = dev.nodes()
    assert np.array_equal(th, td) and np.array_equal(xh, xd)
    assert np.array_equal(dev.node_xyz_device().cpu().numpy(), host.node_xyz())
    torch.cuda.synchronize()


@pytest.mark.parametrize("name", sorted(GRIDS))
def test_device_tags_match_host(name):
    import torch
    a = GRIDS[name]()
    b = a.copy()
    b.build_nodes(device=True)
    x = a.node_xyz()
    phi = np.sqrt(np.sum((x - 0.13) ** 2, axis=1)) - 0.4
    lv = (2, 7) if a.dim == 2 else (1, 5)
    ca = a.refine_and_coarsen(*lv, phi, lip=1.2)
    cb = b.refine_and_coarsen(*lv, torch.from_numpy(phi).cuda(), lip=1.2)
    assert ca == cb
    ta, la, xa = a.leaves()
    tb, lb, xb = b.leaves()
    assert np.array_equal(ta, tb) and np.array_equal(la, lb) and np.array_equal(xa, xb)


def transport_setup():
    lmin, lmax = 4, 7
    sphere = G.shapes.sphere([0.35, 0.35, 0.35], 0.15)
    f = G.my_p4est_brick_new([1, 1, 1], [0, 0, 0], [1, 1, 1])
    f.refine_levelset(sphere, lmin, lmax, lip=1.2)
    f.build_nodes()
    return f, f.sample(sphere), (lmin, lmax, 1.2), 1.0 / (1 << lmax)


def test_update_p4est_device_matches_host_vortex():
    import torch
    f, phi, split, dt = transport_setup()
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    v = G.VortexVelocity(math.cos(math.pi * 0.5 * dt / 3.0))
    sl_h = G.my_p4est_semi_lagrangian_t(f.copy(), ls, splitting=split)
    want = sl_h.update_p4est(v, 4 * dt, phi)
    sl_d = G.my_p4est_semi_lagrangian_t(f.copy(), ls, splitting=split)
    got = sl_d.update_p4est(v, 4 * dt, torch.from_numpy(phi).cuda())
    torch.cuda.synchronize()
    assert sl_h.iterations == sl_d.iterations and sl_h.iterations > 1
    assert np.array_equal(sl_h.forest_np1.leaves()[2], sl_d.forest_np1.leaves()[2])
    assert np.array_equal(got.cpu().numpy(), want)
    # a level set built on the device from the device copy of the new grid
    ls_h = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(sl_h.forest_np1))
    ls_d = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(sl_d.forest_np1), device_build=True)
    a = want.copy()
    ls_h.reinitialize_2nd_order(a, 5, precision="mixed")
    ls_d.set_stream(torch.cuda.current_stream().cuda_stream)
    ls_d.reinitialize_2nd_order(got, 5, precision="mixed")
    torch.cuda.synchronize()
    assert np.array_equal(got.cpu().numpy(), a)


def test_update_p4est_device_matches_host_node_velocity():
    import torch
    f, phi, split, dt = transport_setup()
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    x = f.node_xyz()
    v = np.ascontiguousarray(np.stack([-(x[:, 1] - 0.5), x[:, 0] - 0.5, 0.2 * np.ones(len(x))]))
    sl_h = G.my_p4est_semi_lagrangian_t(f.copy(), ls, splitting=split)
    want = sl_h.update_p4est(v, 3 * dt, phi)
    sl_d = G.my_p4est_semi_lagrangian_t(f.copy(), ls, splitting=split)
    got = sl_d.update_p4est(torch.from_numpy(v).cuda(), 3 * dt, torch.from_numpy(phi).cuda())
    torch.cuda.synchronize()
    assert sl_h.iterations == sl_d.iterations
    assert np.array_equal(got.cpu().numpy(), want)
