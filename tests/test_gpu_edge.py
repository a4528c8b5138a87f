"""Edge cases on the GPU: the smallest complete grids (2^dim leaves: every node on a wall, no regular
node), uniform grids, zero iterations, a field with no interface, a field that is zero at nodes, and
the same cases through the device flattener; FP64 results equal the oracle's bit for bit, mixed results
stay within the band tolerance. A single leaf cannot carry the wall stencils (no cell past the
neighbour): the reference's construct_neighbors fails there and so do the oracle and both flatteners."""
import numpy as np
import pytest

import casl_p4est_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu


def grid(dim, lmin, lmax, shape=None):
    f = G.my_p4est_brick_new([1] * dim, [-1] * dim, [1] * dim)
    if lmax > 0:
        f.refine_levelset(shape or G.shapes.sphere([0.1] * dim, 0.45), lmin, lmax, lip=2.4)
    f.build_nodes()
    return f


CASES = {
    "min_2d": lambda: grid(2, 1, 1),
    "min_3d": lambda: grid(3, 1, 1),
    "uniform_2d": lambda: grid(2, 4, 4),
    "uniform_3d": lambda: grid(3, 3, 3),
    "two_levels_3d": lambda: grid(3, 1, 3),
}


def phis(f):
    x = f.node_xyz()
    r = np.sqrt(np.sum((x - 0.1) ** 2, axis=1))
    return {
        "circle": (r - 0.45) * (1.0 + 0.5 * x[:, 0] ** 2),
        "no_interface": r + 0.3,
        "zeros_at_nodes": np.round(x[:, 0] * 4) / 4 - 0.25,
    }


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("device_build", [False, True])
def test_edge_grids(name, device_build):
    f = CASES[name]()
    og = O.OracleGrid.from_forest(f)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f), device_build=device_build)
    _, dmin, _ = f.dxyz_min()
    for key, phi in phis(f).items():
        for iters in (0, 1, 7):
            want = phi.copy()
            og.reinitialize(want, 2, 2, iterations=iters)
            got = phi.copy()
            ls.reinitialize_2nd_order(got, iters)
            assert np.array_equal(got, want), (key, iters)
            mixed = phi.copy()
            ls.reinitialize_2nd_order(mixed, iters, precision="mixed")
            band = np.abs(want) < 3 * dmin
            if iters == 0:
                assert np.array_equal(mixed, phi)
            elif band.any():
                assert np.max(np.abs(mixed[band] - want[band])) <= 1e-4 * dmin, (key, iters)
        a = phi.copy()
        dt = ls.advect_in_normal_direction(np.ones(len(phi)), a, 0.3 * dmin)
        b = phi.copy()
        og.advect_in_normal_direction(np.ones(len(phi)), b, dt)
        assert np.array_equal(a, b), key


@pytest.mark.parametrize("dim", [2, 3])
def test_single_leaf_is_rejected(dim):
    f = grid(dim, 0, 0)
    with pytest.raises(RuntimeError):
        O.OracleGrid.from_forest(f)
    for device_build in (False, True):
        with pytest.raises(G.LsgError):
            G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f), device_build=device_build)


@pytest.mark.parametrize("name", ["min_2d", "uniform_3d"])
def test_edge_interpolation_and_extension(name):
    f = CASES[name]()
    og = O.OracleGrid.from_forest(f)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    phi = phis(f)["circle"]
    pts = np.ascontiguousarray(np.random.default_rng(3).uniform(-1.2, 1.2, (500, f.dim)))
    interp = G.my_p4est_interpolation_nodes_t(ls)
    for m in range(5):
        assert np.array_equal(interp.interpolate_points(pts, phi, m), og.interpolate(m, phi, pts)), m
    q0 = np.where(phi < 0, 1.0 + f.node_xyz()[:, 0], 0.0)
    for order in (0, 1, 2):
        want = q0.copy()
        og.extend_over_interface_tvd(phi, want, 5, order)
        got = q0.copy()
        ls.extend_Over_Interface_TVD(phi, got, 5, order)
        assert np.array_equal(got, want), order
