"""Device flattener (level sets created with device_build=True): the node-neighbour tables built on the
GPU give exactly the results of the host-built tables for every operation that reads them (FP64
reinitialisation in all orders, normal advection with its CFL step, second and first derivatives, both
extensions, the mixed path), on single- and multi-tree bricks in 2D and 3D, and the mixed tables have
the same sizes (regular, uniform, irregular, extended set, geometry classes, corrections)."""
import numpy as np
import pytest

import casl_p4est_gb300 as G
from grids import brick_2d, brick_3d, circle_2d, flower_3d, phi0_circle_2d, phi0_flower_3d

pytestmark = pytest.mark.gpu

GRIDS = {
    "circle2d": lambda: circle_2d(3, 8),
    "brick2d": lambda: brick_2d(1, 6),
    "flower3d": lambda: flower_3d(3, 6),
    "brick3d": lambda: brick_3d(1, 5),
}


def phi_of(f):
    x = f.node_xyz()
    return (np.sqrt(np.sum((x - 0.07) ** 2, axis=1)) - 0.45) * (1.0 + 0.3 * x[:, 0])


@pytest.fixture(params=sorted(GRIDS), scope="module")
def pair(request):
    f = GRIDS[request.param]()
    ngbd = G.my_p4est_node_neighbors_t(f)
    return f, G.my_p4est_level_set_t(ngbd), G.my_p4est_level_set_t(ngbd, device_build=True)


def test_fp64_operations_identical(pair):
    f, host, dev = pair
    phi = phi_of(f)
    assert np.array_equal(host.compute_derivatives(phi), dev.compute_derivatives(phi))
    assert np.array_equal(host.first_derivatives_central(phi), dev.first_derivatives_central(phi))
    for os_, ot in ((1, 1), (1, 2), (2, 1), (2, 2)):
        a, b = phi.copy(), phi.copy()
        host.reinitialize_within_range_of_phi_0(a, os_, ot, 0.3, -0.2, 6)
        dev.reinitialize_within_range_of_phi_0(b, os_, ot, 0.3, -0.2, 6)
        assert np.array_equal(a, b), (os_, ot)
    a, b = phi.copy(), phi.copy()
    vn = lambda xyz: 1.0 + 0.5 * np.sin(3 * xyz[:, 0])
    assert host.advect_in_normal_direction(vn, a) == dev.advect_in_normal_direction(vn, b)
    assert np.array_equal(a, b)
    x = f.node_xyz()
    q0 = np.where(phi < 0, np.cos(x[:, 0]) + x[:, 1], 0.0)
    a, b = q0.copy(), q0.copy()
    host.extend_Over_Interface_TVD(phi, a, 5, 2)
    dev.extend_Over_Interface_TVD(phi, b, 5, 2)
    assert np.array_equal(a, b)
    assert np.array_equal(host.extend_from_interface_to_whole_domain_TVD(phi, np.cos(x[:, 0]), iterations=4),
                          dev.extend_from_interface_to_whole_domain_TVD(phi, np.cos(x[:, 0]), iterations=4))


def test_mixed_path_identical(pair):
    f, host, dev = pair
    phi = phi0_flower_3d(f) if f.dim == 3 else phi0_circle_2d(f)
    a, b = phi.copy(), phi.copy()
    host.reinitialize_2nd_order(a, 9, precision="mixed")
    dev.reinitialize_2nd_order(b, 9, precision="mixed")
    assert np.array_equal(a, b)
    assert host.table_stats() == dev.table_stats()
    a, b = phi.copy(), phi.copy()
    host.advect_in_normal_direction(np.full(len(phi), 0.7), a, 0.01, precision="mixed")
    dev.advect_in_normal_direction(np.full(len(phi), 0.7), b, 0.01, precision="mixed")
    assert np.array_equal(a, b)
