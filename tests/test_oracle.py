"""Pins the CPU oracle with analytic known answers and the reference examples' convergence behaviour
(the reference has no value-level golden vectors for this path; SURVEY of its tests: the examples
print L-infinity errors and orders only)."""
import numpy as np
import pytest

import casl_p4est_gb300 as G
from casl_p4est_gb300 import shapes
import oracle as O

from grids import band_error, brick_2d, brick_3d, circle_2d, flower_3d


def quadratic(xyz):
    x = xyz[:, 0]
    y = xyz[:, 1]
    if xyz.shape[1] == 2:
        return 0.7 * x * x - 0.3 * y * y + 0.45 * x * y + 0.2 * x - 0.1 * y + 0.05, np.array([1.4, -0.6])
    z = xyz[:, 2]
    return (0.7 * x * x - 0.3 * y * y + 0.25 * z * z + 0.45 * x * y - 0.35 * y * z + 0.15 * x * z + 0.2 * x - 0.1 * y + 0.3 * z,
            np.array([1.4, -0.6, 0.5]))


@pytest.mark.parametrize("builder", [lambda: circle_2d(2, 7), lambda: brick_2d(1, 6), lambda: flower_3d(2, 5),
                                     lambda: brick_3d(1, 5)])
def test_laplace_exact_on_quadratics(builder):
    """laplace + correct_naive_second_derivatives is exact for quadratics on uniform, hanging and
    wall stencils (including the cross terms)."""
    f = builder()
    og = O.OracleGrid.from_forest(f)
    v, dd = quadratic(f.node_xyz())
    out = og.compute_derivatives(v)
    for a in range(f.dim):
        np.testing.assert_allclose(out[a], dd[a], rtol=0, atol=2e-8)


def reinit_error(lmax, dim=2, iters=50):
    """examples/reinitialization/main_2d.cpp:103-116, 234, 254-262: circle r=0.5 times
    (1 + 0.5 sin5x cos4y), reinitialize_2nd_order, error max|phi - phi_exact| for |phi| < 3 diag_min."""
    f = G.my_p4est_brick_new([1, 1], [-1, -1], [1, 1])
    f.refine_levelset(shapes.sphere([0, 0], 0.5), 0, lmax, lip=1.2)
    f.build_nodes()
    xyz = f.node_xyz()
    exact = 0.5 - np.sqrt((xyz ** 2).sum(1))
    phi = exact * (1 + 0.5 * np.sin(5 * xyz[:, 0]) * np.cos(4 * xyz[:, 1]))
    og = O.OracleGrid.from_forest(f)
    og.reinitialize(phi, iterations=iters)
    _, _, diag = f.dxyz_min(lmax)
    return band_error(phi, exact, 3 * diag)


def test_reinit_second_order_convergence():
    errs = [reinit_error(l) for l in (6, 7, 8)]
    orders = [np.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert errs[2] < 1e-3
    assert min(orders) > 1.5, (errs, orders)


def test_reinit_keeps_a_signed_distance():
    f = circle_2d(3, 7)
    xyz = f.node_xyz()
    sdf = np.sqrt((xyz ** 2).sum(1)) - 0.5
    phi = sdf.copy()
    og = O.OracleGrid.from_forest(f)
    og.reinitialize(phi, iterations=20)
    _, dmin, diag = f.dxyz_min(7)
    assert band_error(phi, sdf, 3 * diag) < 0.05 * dmin


def test_reinit_orders_and_limits():
    """All four (space, pseudo-time) orders run and a limit leaves far nodes untouched."""
    f = circle_2d(3, 6)
    from grids import phi0_circle_2d
    base = phi0_circle_2d(f)
    og = O.OracleGrid.from_forest(f)
    for os_, ot in ((1, 1), (1, 2), (2, 1), (2, 2)):
        phi = base.copy()
        og.reinitialize(phi, os_, ot, iterations=5)
        assert np.all(np.isfinite(phi))
        assert np.array_equal(np.sign(phi[np.abs(base) > 1e-3]), np.sign(base[np.abs(base) > 1e-3]))
    phi = base.copy()
    og.reinitialize(phi, 2, 2, 0.05, -0.05, iterations=5)
    far = np.abs(base) > 0.06
    assert np.array_equal(phi[far], base[far])


def test_advect_normal_moves_circle_outward():
    """advect_in_normal_direction with vn = 1 on a signed distance shrinks phi by ~dt (circle grows)."""
    f = circle_2d(3, 7)
    xyz = f.node_xyz()
    phi = np.sqrt((xyz ** 2).sum(1)) - 0.5
    og = O.OracleGrid.from_forest(f)
    vn = np.ones(og.N)
    dt = og.advect_cfl_dt(vn)
    _, dmin, _ = f.dxyz_min(7)
    assert abs(dt - 0.8 * dmin) < 1e-15
    p = phi.copy()
    og.advect_in_normal_direction(vn, p, dt)
    band = np.abs(phi) < 3 * dmin
    np.testing.assert_allclose(p[band], phi[band] - dt, atol=0.05 * dt)
