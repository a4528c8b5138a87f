"""The oracle pinned to the reference itself.

oracle/_ref/libref{2,3}d.so hold the reference's own level-set sources (casl_math, utils, hierarchy,
cell/node neighbours, quad_neighbor_nodes_of_node, level_set, interpolation, interpolation_nodes,
semi_lagrangian), compiled unchanged from the reference tree with single-process stand-ins for p4est, PETSc
and MPI (oracle/Makefile, target `ref`). Every check here is bit-for-bit: the restatement in oracle/ and the
product grid against the reference's own construct_neighbors, second_derivatives_central,
reinitialize_*, advect_in_normal_direction, my_p4est_interpolation_nodes_t and
my_p4est_semi_lagrangian_t::advect_from_n_to_np1. They run wherever the reference tree is present (CPU only)
and are skipped elsewhere; tests/golden/*.npz carry the reference's outputs to machines without it.
"""
import numpy as np
import pytest

import casl_p4est_gb300 as G
import oracle as O
import ref as R
from casl_p4est_gb300 import shapes
from grids import brick_2d, brick_2d_odd, brick_3d, brick_3d_odd, circle_2d, flower_3d, phi0_circle_2d, phi0_flower_3d

pytestmark = pytest.mark.skipif(not R.available(), reason="the reference tree is not present on this machine")

DBL_MAX = np.finfo(np.float64).max


def _grids():
    out = []
    f = circle_2d(3, 7)
    out.append(("circle2d_L3-7", f, phi0_circle_2d(f)))
    f = flower_3d(3, 5)
    out.append(("flower3d_L3-5", f, phi0_flower_3d(f)))
    f = brick_2d(1, 5)
    out.append(("brick2d_3x2_L1-5", f, f.sample(shapes.sphere_scaled([0.3, 0.1], 0.6, 0.1, [0.2, 0.3]))))
    f = brick_3d(1, 4)
    out.append(("brick3d_2x1x2_L1-4", f, f.sample(shapes.sphere_scaled([0.7, 0.5, 0.9], 0.3, 0.1, [0.2, 0.3, 0.1]))))
    # trees whose sizes are not powers of two (every division stays a division)
    f = brick_2d_odd(1, 5)
    out.append(("brick2d_odd_L1-5", f, f.sample(shapes.sphere_scaled([0.45, 0.35], 0.2, 0.1, [0.3, 0.2]))))
    f = brick_3d_odd(1, 4)
    out.append(("brick3d_odd_L1-4", f, f.sample(shapes.sphere_scaled([0.5, 0.15, 0.25], 0.1, 0.1, [0.3, 0.1, 0.2]))))
    return out


GRIDS = _grids()


@pytest.fixture(scope="module", params=range(len(GRIDS)), ids=[g[0] for g in GRIDS])
def case(request):
    name, f, phi0 = GRIDS[request.param]
    return f, phi0, R.RefGrid.from_forest(f), O.OracleGrid.from_forest(f)


def test_node_numbering_matches_reference(case):
    f, _, rg, og = case
    rt, rx = rg.nodes()
    ot, ox = og.nodes()
    assert np.array_equal(rt, ot) and np.array_equal(rx.astype(np.int64), ox)
    assert np.array_equal(rg.local_nodes(f.num_leaves), f.local_nodes())
    assert np.array_equal(rg.node_xyz(), f.node_xyz())


def test_neighbours_and_walls_match_reference(case):
    """construct_neighbors (src/my_p4est_node_neighbors.cpp:114-1201) and is_node_*Wall, against the
    restatement and the product's host build."""
    f, _, rg, og = case
    dt = G.qnnn_dtype(f.dim)
    ref = rg.qnnn(dt)
    assert ref.tobytes() == og.qnnn(dt).tobytes()
    assert ref.tobytes() == G.my_p4est_node_neighbors_t(f).get_neighbors().tobytes()
    assert np.array_equal(rg.wall_mask(), og.wall_mask())
    assert np.array_equal(rg.wall_mask(), f.wall_mask())


def test_derivatives_match_reference(case):
    _, phi0, rg, og = case
    assert np.array_equal(rg.second_derivatives(phi0), og.compute_derivatives(phi0))
    assert np.array_equal(rg.first_derivatives(phi0), og.first_derivatives(phi0))


@pytest.mark.parametrize("orders", [(2, 2), (1, 1), (1, 2), (2, 1)])
def test_reinitialize_matches_reference(case, orders):
    _, phi0, rg, og = case
    os_, ot = orders
    a = phi0.copy()
    og.reinitialize(a, os_, ot, iterations=9)
    assert np.array_equal(a, rg.reinitialize(phi0, os_, ot, DBL_MAX, -DBL_MAX, 9))
    a = phi0.copy()
    og.reinitialize(a, os_, ot, limit_high=0.25, limit_low=-0.15, iterations=6)
    assert np.array_equal(a, rg.reinitialize(phi0, os_, ot, 0.25, -0.15, 6))


def test_reinitialize_2nd_order_default_and_mask(case):
    f, phi0, rg, og = case
    a = phi0.copy()
    og.reinitialize(a, 2, 2, iterations=12)
    assert np.array_equal(a, rg.reinitialize_2nd_order(phi0, 12))
    x = f.node_xyz()
    mask = (x[:, 0] < 0.2).astype(np.float64)
    a = phi0.copy()
    og.reinitialize_with_mask(a, mask, 2, 2, iterations=7)
    assert np.array_equal(a, rg.reinitialize_2nd_order_with_mask(phi0, mask, 7))


def test_advect_in_normal_direction_matches_reference(case):
    f, phi0, rg, og = case
    x = f.node_xyz()
    vn = 1.0 + 0.5 * np.sin(3 * x[:, 0])
    vn1 = 0.8 + 0.3 * np.cos(2 * x[:, 1])
    dt = og.advect_cfl_dt(vn)
    a = phi0.copy()
    og.advect_in_normal_direction(vn, a, 0.5 * dt)
    b, r = rg.advect_in_normal_direction(vn, phi0, 0.5 * dt)
    assert np.array_equal(a, b) and r == 0.5 * dt
    a = phi0.copy()
    og.advect_in_normal_direction(vn, a, 0.4 * dt, vn_np1=vn1)
    b, _ = rg.advect_in_normal_direction(vn, phi0, 0.4 * dt, vn_np1=vn1)
    assert np.array_equal(a, b)
    # caller-given second derivatives are in/out: both overwrite them with those of the first stage's result
    dd_o = og.compute_derivatives(phi0)
    dd_r = dd_o.copy()
    a = phi0.copy()
    og.advect_in_normal_direction(vn, a, 0.3 * dt, phi_dd=dd_o)
    b, _ = rg.advect_in_normal_direction(vn, phi0, 0.3 * dt, phi_dd=dd_r)
    assert np.array_equal(a, b) and np.array_equal(dd_o, dd_r)


def test_interpolation_matches_reference(case):
    f, phi0, rg, og = case
    rng = np.random.default_rng(7)
    lo = np.array(f.xyz_min[:f.dim]) - 0.02
    hi = np.array(f.xyz_max[:f.dim]) + 0.02
    pts = np.concatenate([lo + (hi - lo) * rng.random((600, f.dim)), f.node_xyz()[::11]])
    F = np.stack([phi0, np.cos(3 * f.node_xyz()[:, 0])])
    dd = np.stack([og.compute_derivatives(F[k]) for k in range(2)])
    for m in range(5):
        assert np.array_equal(og.interpolate(m, F, pts), rg.interpolate(m, F, pts)), m
        assert np.array_equal(og.interpolate(m, F, pts, Fdd=dd), rg.interpolate(m, F, pts, Fdd=dd)), m


def test_semi_lagrangian_step_matches_reference(case):
    f, phi0, rg, og = case
    x = f.node_xyz()
    v = np.stack([-x[:, 1] + 0.1, x[:, 0]] + ([0.3 * x[:, 0]] if f.dim == 3 else []))
    vxx = np.stack([og.compute_derivatives(v[c]) for c in range(f.dim)])
    dd = og.compute_derivatives(phi0)
    for vm, pm in [(4, 4), (1, 2), (0, 3)]:
        a = og.sl_advect(x, 0.07, v, phi0, vdd=vxx, phi_dd=dd, velo_method=vm, phi_method=pm)
        assert np.array_equal(a, rg.sl_advect(0.07, v, vxx, phi0, dd, vm, pm)), (vm, pm)
    # second derivatives computed by the oracle itself when none are given
    assert np.array_equal(og.sl_advect(x, 0.07, v, phi0), rg.sl_advect(0.07, v, vxx, phi0, dd))


def _neighbour_grids(name):
    """Two more grids on the same brick: the grid at n-1 and the new grid at n+1."""
    if name.startswith("circle2d"):
        return circle_2d(3, 6, center=(0.04, -0.03)), circle_2d(3, 7, center=(0.02, 0.01))
    if name.startswith("flower3d"):
        return flower_3d(3, 4), flower_3d(2, 5)
    if name.startswith("brick2d"):
        return brick_2d(1, 4), brick_2d(2, 5)
    return brick_3d(1, 3), brick_3d(2, 4)


@pytest.mark.parametrize("methods", [(4, 4), (1, 1), (0, 2)])
def test_two_velocity_step_matches_reference(case, methods):
    """advect_from_n_to_np1(dt_nm1, dt_n, vnm1, vxx_nm1, vn, vxx_n, phi_n, phi_xx_n, phi_np1)
    (src/my_p4est_semi_lagrangian.cpp:225-319) across three different grids."""
    f, phi0, rg, og = case
    name = [g[0] for g in GRIDS if g[1] is f][0]
    f_nm1, f_np1 = _neighbour_grids(name)
    r_nm1, r_np1 = R.RefGrid.from_forest(f_nm1), R.RefGrid.from_forest(f_np1)
    o_nm1 = O.OracleGrid.from_forest(f_nm1)
    x, xm = f.node_xyz(), f_nm1.node_xyz()
    vn = np.stack([-x[:, 1] + 0.1, x[:, 0]] + ([0.3 * x[:, 0]] if f.dim == 3 else []))
    vm = np.stack([-0.9 * xm[:, 1], 1.1 * xm[:, 0] - 0.05] + ([0.2 * xm[:, 1]] if f.dim == 3 else []))
    vxx_n = np.stack([og.compute_derivatives(vn[c]) for c in range(f.dim)])
    vxx_m = np.stack([o_nm1.compute_derivatives(vm[c]) for c in range(f.dim)])
    pdd = og.compute_derivatives(phi0)
    vmth, pmth = methods
    ref = r_np1.sl_advect2(rg, r_nm1, 0.04, 0.06, vm, vxx_m, vn, vxx_n, phi0, pdd, vmth, pmth)
    got = og.sl_advect2(o_nm1, f_np1.node_xyz(), 0.04, 0.06, vm, vn, phi0, vnm1_dd=vxx_m, vn_dd=vxx_n, phi_dd=pdd, velo_method=vmth,
                        phi_method=pmth)
    assert np.array_equal(got, ref)
    # second derivatives computed by the oracle itself when none are given
    got = og.sl_advect2(o_nm1, f_np1.node_xyz(), 0.04, 0.06, vm, vn, phi0, velo_method=vmth, phi_method=pmth)
    assert np.array_equal(got, ref)


def test_casl_math_matches_reference():
    """interface_Location, interface_Location_With_Second_Order_Derivative (src/casl_math.cpp:55-97) and
    MINMOD (src/casl_math.h:80-88) on random and edge inputs: |f| < EPS at either end, |c2| < EPS, both
    signs of fb, equal and opposite curvatures."""
    lib = O.load()
    rng = np.random.default_rng(3)
    cases = []
    for _ in range(4000):
        a = rng.uniform(-1, 1)
        b = a + rng.uniform(1e-4, 0.5)
        fa, fb = rng.normal(size=2) * 10.0 ** rng.integers(-6, 1)
        if fa * fb > 0:
            fb = -fb
        cases.append((a, b, fa, fb, rng.normal() * 10.0 ** rng.integers(-14, 2), rng.normal() * 10.0 ** rng.integers(-14, 2)))
    cases += [(0.0, 0.1, 1e-14, -1.0, 1.0, 1.0), (0.0, 0.1, 1.0, -5e-14, 1.0, 2.0), (0.0, 0.1, -0.5, 0.5, 1e-14, 1e-14),
              (0.0, 0.1, -0.5, 0.5, 1.0, -1.0), (0.0, 0.1, 0.5, -0.5, 3.0, 2.0), (-0.2, 0.0, 0.3, -0.1, -4.0, -5.0),
              (0.0, 0.1, -1e-13, 0.2, 0.0, 0.0)]
    for a, b, fa, fb, xa, xb in cases:
        assert lib.ora_interface_location(a, b, fa, fb) == R.interface_location(2, a, b, fa, fb)
        r = R.interface_location_2nd(3, a, b, fa, fb, xa, xb)
        o = lib.ora_interface_location_2nd(a, b, fa, fb, xa, xb)
        assert o == r or (np.isnan(o) and np.isnan(r))
    for a, b in [(1.0, 2.0), (-1.0, -0.5), (1.0, -1.0), (0.0, 3.0), (2.0, 2.0), (-3.0, -3.0)]:
        assert R.minmod(2, a, b) == (0.0 if a * b <= 0 else (a if abs(a) < abs(b) else b))
