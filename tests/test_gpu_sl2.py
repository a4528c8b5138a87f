"""The two-velocity second-order semi-Lagrangian step on the GPU against the oracle, through the C ABI.

advect_from_n_to_np1(dt_nm1, dt_n, vnm1, vxx_nm1, vn, vxx_n, phi_n, phi_xx_n, phi_np1)
(src/my_p4est_semi_lagrangian.cpp:225-319) and update_p4est(vnm1, vn, dt_nm1, dt_n, phi, ...) (:779-939):
three different grids (n-1, n, n+1) on one brick; v_n interpolated quadratically at the new nodes, v_n and
v_nm1 at the midpoint on their own grids, phi_n at the departure point. The kernels evaluate the reference's
expressions in the same order with no contracted multiply-adds, so the results are bit-identical to the
oracle (which tests/test_ref_pin.py holds bit-identical to the reference itself)."""
import numpy as np
import pytest

import casl_p4est_gb300 as G
import oracle as O

from grids import brick_2d, brick_3d, circle_2d, flower_3d

pytestmark = pytest.mark.gpu

# (grid n, grid n-1, grid n+1) per case
GRIDS = {
    "circle2d": (lambda: circle_2d(3, 8), lambda: circle_2d(3, 7, center=(0.04, -0.03)), lambda: circle_2d(3, 7, center=(0.05, -0.03))),
    "flower3d": (lambda: flower_3d(3, 6), lambda: flower_3d(3, 5), lambda: flower_3d(2, 6)),
    "brick2d": (lambda: brick_2d(1, 6), lambda: brick_2d(1, 5), lambda: brick_2d(2, 6)),
    "brick3d": (lambda: brick_3d(1, 5), lambda: brick_3d(1, 4), lambda: brick_3d(2, 5)),
}


def velocity(x, dim, s, shift):
    v = [-s * x[:, 1] + shift, s * x[:, 0]] + ([0.3 * s * x[:, 0] - 0.1 * x[:, 1]] if dim == 3 else [])
    return np.ascontiguousarray(np.stack(v))


@pytest.fixture(scope="module", params=sorted(GRIDS))
def case(request):
    import torch
    fn, fm, f1 = (g() for g in GRIDS[request.param])
    stream = torch.cuda.current_stream().cuda_stream
    ls_n = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(fn))
    ls_m = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(fm))
    ls_n.set_stream(stream)
    ls_m.set_stream(stream)
    x, xm = fn.node_xyz(), fm.node_xyz()
    r = np.sqrt(np.sum((x - 0.1) ** 2, axis=1))
    phi = np.ascontiguousarray((r - 0.5) * (0.2 + x[:, 0] ** 2))
    return dict(fn=fn, fm=fm, f1=f1, ls_n=ls_n, ls_m=ls_m, og=O.OracleGrid.from_forest(fn), om=O.OracleGrid.from_forest(fm),
                vn=velocity(x, fn.dim, 1.0, 0.1), vm=velocity(xm, fn.dim, 0.8, -0.05), phi=phi)


@pytest.mark.parametrize("methods", [(4, 4), (1, 2), (0, 3), (2, 0)])
def test_two_velocity_step_bitwise(case, methods):
    c = case
    vm_, pm = methods
    _, dmin, _ = c["fn"].dxyz_min()
    dt_nm1, dt_n = 1.5 * dmin, 2.0 * dmin
    sl = G.my_p4est_semi_lagrangian_t(c["f1"], c["ls_n"], ls_nm1=c["ls_m"])
    sl.set_velo_interpolation(vm_)
    sl.set_phi_interpolation(pm)
    x1 = c["f1"].node_xyz()
    ref = c["og"].sl_advect2(c["om"], x1, dt_nm1, dt_n, c["vm"], c["vn"], c["phi"], velo_method=vm_, phi_method=pm)
    got = sl.advect_from_n_to_np1(dt_nm1, dt_n, c["vm"], c["vn"], c["phi"])
    assert np.array_equal(got, ref), np.max(np.abs(got - ref))
    # caller-given second derivatives (the reference's vxx_nm1 / vxx_n / phi_xx_n arguments)
    d = c["fn"].dim
    vxx_n = np.stack([c["og"].compute_derivatives(c["vn"][k]) for k in range(d)])
    vxx_m = np.stack([c["om"].compute_derivatives(c["vm"][k]) for k in range(d)])
    pdd = c["og"].compute_derivatives(c["phi"])
    got2 = sl.advect_from_n_to_np1(dt_nm1, dt_n, c["vm"], c["vn"], c["phi"], vxx_nm1=vxx_m, vxx_n=vxx_n, phi_xx_n=pdd)
    assert np.array_equal(got2, ref)


def test_two_velocity_step_device_matches_host(case):
    import torch
    c = case
    _, dmin, _ = c["fn"].dxyz_min()
    sl = G.my_p4est_semi_lagrangian_t(c["f1"], c["ls_n"], ls_nm1=c["ls_m"])
    host = sl.advect_from_n_to_np1(dmin, 2.0 * dmin, c["vm"], c["vn"], c["phi"])
    dev = sl.advect_from_n_to_np1(dmin, 2.0 * dmin, torch.from_numpy(c["vm"]).cuda(), torch.from_numpy(c["vn"]).cuda(),
                                  torch.from_numpy(c["phi"]).cuda())
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy(), host)


def test_two_velocity_step_equals_one_velocity_for_steady_flow(case):
    """With v_nm1 = v_n on the same grid and dt_nm1 = dt_n, v* = v_n(x*) (1.5 v - 0.5 v), so the step differs
    from the one-velocity RK2 step only through the quadratic first round: with velo_method quadratic both
    are the same step."""
    c = case
    _, dmin, _ = c["fn"].dxyz_min()
    sl = G.my_p4est_semi_lagrangian_t(c["f1"], c["ls_n"], ls_nm1=c["ls_n"])
    sl.set_velo_interpolation(G.interpolation.quadratic)
    two = sl.advect_from_n_to_np1(dmin, dmin, c["vn"], c["vn"], c["phi"])
    one = sl.advect_from_n_to_np1(dmin, c["vn"], c["phi"])
    assert np.max(np.abs(two - one)) <= 1e-12 * np.max(np.abs(c["phi"]))


def test_two_velocity_needs_grid_nm1(case):
    c = case
    sl = G.my_p4est_semi_lagrangian_t(c["f1"], c["ls_n"])
    with pytest.raises(ValueError):
        sl.advect_from_n_to_np1(0.01, 0.01, c["vm"], c["vn"], c["phi"])


@pytest.mark.parametrize("device", [False, True])
def test_two_velocity_update_p4est_matches_oracle_loop(device):
    """update_p4est(vnm1, vn, dt_nm1, dt_n, phi): the two-velocity step repeated while the new grid is refined
    and coarsened from the advected values, against the same loop driven by the oracle."""
    import torch
    sphere = G.shapes.sphere([0.35, 0.35, 0.35], 0.15)
    f = G.my_p4est_brick_new([1, 1, 1], [0, 0, 0], [1, 1, 1])
    f.refine_levelset(sphere, 2, 6, lip=1.2)
    f.build_nodes()
    fm = G.my_p4est_brick_new([1, 1, 1], [0, 0, 0], [1, 1, 1])
    fm.refine_levelset(G.shapes.sphere([0.34, 0.36, 0.35], 0.15), 2, 6, lip=1.2)
    fm.build_nodes()
    phi = f.sample(sphere)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    lm = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(fm))
    stream = torch.cuda.current_stream().cuda_stream
    ls.set_stream(stream)
    lm.set_stream(stream)
    og, om = O.OracleGrid.from_forest(f), O.OracleGrid.from_forest(fm)
    vn = np.ascontiguousarray(O.vortex(3, f.node_xyz(), 1.0))
    vm = np.ascontiguousarray(O.vortex(3, fm.node_xyz(), 0.9))
    dt_nm1, dt_n = 3.0 / 64, 4.0 / 64
    sl = G.my_p4est_semi_lagrangian_t(f.copy(), ls, splitting=(2, 6, 1.2), ls_nm1=lm)
    if device:
        got = sl.update_p4est(torch.from_numpy(vm).cuda(), torch.from_numpy(vn).cuda(), dt_nm1, dt_n, torch.from_numpy(phi).cuda())
        got = got.cpu().numpy()
    else:
        got = sl.update_p4est(vm, vn, dt_nm1, dt_n, phi)
    g = f.copy()
    while True:
        ref = og.sl_advect2(om, g.node_xyz(), dt_nm1, dt_n, vm, vn, phi)
        if not g.refine_and_coarsen(2, 6, ref, lip=1.2):
            break
        g.build_nodes()
    assert sl.iterations >= 2
    assert np.array_equal(sl.forest_np1.leaves()[2], g.leaves()[2])
    assert np.array_equal(got, ref)
