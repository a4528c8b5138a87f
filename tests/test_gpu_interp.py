"""Node interpolation, point location and the semi-Lagrangian step: CUDA path against the oracle,
through the C ABI.

The kernels evaluate the reference's expressions in the same order with no contracted multiply-adds,
so interpolated values, located leaves and the node-sampled-velocity semi-Lagrangian step are
bit-identical to the oracle (tolerance 0). The analytic-velocity step evaluates sin() on the device,
which may differ from the host's by an ulp, so it is held to the FP64 path's tolerance
1e-12 * max|phi|."""
import numpy as np
import pytest

import casl_p4est_gb300 as G
from casl_p4est_gb300 import _lib as L
import oracle as O

from grids import brick_2d, brick_3d, circle_2d, flower_3d

pytestmark = pytest.mark.gpu

GRIDS = {
    "circle2d": lambda: circle_2d(3, 8),
    "flower3d": lambda: flower_3d(3, 6),
    "brick2d": lambda: brick_2d(1, 6),
    "brick3d": lambda: brick_3d(1, 5),
}
# grids at n+1 for the semi-Lagrangian step (other refinements of the same bricks)
NEXT = {
    "circle2d": lambda: circle_2d(3, 7, center=(0.05, -0.03)),
    "flower3d": lambda: flower_3d(3, 5),
    "brick2d": lambda: brick_2d(1, 5),
    "brick3d": lambda: brick_3d(1, 4),
}


@pytest.fixture(scope="module", params=sorted(GRIDS))
def case(request):
    import torch
    f = GRIDS[request.param]()
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    ls.set_stream(torch.cuda.current_stream().cuda_stream)
    og = O.OracleGrid.from_forest(f)
    return request.param, f, ls, og


def test_points(f, n=6000, seed=0):
    """random points (some outside the domain), the grid's nodes, and points on cell faces."""
    rng = np.random.default_rng(seed)
    lo = np.array(f.xyz_min[:f.dim])
    hi = np.array(f.xyz_max[:f.dim])
    span = hi - lo
    rnd = lo + rng.uniform(-0.05, 1.05, (n, f.dim)) * span
    nodes = f.node_xyz()
    face = nodes[rng.integers(0, len(nodes), n // 2)].copy()
    face[:, 0] += rng.uniform(0, 1e-3, len(face)) * span[0]  # on faces normal to y (and z)
    return np.ascontiguousarray(np.concatenate([rnd, nodes, face]))


test_points.__test__ = False


def fields(f):
    x = f.node_xyz()
    r = np.sqrt(np.sum((x - 0.1) ** 2, axis=1))
    F0 = (r - 0.5) * (0.2 + x[:, 0] ** 2)
    F1 = np.sin(3 * x[:, 0]) * np.cos(2 * x[:, 1])
    return np.ascontiguousarray(np.stack([F0, F1]))


def test_locate_bitwise(case):
    name, f, ls, og = case
    import torch
    pts = test_points(f)
    pts_d = torch.from_numpy(pts).cuda()
    got = torch.empty(len(pts), dtype=torch.int32, device="cuda")
    L.check(L.load().lsg_locate_points_device(ls.handle, pts_d.data_ptr(), len(pts), got.data_ptr()))
    torch.cuda.synchronize()
    assert np.array_equal(got.cpu().numpy(), og.locate(pts))


@pytest.mark.parametrize("method", [0, 1, 2, 3, 4])
def test_interpolate_bitwise(case, method):
    name, f, ls, og = case
    interp = G.my_p4est_interpolation_nodes_t(ls)
    pts = test_points(f, seed=method)
    F = fields(f)
    got = interp.interpolate_points(pts, F, method)
    ref = og.interpolate(method, F, pts)
    assert np.array_equal(got, ref), np.nanmax(np.abs(got - ref))
    # caller-supplied second derivatives (the precomputed-derivative form of set_input)
    dd = np.stack([og.compute_derivatives(F[k]) for k in range(len(F))])
    got2 = interp.interpolate_points(pts, F, method, Fdd=dd)
    assert np.array_equal(got2, ref)


def test_interpolate_device_matches_host(case):
    import torch
    name, f, ls, og = case
    interp = G.my_p4est_interpolation_nodes_t(ls)
    pts = test_points(f, seed=7)
    F = fields(f)
    out = torch.empty(2 * len(pts), dtype=torch.float64, device="cuda")
    pts_d = torch.from_numpy(pts.ravel()).cuda()
    F_d = torch.from_numpy(F.ravel()).cuda()
    interp.interpolate_device(pts_d, F_d, 2, 4, out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy().reshape(2, -1), og.interpolate(4, F, pts))


def test_add_point_interface(case):
    name, f, ls, og = case
    interp = G.my_p4est_interpolation_nodes_t(ls)
    pts = test_points(f, n=200, seed=3)[:300]
    F = fields(f)[0]
    for i in reversed(range(len(pts))):
        interp.add_point(i, pts[i])
    interp.set_input(F, G.interpolation.quadratic_non_oscillatory_continuous_v2)
    out = interp.interpolate()
    assert np.array_equal(out, og.interpolate(4, F, pts))


@pytest.mark.parametrize("methods", [(4, 4), (1, 2), (0, 3), (2, 0)])
def test_semi_lagrangian_bitwise(case, methods):
    name, f, ls, og = case
    vm, pm = methods
    x = f.node_xyz()
    v = np.ascontiguousarray(O.vortex(f.dim, x, 1.0))
    phi = fields(f)[0]
    _, dmin, _ = f.dxyz_min()
    dt = 2.0 * dmin
    f1 = NEXT[name]()
    xyz1 = f1.node_xyz()
    sl = G.my_p4est_semi_lagrangian_t(f1, ls)
    sl.set_velo_interpolation(vm)
    sl.set_phi_interpolation(pm)
    got = sl.advect_from_n_to_np1(dt, v, phi)
    ref = og.sl_advect(xyz1, dt, v, phi, velo_method=vm, phi_method=pm)
    assert np.array_equal(got, ref), np.max(np.abs(got - ref))
    vdd = np.stack([og.compute_derivatives(v[k]) for k in range(f.dim)])
    pdd = og.compute_derivatives(phi)
    got2 = sl.advect_from_n_to_np1(dt, v, phi, vxx=vdd, phi_xx_n=pdd)
    assert np.array_equal(got2, ref)


def test_semi_lagrangian_vortex(case):
    name, f, ls, og = case
    x = f.node_xyz()
    phi = fields(f)[0]
    _, dmin, _ = f.dxyz_min()
    sl = G.my_p4est_semi_lagrangian_t(f, ls)
    for scale in (1.0, -0.5):
        got = sl.advect_from_n_to_np1(3.0 * dmin, G.VortexVelocity(scale), phi)
        ref = og.sl_advect_vortex(x, 3.0 * dmin, scale, phi)
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(phi))


def test_semi_lagrangian_callback_velocity(case):
    """The CF overload with a host callback: departure points formed on the host with the same
    velocity the oracle uses (its single vortex), so the result is the oracle's bit for bit."""
    name, f, ls, og = case
    x = f.node_xyz()
    phi = fields(f)[0]
    _, dmin, _ = f.dxyz_min()
    sl = G.my_p4est_semi_lagrangian_t(f, ls)
    got = sl.advect_from_n_to_np1(3.0 * dmin, lambda p: O.vortex(f.dim, p, -0.5), phi)
    assert np.array_equal(got, og.sl_advect_vortex(x, 3.0 * dmin, -0.5, phi))
    with pytest.raises(ZeroDivisionError):
        sl.advect_from_n_to_np1(dmin, lambda p: 1 / 0, phi)


def test_bad_method_is_rejected(case):
    name, f, ls, og = case
    interp = G.my_p4est_interpolation_nodes_t(ls)
    with pytest.raises(G.LsgInvalidArgument):
        L.check(L.load().lsg_interpolate_nodes(ls.handle, L.dptr(np.zeros(f.dim)), 1, L.dptr(fields(f)[0].copy()), 1, None, 7,
                                               L.dptr(np.zeros(1))))
    with pytest.raises(ValueError):
        interp.set_input(fields(f)[0], 9)


@pytest.mark.parametrize("velocity", ["nodes", "vortex"])
def test_update_p4est_matches_oracle_loop(velocity):
    """update_p4est: repeated advect + refine_and_coarsen until the grid settles, against the same loop
    driven by the oracle's semi-Lagrangian step (same host regrid)."""
    f = G.my_p4est_brick_new([1, 1, 1], [0, 0, 0], [1, 1, 1])
    sphere = G.shapes.sphere([0.35, 0.35, 0.35], 0.15)
    f.refine_levelset(sphere, 2, 6, lip=1.2)
    f.build_nodes()
    phi = f.sample(sphere)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    og = O.OracleGrid.from_forest(f)
    dt = 4.0 / 64
    x = f.node_xyz()
    v = G.VortexVelocity(1.0) if velocity == "vortex" else np.ascontiguousarray(O.vortex(3, x, 1.0))
    sl = G.my_p4est_semi_lagrangian_t(f.copy(), ls, splitting=(2, 6, 1.2))
    got = sl.update_p4est(v, dt, phi)
    # oracle-driven loop
    g = f.copy()
    while True:
        xyz = g.node_xyz()
        if velocity == "vortex":
            ref = og.sl_advect_vortex(xyz, dt, 1.0, phi)
        else:
            ref = og.sl_advect(xyz, dt, v, phi)
        if not g.refine_and_coarsen(2, 6, ref, lip=1.2):
            break
        g.build_nodes()
    assert sl.iterations >= 2
    assert np.array_equal(sl.forest_np1.leaves()[2], g.leaves()[2])
    if velocity == "vortex":
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(phi))
    else:
        assert np.array_equal(got, ref)
