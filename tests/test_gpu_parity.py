"""CUDA path against the CPU oracle, through the C ABI.

FP64: the kernels evaluate the reference's expressions in the same order with no contracted
multiply-adds, so the results must be bit-identical to the oracle (tolerance 0). The north-star
tolerance for the FP64 GPU path is 1e-12*max|phi|; the tests hold it to exact equality.
Mixed: FP32 stencil/RK with the FP64 subcell step; band L-infinity error against the FP64 path
<= 1e-4 * dx_min (spec target), interface sign pattern identical.
"""
import numpy as np
import pytest

import casl_p4est_gb300 as G
import oracle as O

from grids import (band_error, brick_2d, brick_2d_odd, brick_3d, brick_3d_odd, circle_2d, flower_3d, phi0_circle_2d,
                   phi0_flower_3d)

pytestmark = pytest.mark.gpu

GRIDS = {
    "circle2d": (lambda: circle_2d(3, 8), phi0_circle_2d),
    "brick2d": (lambda: brick_2d(1, 7), lambda f: f.sample(G.shapes.sphere_scaled([0.3, 0.1], 0.6, 0.2, [0.5, 0.5]))),
    "flower3d": (lambda: flower_3d(3, 6), phi0_flower_3d),
    "brick3d": (lambda: brick_3d(1, 5), lambda f: f.sample(G.shapes.sphere_scaled([0.7, 0.5, 0.9], 0.3, 0.1, [1, 0.5, 1]))),
    # tree sizes that are not powers of two: the FP64 kernels divide instead of multiplying by exact reciprocals
    "brick2d_odd": (lambda: brick_2d_odd(1, 7), lambda f: f.sample(G.shapes.sphere_scaled([0.45, 0.35], 0.2, 0.1, [0.3, 0.2]))),
    "brick3d_odd": (lambda: brick_3d_odd(1, 5), lambda f: f.sample(G.shapes.sphere_scaled([0.5, 0.15, 0.25], 0.1, 0.1, [0.3, 0.1, 0.2]))),
}


@pytest.fixture(scope="module", params=sorted(GRIDS))
def case(request):
    build, phi0 = GRIDS[request.param]
    f = build()
    ngbd = G.my_p4est_node_neighbors_t(f)
    ngbd.init_neighbors()
    ls = G.my_p4est_level_set_t(ngbd)
    og = O.OracleGrid.from_forest(f)
    return request.param, f, ls, og, phi0(f)


def test_second_derivatives_bitwise(case):
    name, f, ls, og, phi = case
    got = ls.compute_derivatives(phi)
    ref = og.compute_derivatives(phi)
    assert np.array_equal(got, ref), np.max(np.abs(got - ref))


@pytest.mark.parametrize("orders", [(2, 2), (1, 1), (1, 2), (2, 1)])
def test_reinit_fp64_bitwise(case, orders):
    name, f, ls, og, phi0 = case
    iters = 6
    a = phi0.copy()
    b = phi0.copy()
    ls.reinitialize_within_range_of_phi_0(a, orders[0], orders[1], G.DBL_MAX, -G.DBL_MAX, iters, precision="fp64")
    og.reinitialize(b, orders[0], orders[1], iterations=iters)
    assert np.array_equal(a, b), (name, orders, np.max(np.abs(a - b)))


def test_reinit_fp64_limits_bitwise(case):
    name, f, ls, og, phi0 = case
    lim = 0.1 * float(np.max(np.abs(phi0)))
    a = phi0.copy()
    b = phi0.copy()
    ls.reinitialize_2nd_order(a, 5, lim, precision="fp64")
    og.reinitialize(b, 2, 2, lim, -lim, iterations=5)
    assert np.array_equal(a, b)
    a = phi0.copy()
    b = phi0.copy()
    ls.reinitialize_2nd_order_above_threshold(a, -0.5 * lim, 5, precision="fp64")
    og.reinitialize(b, 2, 2, np.finfo(np.float64).max, -0.5 * lim, iterations=5)
    assert np.array_equal(a, b)


def test_advect_fp64_bitwise(case):
    name, f, ls, og, phi0 = case
    xyz = f.node_xyz()
    vn = 1.0 + 0.5 * np.sin(3 * xyz[:, 0]) * np.cos(2 * xyz[:, 1])
    dt_gpu = ls.advect_in_normal_direction(lambda x: 1.0 + 0.5 * np.sin(3 * x[:, 0]) * np.cos(2 * x[:, 1]), phi0.copy())
    dt = og.advect_cfl_dt(vn)
    assert dt_gpu == dt
    a = phi0.copy()
    b = phi0.copy()
    ls.advect_in_normal_direction(vn, a, dt, precision="fp64")
    og.advect_in_normal_direction(vn, b, dt)
    assert np.array_equal(a, b)
    # two velocities + caller-supplied second derivatives (overwritten as the reference does)
    vn1 = 0.5 * vn
    dd_a = ls.compute_derivatives(phi0)
    dd_b = dd_a.copy()
    a = phi0.copy()
    b = phi0.copy()
    ls.advect_in_normal_direction(vn, a, dt, phi_xx=dd_a, vn_np1=vn1, precision="fp64")
    og.advect_in_normal_direction(vn, b, dt, vn_np1=vn1, phi_dd=dd_b)
    assert np.array_equal(a, b)
    assert np.array_equal(dd_a, dd_b)


def test_fp64_node_order_fallback_bitwise(case, monkeypatch):
    """The FP64 sweeps on the node-ordered tables (their layout when the copy sorted by stencil pattern does not
    fit in memory) give the same bits as the sorted ones and the oracle."""
    name, f, ls, og, phi0 = case
    monkeypatch.setenv("LSGPU_FP64_NODE_ORDER", "1")
    ngbd = G.my_p4est_node_neighbors_t(f)
    ngbd.init_neighbors()
    ls_node = G.my_p4est_level_set_t(ngbd)
    a = phi0.copy()
    b = phi0.copy()
    ls_node.reinitialize_2nd_order(a, 4, precision="fp64")
    og.reinitialize(b, 2, 2, iterations=4)
    assert np.array_equal(a, b)
    xyz = f.node_xyz()
    vn = 1.0 + 0.5 * np.sin(3 * xyz[:, 0]) * np.cos(2 * xyz[:, 1])
    dt = og.advect_cfl_dt(vn)
    dd_a = ls_node.compute_derivatives(phi0)
    dd_b = dd_a.copy()
    a = phi0.copy()
    b = phi0.copy()
    ls_node.advect_in_normal_direction(vn, a, dt, phi_xx=dd_a, vn_np1=0.5 * vn, precision="fp64")
    og.advect_in_normal_direction(vn, b, dt, vn_np1=0.5 * vn, phi_dd=dd_b)
    assert np.array_equal(a, b)
    assert np.array_equal(dd_a, dd_b)


def test_mixed_band_error_vs_fp64(case):
    name, f, ls, og, phi0 = case
    a = phi0.copy()
    b = phi0.copy()
    ls.reinitialize_2nd_order(a, 20, precision="fp64")
    ls.reinitialize_2nd_order(b, 20, precision="mixed")
    lvl = f.leaves()[1].max()
    _, dmin, _ = f.dxyz_min(int(lvl))
    err = band_error(b, a, 3 * dmin)
    assert err <= 1e-4 * dmin, (name, err, dmin)
    assert np.all(np.sign(a[np.abs(a) > 1e-9]) == np.sign(b[np.abs(a) > 1e-9]))


def test_mixed_advect_close_to_fp64(case):
    name, f, ls, og, phi0 = case
    xyz = f.node_xyz()
    vn = 1.0 + 0.5 * np.sin(3 * xyz[:, 0])
    dt = og.advect_cfl_dt(vn)
    a = phi0.copy()
    b = phi0.copy()
    ls.advect_in_normal_direction(vn, a, dt, precision="fp64")
    ls.advect_in_normal_direction(vn, b, dt, precision="mixed")
    lvl = f.leaves()[1].max()
    _, dmin, _ = f.dxyz_min(int(lvl))
    assert band_error(b, a, 3 * dmin) <= 1e-4 * dmin


def test_mixed_advect_two_velocities_both_signs(case):
    """The mixed normal advection runs on the reinitialisation's stage kernels (upwinding by the sign of vn):
    speeds of both signs and a second velocity for the second RK stage, several steps, against the FP64 path."""
    name, f, ls, og, phi0 = case
    xyz = f.node_xyz()
    vn = 0.8 * np.sin(4 * xyz[:, 0] + 1.0) * np.cos(3 * xyz[:, 1])
    vn1 = vn + 0.3 * np.cos(2 * xyz[:, 0])
    dt = 0.5 * og.advect_cfl_dt(np.maximum(np.abs(vn), np.abs(vn1)))
    a = phi0.copy()
    b = phi0.copy()
    for _ in range(3):
        ls.advect_in_normal_direction(vn, a, dt, vn_np1=vn1, precision="fp64")
        ls.advect_in_normal_direction(vn, b, dt, vn_np1=vn1, precision="mixed")
    lvl = f.leaves()[1].max()
    _, dmin, _ = f.dxyz_min(int(lvl))
    assert band_error(b, a, 3 * dmin) <= 1e-4 * dmin, (name, band_error(b, a, 3 * dmin) / dmin)


def test_mixed_advect_launch_shapes_agree(case):
    """The advection stage gives the same bits for every launch shape and stream schedule (Jacobi update)."""
    name, f, ls, og, phi0 = case
    xyz = f.node_xyz()
    vn = 1.0 - 0.7 * np.cos(2 * xyz[:, 1])
    dt = 0.5 * og.advect_cfl_dt(vn)
    cfg = ls.stage_config
    out = []
    try:
        for shape in ({"threads_per_block": 256, "uniform_blocks": 0, "regular_blocks": 0, "uniform_depth": 1, "streams": 2, "priority": 2},
                      {"threads_per_block": 64, "uniform_blocks": 152, "regular_blocks": 304, "uniform_depth": 2, "streams": 1},
                      {"threads_per_block": 128, "uniform_blocks": 0, "regular_blocks": 0, "uniform_depth": 3, "streams": 2, "priority": 0},
                      {"threads_per_block": 128, "uniform_blocks": 1216, "regular_blocks": 0, "uniform_depth": 5, "streams": 2}):
            ls.stage_config = shape
            p = phi0.copy()
            ls.advect_in_normal_direction(vn, p, dt, precision="mixed")
            out.append(p)
    finally:
        ls.stage_config = cfg
    assert all(np.array_equal(out[0], o) for o in out[1:])


def test_device_resident_matches_host(case):
    torch = pytest.importorskip("torch")
    name, f, ls, og, phi0 = case
    a = phi0.copy()
    ls.reinitialize_2nd_order(a, 4, precision="fp64")
    t = torch.from_numpy(phi0.copy()).cuda()
    torch.cuda.synchronize()
    ls.reinitialize_2nd_order(t, 4, precision="fp64")
    torch.cuda.synchronize()
    assert np.array_equal(t.cpu().numpy(), a)


def test_deterministic(case):
    name, f, ls, og, phi0 = case
    a = phi0.copy()
    b = phi0.copy()
    ls.reinitialize_2nd_order(a, 5, precision="mixed")
    ls.reinitialize_2nd_order(b, 5, precision="mixed")
    assert np.array_equal(a, b)


def test_errors_are_reported():
    f = circle_2d(2, 5)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    phi = phi0_circle_2d(f)
    with pytest.raises(ValueError):
        ls.reinitialize_within_range_of_phi_0(phi, 3, 2, 1.0, -1.0, 5)
    with pytest.raises(G.LsgInvalidArgument):
        ls.reinitialize_within_range_of_phi_0(phi, 2, 2, -1.0, 1.0, 5)
    with pytest.raises(ValueError):
        ls.reinitialize_2nd_order(phi[:-1], 5)
    with pytest.raises(G.LsgInvalidArgument):
        ls.reinitialize_2nd_order(phi, -1)


def test_band_linf_device_matches_numpy():
    """FP64 band check on the device: same value and count as numpy; NaN reported."""
    import torch
    f = flower_3d(3, 6)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    ls.set_stream(torch.cuda.current_stream().cuda_stream)
    ref = phi0_flower_3d(f)
    rng = np.random.default_rng(5)
    a = ref + rng.normal(0, 1e-6, ref.size)
    _, dmin, _ = f.dxyz_min()
    band = 3 * dmin
    val, cnt = ls.band_linf(torch.from_numpy(a).cuda(), torch.from_numpy(ref).cuda(), band)
    m = np.abs(ref) < band
    assert cnt == int(m.sum()) and val == float(np.max(np.abs(a[m] - ref[m])))
    a[np.flatnonzero(m)[0]] = np.nan
    val, _ = ls.band_linf(torch.from_numpy(a).cuda(), torch.from_numpy(ref).cuda(), band)
    assert np.isnan(val)


@pytest.mark.parametrize("shape", [(256, 0, 0, 1, 512, 2), (128, 912, 304, 2, 512, 2), (64, 152, 0, 2, 512, 2), (256, 0, 0, 3, 512, 2),
                                   (256, 4, 0, 3, 0, 2), (32, 2, 304, 3, 128, 2), (128, 608, 0, 3, 2048, 2), (256, 0, 0, 4, 512, 2),
                                   (256, 4, 0, 4, 1024, 2), (64, 3, 0, 4, 4096, 2), (128, 0, 304, 4, 4, 2), (256, 0, 0, 1, 512, 1),
                                   (128, 912, 304, 2, 512, 1), (256, 4, 0, 3, 256, 1), (128, 1216, 608, 1, 512, 2, 1),
                                   (256, 0, 0, 3, 512, 2, 0), (128, 1216, 608, 1, 512, 2, 0), (128, 912, 0, 1, 512, 2, 3),
                                   (256, 0, 304, 2, 512, 2, 4), (64, 3, 0, 4, 256, 2, 3), (128, 1216, 0, 5, 512, 2),
                                   (256, 0, 0, 5, 512, 1), (64, 152, 304, 5, 512, 2, 0)])
@pytest.mark.parametrize("grid", ["flower3d", "circle2d"])
def test_mixed_result_independent_of_launch_shape(shape, grid):
    """The mixed stages are Jacobi updates: threads per block, persistent grids, the uniform kernel's
    pipeline (depth 3 / 4: bulk-copied tiles two / three ahead; a grid of 2 to 4 CTAs makes every CTA cycle
    through its stages many times; depth 5: registers capped), the phi window around each tile (halo 0 to 4096 nodes), one or two
    streams per stage and their priorities change no bit of the result."""
    f = flower_3d(3, 6) if grid == "flower3d" else circle_2d(3, 9)
    phi0 = phi0_flower_3d(f) if grid == "flower3d" else phi0_circle_2d(f)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f), precision="mixed")
    ref = phi0.copy()
    ls.reinitialize_2nd_order(ref, 7)
    tpb, ub, rb, depth, halo, streams = shape[:6]
    priority = shape[6] if len(shape) > 6 else 2
    ls.stage_config = {"threads_per_block": tpb, "uniform_blocks": ub, "regular_blocks": rb, "uniform_depth": depth,
                       "window_halo": halo, "streams": streams, "priority": priority}
    assert ls.stage_config["window_halo"] == halo and ls.stage_config["streams"] == streams
    assert ls.stage_config["priority"] == priority
    got = phi0.copy()
    ls.reinitialize_2nd_order(got, 7)
    assert np.array_equal(got, ref)
