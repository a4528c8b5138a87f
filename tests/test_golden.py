"""Reference fixtures (tests/golden, made by tests/golden/make_golden.py from the reference's own code compiled
from its sources): the grid rebuilt leaf by leaf, the restatement's FP64 outputs reproduced bit for bit on the
CPU, and the CUDA path's FP64 outputs equal to the same numbers on the GPU (nothing from the reference tree
or the oracle at run time). Also the known answer of the quadratic interface root (src/casl_math.cpp:67-97):
exact for a quadratic sampled at the cell ends."""
import glob
import os

import numpy as np
import pytest

import casl_p4est_gb300 as G
import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(p for p in glob.glob(os.path.join(HERE, "golden", "*.npz")) if "config1" not in p)
CONFIG1 = os.path.join(HERE, "golden", "circle2d_L4-9_config1.npz")


def grid_from(z, prefix=""):
    dim = int(z["dim"])
    f = G.my_p4est_brick_new(list(z["n_xyz"][:dim]), list(z["xyz_min"][:dim]), list(z["xyz_max"][:dim]))
    f.set_leaves(z[prefix + "tree"], z[prefix + "level"], z[prefix + "lxyz"])
    f.build_nodes()
    return f


def load(path):
    z = dict(np.load(path))
    return grid_from(z), z


@pytest.fixture(params=FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def golden(request):
    return load(request.param)


def test_fixtures_present():
    assert len(FIXTURES) >= 3 and os.path.exists(CONFIG1)


def test_grid_rebuilds_from_leaves(golden):
    f, z = golden
    assert np.array_equal(f.node_xyz(), z["node_xyz"])


def test_oracle_reproduces_fixtures(golden):
    f, z = golden
    og = O.OracleGrid.from_forest(f)
    phi0 = z["phi0"]
    assert np.array_equal(og.compute_derivatives(phi0), z["dd"])
    for key, (os_, ot) in {"reinit_22": (2, 2), "reinit_11": (1, 1), "reinit_12": (1, 2), "reinit_21": (2, 1)}.items():
        p = phi0.copy()
        og.reinitialize(p, os_, ot, iterations=8)
        assert np.array_equal(p, z[key]), key
    p = phi0.copy()
    og.reinitialize(p, 2, 2, limit_high=0.3, limit_low=-0.2, iterations=8)
    assert np.array_equal(p, z["reinit_22_limited"])
    adv = z["reinit_22"].copy()
    og.advect_in_normal_direction(z["vn"], adv, float(z["advect_dt"]))
    assert np.array_equal(adv, z["advect"])
    for m in range(5):
        assert np.array_equal(og.interpolate(m, z["reinit_22"], z["points"]), z[f"interp_{m}"]), m
    assert np.array_equal(og.sl_advect(z["node_xyz"], 0.05, z["velocity"], z["reinit_22"]), z["sl"])
    if "vnm1" in z:
        o_nm1 = O.OracleGrid.from_forest(grid_from(z, "nm1_"))
        x_np1 = grid_from(z, "np1_").node_xyz()
        for vm in (4, 1):
            got = og.sl_advect2(o_nm1, x_np1, 0.04, 0.05, z["vnm1"], z["velocity"], z["reinit_22"], velo_method=vm, phi_method=vm)
            assert np.array_equal(got, z[f"sl2_{vm}"]), vm


def test_oracle_reproduces_configuration_1():
    """2D, levels 4-9, 20 iterations of reinitialize_2nd_order: the reference's result and error."""
    z = dict(np.load(CONFIG1))
    f = grid_from(z)
    og = O.OracleGrid.from_forest(f)
    p = z["phi0"].copy()
    og.reinitialize(p, 2, 2, iterations=20)
    assert np.array_equal(p, z["reinit_20"])
    x = z["node_xyz"]
    band = np.abs(p) < 3 * float(z["dx_min"])
    err = float(np.max(np.abs(p[band] - (np.sqrt(x[band, 0] ** 2 + x[band, 1] ** 2) - 0.5))))
    assert err == float(z["band_error"]) and err < 1e-3 * float(z["dx_min"])


@pytest.mark.parametrize("c", [(0.7, 0.3, -0.005), (-1.3, 0.2, 0.01), (0.0, 1.0, -0.0125), (40.0, 3.0, 0.01)])
def test_interface_location_exact_on_quadratics(c):
    """f(x) = c2 (x - xm)^2 + c1 (x - xm) + c0 on [a, b] with the exact second derivative at both ends."""
    c2, c1, c0 = c
    a, b = -0.05, 0.05
    xm = 0.5 * (a + b)
    f = lambda x: c2 * (x - xm) ** 2 + c1 * (x - xm) + c0
    lib = O.load()
    got = lib.ora_interface_location_2nd(a, b, f(a), f(b), 2 * c2, 2 * c2)
    roots = np.roots([c2, c1, c0]) + xm if c2 != 0 else np.array([-c0 / c1 + xm])
    root = roots[(roots >= a) & (roots <= b)]
    assert len(root) == 1 and abs(got - root[0]) < 1e-15
    # linear fall-back
    assert abs(lib.ora_interface_location(a, b, -1.0, 3.0) - (a + 0.25 * (b - a))) < 1e-16


@pytest.mark.gpu
def test_cuda_path_matches_fixtures(golden):
    f, z = golden
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    phi0 = z["phi0"]
    assert np.array_equal(ls.compute_derivatives(phi0), z["dd"])
    for key, fn in {"reinit_22": ls.reinitialize_2nd_order, "reinit_11": ls.reinitialize_1st_order,
                    "reinit_12": ls.reinitialize_2nd_order_time_1st_order_space,
                    "reinit_21": ls.reinitialize_1st_order_time_2nd_order_space}.items():
        p = phi0.copy()
        fn(p, 8)
        assert np.array_equal(p, z[key]), key
    p = phi0.copy()
    ls.reinitialize_within_range_of_phi_0(p, 2, 2, 0.3, -0.2, 8)
    assert np.array_equal(p, z["reinit_22_limited"])
    adv = z["reinit_22"].copy()
    dt = ls.advect_in_normal_direction(lambda xyz: 1.0 + 0.5 * np.sin(3 * xyz[:, 0]), adv.copy())
    assert 0.4 * dt == float(z["advect_dt"])
    ls.advect_in_normal_direction(z["vn"], adv, float(z["advect_dt"]))
    assert np.array_equal(adv, z["advect"])
    interp = G.my_p4est_interpolation_nodes_t(ls)
    for m in range(5):
        assert np.array_equal(interp.interpolate_points(z["points"], z["reinit_22"], m), z[f"interp_{m}"]), m
    sl = G.my_p4est_semi_lagrangian_t(f, ls)
    assert np.array_equal(sl.advect_from_n_to_np1(0.05, z["velocity"], z["reinit_22"]), z["sl"])
    if "vnm1" in z:
        f_nm1, f_np1 = grid_from(z, "nm1_"), grid_from(z, "np1_")
        ls_nm1 = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f_nm1))
        sl2 = G.my_p4est_semi_lagrangian_t(f_np1, ls, ls_nm1=ls_nm1)
        for vm in (4, 1):
            sl2.set_velo_interpolation(vm)
            sl2.set_phi_interpolation(vm)
            got = sl2.advect_from_n_to_np1(0.04, 0.05, z["vnm1"], z["velocity"], z["reinit_22"])
            assert np.array_equal(got, z[f"sl2_{vm}"]), vm


@pytest.mark.gpu
def test_cuda_path_matches_configuration_1():
    """The 2D configuration on the GPU: FP64 equal to the reference's numbers; mixed within 1e-4 dx_min of
    them in |phi| < 3 dx_min; the error against r - 0.5 reported for both."""
    z = dict(np.load(CONFIG1))
    f = grid_from(z)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    dmin = float(z["dx_min"])
    p = z["phi0"].copy()
    ls.reinitialize_2nd_order(p, 20, precision="fp64")
    assert np.array_equal(p, z["reinit_20"])
    m = z["phi0"].copy()
    ls.reinitialize_2nd_order(m, 20, precision="mixed")
    band = np.abs(p) < 3 * dmin
    assert float(np.max(np.abs(m[band] - p[band]))) <= 1e-4 * dmin
    x = z["node_xyz"]
    exact = np.sqrt(x[:, 0] ** 2 + x[:, 1] ** 2) - 0.5
    err64 = float(np.max(np.abs(p[band] - exact[band])))
    err32 = float(np.max(np.abs(m[band] - exact[band])))
    assert err64 == float(z["band_error"])
    assert abs(err32 - err64) <= 1e-4 * dmin
    print(f"configuration 1: {f.num_nodes} nodes, error |phi-(r-0.5)| in the band: FP64 {err64:.3e} ({err64 / dmin:.2e} dx_min), "
          f"mixed {err32:.3e}")
