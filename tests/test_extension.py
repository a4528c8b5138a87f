"""Extension of a field over the interface (extend_Over_Interface_TVD, src/my_p4est_level_set.cpp:969-1764,
without boundary conditions or initial guesses, one-step extrapolation).

CPU: the oracle's constant / linear / quadratic extensions of a smooth field from the inside of a circle
converge at orders 1 / 2 / 3 in a band of three cells outside it (to the value at the projection on the
interface for the constant extension, to the field itself for the others).
GPU: the FP64 kernels reproduce the oracle bit for bit, with computed or given normals and with a mask."""
import numpy as np
import pytest

import casl_p4est_gb300 as G
import oracle as O

from grids import brick_2d, brick_3d, circle_2d, flower_3d


def sphere_grid(dim, lmax):
    f = G.my_p4est_brick_new([1] * dim, [-1] * dim, [1] * dim)
    f.refine_levelset(G.shapes.sphere([0.0] * dim, 0.5), 2, lmax, lip=2.4)
    f.build_nodes()
    return f


def field(x):
    v = np.cos(x[:, 0]) + np.sin(1.3 * x[:, 1])
    return v + 0.5 * x[:, 2] if x.shape[1] == 3 else v


@pytest.mark.parametrize("order,rate", [(0, 0.9), (1, 1.8), (2, 2.6)])
def test_oracle_extension_converges(order, rate):
    errs = []
    for lmax in (6, 7, 8):
        f = sphere_grid(2, lmax)
        og = O.OracleGrid.from_forest(f)
        x = f.node_xyz()
        r = np.sqrt(np.sum(x ** 2, axis=1))
        phi = r - 0.5
        q = np.where(phi < 0, field(x), 0.0)
        og.extend_over_interface_tvd(phi, q, iterations=60, order=order, nthreads=8)
        want = field(0.5 * x / np.maximum(r, 1e-12)[:, None]) if order == 0 else field(x)
        h = 2.0 / (1 << lmax)
        band = (phi > 0) & (phi < 3 * h)
        errs.append(np.max(np.abs(q[band] - want[band])))
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert np.all(rates > rate), (errs, rates)


def test_oracle_extension_leaves_the_inside_alone():
    f = sphere_grid(2, 6)
    og = O.OracleGrid.from_forest(f)
    x = f.node_xyz()
    phi = np.sqrt(np.sum(x ** 2, axis=1)) - 0.5
    q0 = np.where(phi < 0, field(x), 0.0)
    for order in (0, 1, 2):
        q = q0.copy()
        og.extend_over_interface_tvd(phi, q, iterations=10, order=order)
        inside = phi < -1e-9
        assert np.array_equal(q[inside], q0[inside])


GRIDS = {
    "circle2d": lambda: circle_2d(3, 8),
    "brick2d": lambda: brick_2d(1, 6),
    "flower3d": lambda: flower_3d(3, 6),
    "brick3d": lambda: brick_3d(1, 5),
}


def case(f):
    x = f.node_xyz()
    phi = (np.sqrt(np.sum((x - 0.07) ** 2, axis=1)) - 0.45) * (1.0 + 0.3 * x[:, 0])
    q = np.where(phi < 0, field(x), 0.0)
    return x, phi, q


@pytest.mark.gpu
@pytest.mark.parametrize("order", [0, 1, 2])
@pytest.mark.parametrize("name", sorted(GRIDS))
def test_gpu_extension_bitwise(name, order):
    f = GRIDS[name]()
    og = O.OracleGrid.from_forest(f)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    x, phi, q0 = case(f)
    want = q0.copy()
    og.extend_over_interface_tvd(phi, want, iterations=12, order=order, nthreads=8)
    got = q0.copy()
    ls.extend_Over_Interface_TVD(phi, got, 12, order)
    assert np.array_equal(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["circle2d", "flower3d"])
def test_gpu_extension_normals_mask_and_bands(name):
    f = GRIDS[name]()
    og = O.OracleGrid.from_forest(f)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    x, phi, q0 = case(f)
    nrm = np.ascontiguousarray(og.compute_normals(phi)[::-1]) * 0.9  # any field of directions
    mask = phi + 0.05 * np.sin(7 * x[:, 0])
    for order in (1, 2):
        want = q0.copy()
        og.extend_over_interface_tvd(phi, want, 9, order, band_use=-0.1, band_extend=0.2, normals=nrm, mask=mask)
        got = q0.copy()
        ls.extend_Over_Interface_TVD(phi, got, 9, order, band_use=-0.1, band_extend=0.2, normal=nrm, mask=mask)
        assert np.array_equal(got, want), order


@pytest.mark.gpu
def test_gpu_extension_device_entry_and_errors():
    import torch
    f = GRIDS["flower3d"]()
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    x, phi, q0 = case(f)
    host = q0.copy()
    ls.extend_Over_Interface_TVD(phi, host, 7, 2)
    lib = G._lib.load()
    ls.set_stream(torch.cuda.current_stream().cuda_stream)
    tphi = torch.from_numpy(phi).cuda()
    tq = torch.from_numpy(q0).cuda()
    G._lib.check(lib.lsg_extend_over_interface_tvd_device(ls._h, tphi.data_ptr(), tq.data_ptr(), 7, 2, -G.level_set.DBL_MAX,
                                                          G.level_set.DBL_MAX, None, None))
    torch.cuda.synchronize()
    assert np.array_equal(tq.cpu().numpy(), host)
    with pytest.raises(ValueError):
        ls.extend_Over_Interface_TVD(phi, q0.copy(), 7, 3)
    assert lib.lsg_extend_over_interface_tvd(ls._h, G._lib.dptr(phi), G._lib.dptr(q0.copy()), 7, 3, 0.0, 1.0, None, None) != 0
