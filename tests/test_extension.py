"""Extension of fields across the interface.

extend_Over_Interface_TVD (src/my_p4est_level_set.cpp:969-1764, without boundary conditions or initial
guesses, one-step extrapolation): on the CPU the oracle's constant / linear / quadratic extensions of a
smooth field from the inside of a circle converge at orders 1 / 2 / 3 in a band of three cells outside it
(to the value at the projection on the interface for the constant extension, to the field itself for the
others); on the GPU the FP64 kernels reproduce the oracle bit for bit, with computed or given normals and
with a mask.

extend_from_interface_to_whole_domain_TVD (src/my_p4est_level_set.cpp:3181-3767): the oracle's extension
of a field's interface values converges at third order in a band of three cells on both sides of a
circle (to the value at the projection on the interface); on the GPU the kernels reproduce the oracle bit
for bit for every interpolation method, several fields and a given gradient, and within 1e-12 relative
with a mask (whose smoothstep goes through pow, rounded differently by the device library)."""
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


def test_oracle_whole_domain_extension_converges():
    errs = []
    for lmax in (6, 7, 8):
        f = sphere_grid(2, lmax)
        og = O.OracleGrid.from_forest(f)
        x = f.node_xyz()
        r = np.sqrt(np.sum(x ** 2, axis=1))
        phi = r - 0.5
        q = og.extend_from_interface_to_whole_domain_tvd(phi, field(x), iterations=40, nthreads=8)
        want = field(0.5 * x / np.maximum(r, 1e-12)[:, None])
        band = np.abs(phi) < 3 * (2.0 / (1 << lmax))
        errs.append(np.max(np.abs(q[band] - want[band])))
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert np.all(rates > 2.5), (errs, rates)


def test_oracle_whole_domain_extension_keeps_constants():
    f = sphere_grid(3, 5)
    og = O.OracleGrid.from_forest(f)
    x = f.node_xyz()
    phi = np.sqrt(np.sum(x ** 2, axis=1)) - 0.5
    q = og.extend_from_interface_to_whole_domain_tvd(phi, np.full(len(phi), 0.75), iterations=60, nthreads=8)
    near = np.abs(phi) < 0.1  # 1.6 cells: filled from zero by the march, to round-off in 60 steps
    assert np.max(np.abs(q[near] - 0.75)) < 1e-12
    assert np.all(q[np.abs(phi) < 0.05] == 0.75)  # started at qi, constant interface values


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(GRIDS))
def test_gpu_whole_domain_extension_bitwise(name):
    f = GRIDS[name]()
    og = O.OracleGrid.from_forest(f)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    x, phi, _ = case(f)
    qi = field(x)
    want = og.extend_from_interface_to_whole_domain_tvd(phi, qi, iterations=9, nthreads=8)
    assert np.array_equal(ls.extend_from_interface_to_whole_domain_TVD(phi, qi, iterations=9), want)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["circle2d", "flower3d"])
def test_gpu_whole_domain_extension_options(name):
    f = GRIDS[name]()
    og = O.OracleGrid.from_forest(f)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    x, phi, _ = case(f)
    qi = np.stack([field(x), np.sin(2 * x[:, 0]) * x[:, 1]])
    grad = og.first_derivatives(phi) * 1.1  # any gradient field
    for method in range(5):
        ls.set_interpolation_on_interface(method)
        got = ls.extend_from_interface_to_whole_domain_TVD(phi, qi, iterations=6, grad_phi_in=grad)
        for k in range(2):
            want = og.extend_from_interface_to_whole_domain_tvd(phi, qi[k], iterations=6, grad_phi=grad, method=method, nthreads=8)
            assert np.array_equal(got[k], want), (method, k)
    ls.set_interpolation_on_interface(4)
    mask = 0.3 * x[:, 0] + 0.05
    want = og.extend_from_interface_to_whole_domain_tvd(phi, qi[1], iterations=6, mask=mask, band_zero=1.0, band_smooth=8.0,
                                                        nthreads=8)
    got = ls.extend_from_interface_to_whole_domain_TVD(phi, qi[1], iterations=6, mask=mask, band_zero=1.0, band_smooth=8.0)
    assert np.max(np.abs(got - want)) <= 1e-12 * np.max(np.abs(want))
    with pytest.raises(G.LsgInvalidArgument):
        ls.extend_from_interface_to_whole_domain_TVD(phi, qi, iterations=2, mask=mask)


@pytest.mark.gpu
def test_gpu_whole_domain_extension_device_tensors():
    import torch
    f = GRIDS["brick3d"]()
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    x, phi, _ = case(f)
    qi = field(x)
    host = ls.extend_from_interface_to_whole_domain_TVD(phi, qi, iterations=5)
    ls.set_stream(torch.cuda.current_stream().cuda_stream)
    tqi = torch.from_numpy(qi).cuda()
    tq = ls.extend_from_interface_to_whole_domain_TVD(torch.from_numpy(phi).cuda(), tqi, iterations=5)
    torch.cuda.synchronize()
    assert np.array_equal(tq.cpu().numpy(), host)
    with pytest.raises(G.LsgInvalidArgument):  # output over the input
        ls.extend_from_interface_to_whole_domain_TVD(torch.from_numpy(phi).cuda(), tqi, q=tqi, iterations=1)


def iface_value(n, d, dist):
    """interface values of the cf form: any function of (node, direction, distance); exact arithmetic"""
    return 1.0 + 2.0 * dist + 0.01 * d + 1e-4 * n


def test_oracle_whole_domain_extension_cf():
    """cf form: q starts at zero and takes the caller's values at the crossings; a constant cf
    extends to that constant near the interface."""
    f = sphere_grid(2, 6)
    og = O.OracleGrid.from_forest(f)
    x = f.node_xyz()
    phi = np.sqrt(np.sum(x ** 2, axis=1)) - 0.47  # no node on the interface (those keep q = 0)
    calls = []
    q = og.extend_from_interface_to_whole_domain_tvd_cf(phi, np.zeros(len(phi)), lambda n, d, s: (calls.append((n, d)), 0.25)[1],
                                                        iterations=60)
    assert calls == sorted(calls) and len(calls) > 0  # node by node, directions in order
    near = np.abs(phi) < 0.06  # two cells: converged to round-off from zero in 60 steps
    assert np.max(np.abs(q[near] - 0.25)) < 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["circle2d", "flower3d", "brick3d"])
def test_gpu_whole_domain_extension_cf_bitwise(name):
    f = GRIDS[name]()
    og = O.OracleGrid.from_forest(f)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    x, phi, _ = case(f)
    qi = field(x)
    want = og.extend_from_interface_to_whole_domain_tvd_cf(phi, qi, iface_value, iterations=7)
    got = ls.extend_from_interface_to_whole_domain_TVD(phi, qi, iterations=7, cf=iface_value)
    assert np.array_equal(got, want)
    with pytest.raises(ValueError):
        ls.extend_from_interface_to_whole_domain_TVD(phi, qi, iterations=2, cf=iface_value, mask=phi)
    with pytest.raises(ZeroDivisionError):
        ls.extend_from_interface_to_whole_domain_TVD(phi, qi, iterations=2, cf=lambda n, d, s: 1 / 0)


def test_oracle_extension_normal_derivative_outputs():
    """q_n / q_nn given: zero guesses give the same q as without them, and they come back holding the
    extended normal derivatives (for q = x + 2y inside a circle: n . (1, 2) near the interface)."""
    f = sphere_grid(2, 7)
    og = O.OracleGrid.from_forest(f)
    x = f.node_xyz()
    r = np.sqrt(np.sum(x ** 2, axis=1))
    phi = r - 0.47
    q0 = np.where(phi < 0, x[:, 0] + 2 * x[:, 1], 0.0)
    a = q0.copy()
    og.extend_over_interface_tvd(phi, a, 40, 2)
    b = q0.copy()
    qn, qnn = np.zeros(len(phi)), np.zeros(len(phi))
    og.extend_over_interface_tvd(phi, b, 40, 2, q_n=qn, q_nn=qnn)
    assert np.array_equal(a, b)
    nrm = x / np.maximum(r, 1e-12)[:, None]
    err = np.abs(qn - (nrm[:, 0] + 2 * nrm[:, 1]))
    inside = (phi < -0.05) & (phi > -0.2)  # computed by central differences
    assert np.max(err[inside]) < 0.05
    outside = (phi > 0) & (phi < 0.05)  # marched along the normals with the q_nn source
    assert np.median(err[outside]) < 0.05
    c = q0.copy()
    og.extend_over_interface_tvd(phi, c, 40, 2, use_nonzero_guess=True)
    band = np.abs(phi) < 0.05
    assert np.max(np.abs(c[band] - a[band])) < 1e-3  # the steady state does not depend on the guess


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["circle2d", "flower3d", "brick3d"])
@pytest.mark.parametrize("order", [1, 2])
def test_gpu_extension_guesses_and_outputs(name, order):
    f = GRIDS[name]()
    og = O.OracleGrid.from_forest(f)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    x, phi, q0 = case(f)
    rng = np.random.default_rng(7)
    for guess, give in ((False, True), (True, False), (True, True)):
        init_n = rng.uniform(-1, 1, len(phi)) if give else None
        init_nn = rng.uniform(-1, 1, len(phi)) if give else None
        w, g = q0.copy(), q0.copy()
        wn = None if init_n is None else init_n.copy()
        wnn = None if init_nn is None else init_nn.copy()
        gn = None if init_n is None else init_n.copy()
        gnn = None if init_nn is None else init_nn.copy()
        og.extend_over_interface_tvd(phi, w, 9, order, use_nonzero_guess=guess, q_n=wn, q_nn=wnn, nthreads=8)
        ls.extend_Over_Interface_TVD(phi, g, 9, order, use_nonzero_guess=guess, q_n=gn, q_nn=gnn)
        assert np.array_equal(g, w), (guess, give)
        if give:
            assert np.array_equal(gn, wn) and np.array_equal(gnn, wnn), (guess, give)
    with pytest.raises(ValueError):
        ls.extend_Over_Interface_TVD(phi, q0.copy(), 2, order, bc=object())
