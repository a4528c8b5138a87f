"""First derivatives, normals and mean curvature (first_derivatives_central, compute_normals,
compute_mean_curvature, compute_normals_and_mean_curvature).

CPU: the oracle's gradient (with the tangential second-derivative correction at hanging nodes) is exact
on quadratics away from walls, and the curvature of a circle / sphere converges to (dim-1)/r.
GPU: the FP64 kernels are bit-identical to the oracle."""
import numpy as np
import pytest

import casl_p4est_gb300 as G
import oracle as O

from grids import brick_2d, brick_3d, circle_2d, flower_3d


def quad(x):
    f = 0.3 + 0.7 * x[:, 0] - 0.2 * x[:, 1] + 0.5 * x[:, 0] ** 2 + 0.25 * x[:, 1] ** 2 + 0.1 * x[:, 0] * x[:, 1]
    g = [0.7 + x[:, 0] + 0.1 * x[:, 1], -0.2 + 0.5 * x[:, 1] + 0.1 * x[:, 0]]
    if x.shape[1] == 3:
        f = f + 0.4 * x[:, 2] - 0.3 * x[:, 2] ** 2 + 0.2 * x[:, 1] * x[:, 2]
        g[1] = g[1] + 0.2 * x[:, 2]
        g.append(0.4 - 0.6 * x[:, 2] + 0.2 * x[:, 1])
    return f, np.stack(g)


@pytest.mark.parametrize("make", [lambda: circle_2d(3, 7), lambda: flower_3d(2, 5)])
def test_oracle_gradient_exact_on_quadratics(make):
    f = make()
    og = O.OracleGrid.from_forest(f)
    x = f.node_xyz()
    F, g = quad(x)
    got = og.first_derivatives(F)
    inner = og.wall_mask() == 0
    assert np.max(np.abs(got[:, inner] - g[:, inner])) < 1e-12


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_curvature_converges(dim):
    """phi = |x| - 0.5: the level set through a node is the sphere of radius |x|, curvature (dim-1)/|x|."""
    errs = []
    for lmax in ((6, 7, 8) if dim == 2 else (4, 5, 6)):
        f = G.my_p4est_brick_new([1] * dim, [-1] * dim, [1] * dim)
        f.refine_levelset(G.shapes.sphere([0.0] * dim, 0.5), 2, lmax, lip=2.4)
        f.build_nodes()
        og = O.OracleGrid.from_forest(f)
        x = f.node_xyz()
        r = np.sqrt(np.sum(x ** 2, axis=1))
        phi = r - 0.5
        _, kappa = og.normals_and_mean_curvature(phi)
        k2 = og.mean_curvature_from_normals(og.compute_normals(phi))
        h = 2.0 / (1 << lmax)
        band = (np.abs(phi) < 2 * h) & (og.wall_mask() == 0)
        exact = (dim - 1) / r[band]
        errs.append(max(np.max(np.abs(kappa[band] - exact)), np.max(np.abs(k2[band] - exact))))
    assert errs[1] < 0.6 * errs[0] and errs[2] < 0.6 * errs[1], errs


GRIDS = {
    "circle2d": lambda: circle_2d(3, 8),
    "brick2d": lambda: brick_2d(1, 6),
    "flower3d": lambda: flower_3d(3, 6),
    "brick3d": lambda: brick_3d(1, 5),
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(GRIDS))
def test_gpu_derivatives_bitwise(name):
    f = GRIDS[name]()
    og = O.OracleGrid.from_forest(f)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    x = f.node_xyz()
    phi = (np.sqrt(np.sum((x - 0.07) ** 2, axis=1)) - 0.45) * (1.0 + 0.3 * x[:, 0])
    assert np.array_equal(ls.first_derivatives_central(phi), og.first_derivatives(phi))
    nrm = ls.compute_normals(phi)
    assert np.array_equal(nrm, og.compute_normals(phi))
    assert np.array_equal(ls.compute_mean_curvature(nrm), og.mean_curvature_from_normals(nrm))
    n2, k2 = ls.compute_normals_and_mean_curvature(phi)
    on2, ok2 = og.normals_and_mean_curvature(phi)
    assert np.array_equal(n2, on2) and np.array_equal(k2, ok2)
