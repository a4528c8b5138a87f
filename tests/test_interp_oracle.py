"""Known answers for the oracle's node interpolation, point location and semi-Lagrangian step
(the restatement the CUDA path is checked against).

- Every quadratic method reproduces quadratics exactly (second derivatives of a quadratic are exact on
  uniform, hanging and wall stencils, and the minmod of equal values is that value); linear reproduces
  linear functions.
- The located leaf contains the clipped point; a point within the face threshold of several leaves gets
  the finest of them.
- A constant velocity translates a linear phi exactly (away from the clipped boundary)."""
import numpy as np
import pytest

import oracle as O

from grids import circle_2d, flower_3d

METHODS = [0, 1, 2, 3, 4]


def quad_fn(x):
    d = x.shape[1]
    f = 1.0 + 0.3 * x[:, 0] - 0.7 * x[:, 1] + 0.5 * x[:, 0] ** 2 + 0.25 * x[:, 1] ** 2 + 0.1 * x[:, 0] * x[:, 1]
    if d == 3:
        f = f + 0.2 * x[:, 2] - 0.4 * x[:, 2] ** 2 + 0.15 * x[:, 1] * x[:, 2]
    return f


def lin_fn(x):
    f = 0.5 + 0.3 * x[:, 0] - 0.7 * x[:, 1]
    if x.shape[1] == 3:
        f = f + 0.2 * x[:, 2]
    return f


@pytest.fixture(scope="module", params=["circle2d", "flower3d"])
def grid(request):
    f = circle_2d(3, 7) if request.param == "circle2d" else flower_3d(2, 5)
    return f, O.OracleGrid.from_forest(f)


def test_quadratic_methods_exact_on_quadratics(grid):
    f, og = grid
    x = f.node_xyz()
    F = quad_fn(x)
    pts = np.random.default_rng(1).uniform(-1, 1, (4000, f.dim))
    exact = quad_fn(pts)
    for m in METHODS[1:]:
        got = og.interpolate(m, F, pts)
        assert np.max(np.abs(got - exact)) < 1e-13, m
    got = og.interpolate(0, lin_fn(x), pts)
    assert np.max(np.abs(got - lin_fn(pts))) < 1e-13


def test_located_leaf_contains_point(grid):
    f, og = grid
    tree, level, lxyz = f.leaves()
    lo, hi = np.array(f.xyz_min[:f.dim]), np.array(f.xyz_max[:f.dim])
    rng = np.random.default_rng(2)
    pts = rng.uniform(-1.2, 1.2, (3000, f.dim))
    leaf = og.locate(pts)
    clip = np.clip(pts, lo, hi)
    root = 2 ** (30 if f.dim == 2 else 19)
    # single tree on [-1, 1]^dim: logical = (x + 1)/2 * root
    q0 = lxyz[leaf, :f.dim].astype(np.float64)
    h = (root >> level[leaf]).astype(np.float64)[:, None]
    s = (clip - lo) / (hi - lo) * root
    assert np.all(s >= q0 - 1e-6 * root) and np.all(s <= q0 + h + 1e-6 * root)


def test_face_points_take_the_finest_leaf(grid):
    f, og = grid
    tree, level, lxyz = f.leaves()
    x = f.node_xyz()
    leaf = og.locate(x)
    # a node is a corner of every leaf touching it: the chosen leaf is the finest touching one
    ln = f.local_nodes().reshape(len(level), -1)
    finest = np.full(f.num_nodes, -1)
    for c in range(ln.shape[1]):
        np.maximum.at(finest, ln[:, c], level)
    assert np.array_equal(level[leaf], finest)


def test_sl_constant_velocity_translates_linear_phi(grid):
    f, og = grid
    x = f.node_xyz()
    vel = np.array([0.3, -0.2, 0.1][:f.dim])
    v = np.repeat(vel[:, None], f.num_nodes, axis=1)
    phi = lin_fn(x)
    dt = 0.05
    for vm, pm in [(4, 4), (1, 2), (0, 0), (3, 1)]:
        out = og.sl_advect(x, dt, v, phi, velo_method=vm, phi_method=pm)
        inner = np.all(np.abs(x - dt * vel) < 1.0, axis=1)
        assert np.max(np.abs(out[inner] - lin_fn(x[inner] - dt * vel))) < 1e-13


def test_sl_vortex_backtrace_of_linear_phi(grid):
    """CF overload: for a linear phi every method is exact, so phi_np1 is phi at the RK2 departure
    point x_d = clip(x - dt v(clip(x - dt/2 v(x)))) of the single vortex."""
    f, og = grid
    x = f.node_xyz()
    phi = lin_fn(x)
    dt = 0.02
    lo, hi = np.array(f.xyz_min[:f.dim]), np.array(f.xyz_max[:f.dim])
    xs = np.clip(x - 0.5 * dt * O.vortex(f.dim, x, -1.0).T, lo, hi)
    xd = np.clip(x - dt * O.vortex(f.dim, xs, -1.0).T, lo, hi)
    for m in METHODS:
        out = og.sl_advect_vortex(x, dt, -1.0, phi, phi_method=m)
        assert np.max(np.abs(out - lin_fn(xd))) < 1e-13, m
