"""Host grid: node numbering, leaf corners, point location semantics and the node-neighbour records,
checked structurally and against the oracle's independent construction (cell tree + std::map
numbering) on several grids."""
import numpy as np
import pytest

import casl_p4est_gb300 as G
from casl_p4est_gb300 import shapes
import oracle as O

from grids import brick_2d, brick_3d, circle_2d, flower_3d


def morton_key(tree, xyz, dim):
    bits = 30 if dim == 2 else 19
    key = np.zeros(len(tree), dtype=object)
    for i in range(len(tree)):
        k = 0
        for b in range(bits):
            for a in range(dim):
                k |= ((int(xyz[i, a]) >> b) & 1) << (dim * b + a)
        key[i] = (int(tree[i]) << (dim * bits)) | k
    return key


@pytest.mark.parametrize("dim,level", [(2, 3), (2, 5), (3, 2), (3, 3)])
def test_uniform_grid_counts_and_stencils(dim, level):
    f = G.my_p4est_brick_new([1] * dim, [0.0] * dim, [1.0] * dim)
    for _ in range(level):
        f.refine(np.ones(f.num_leaves, np.uint8))
    f.build_nodes()
    assert f.num_leaves == (1 << level) ** dim
    assert f.num_nodes == ((1 << level) + 1) ** dim
    q = G.my_p4est_node_neighbors_t(f).get_neighbors()
    h = 1.0 / (1 << level)
    xyz = f.node_xyz()
    walls = f.wall_mask()
    interior = walls == 0
    assert np.all(q["d"][interior] == h)
    assert np.all(q["dt"][interior][:, :, 0] * q["dt"][interior][:, :, 1] == 0)
    # the m00 neighbour of an interior node is the node at x - h
    for n in np.where(interior)[0][:50]:
        for d in range(2 * dim):
            axis, side = divmod(d, 2)
            target = xyz[n].copy()
            target[axis] += h if side else -h
            cand = q["nb"][n, d]
            hits = [c for c in cand if np.allclose(xyz[c], target)]
            assert hits, (n, d)
    # wall nodes: second-degree neighbour at negative distance -2h
    for n in np.where(walls != 0)[0][:50]:
        for d in range(2 * dim):
            if walls[n] & (1 << d):
                assert q["d"][n, d] == -2 * h


def test_node_numbering_is_tree_morton_sorted_and_covers_leaf_corners():
    for f in (circle_2d(2, 6), brick_2d(1, 5), flower_3d(2, 4), brick_3d(1, 4)):
        tree, xyz = f.nodes()
        key = morton_key(tree, xyz, f.dim)
        assert all(key[i] < key[i + 1] for i in range(len(key) - 1))
        ln = f.local_nodes()
        ltree, level, lxyz = f.leaves()
        nx = f.node_xyz()
        ROOT = (1 << 30) if f.dim == 2 else (1 << 19)
        lo = np.array(f.xyz_min[: f.dim])
        size = (np.array(f.xyz_max[: f.dim]) - lo) / np.array(f.n_xyz[: f.dim])
        # physical corner of each leaf: the leaf's corner-0 node gives its tree origin
        for i in range(0, len(ltree), max(1, len(ltree) // 1500)):
            h = ROOT >> level[i]
            origin = nx[ln[i, 0]] - size * lxyz[i, : f.dim] / ROOT
            for c in range(1 << f.dim):
                off = np.array([h if (c >> a) & 1 else 0 for a in range(f.dim)])
                expect = origin + size * (lxyz[i, : f.dim] + off) / ROOT
                np.testing.assert_allclose(nx[ln[i, c]], expect, rtol=0, atol=1e-12)
        assert len(np.unique(ln)) == f.num_nodes  # every node is a leaf corner


@pytest.mark.parametrize("builder", [lambda: circle_2d(2, 7), lambda: brick_2d(1, 6), lambda: flower_3d(2, 5),
                                     lambda: brick_3d(1, 5)])
def test_neighbours_match_oracle(builder):
    f = builder()
    og = O.OracleGrid.from_forest(f)
    ptree, pxyz = f.nodes()
    otree, oxyz = og.nodes()
    assert np.array_equal(ptree, otree)
    assert np.array_equal(pxyz, oxyz.astype(np.int32))
    dt = G.qnnn_dtype(f.dim)
    pq = G.my_p4est_node_neighbors_t(f).get_neighbors()
    oq = og.qnnn(dt)
    for fld in dt.names:
        assert np.array_equal(pq[fld], oq[fld]), fld
    assert np.array_equal(f.wall_mask(), og.wall_mask())


def test_hanging_node_stencil_by_hand_2d():
    """[0,1]^2 split once, then the lower-left child split again: the node (0.5, 0.25) on the
    coarse/fine face sees the coarse cell [0.5,1]x[0,0.5] on its +x side, so its p00 neighbour is
    the virtual point (1, 0.25) interpolated between (1,0) and (1,0.5) with offsets 0.25/0.25."""
    f = G.my_p4est_brick_new([1, 1], [0, 0], [1, 1])
    f.refine(np.ones(1, np.uint8))
    f.refine(np.array([1, 0, 0, 0], np.uint8))
    f.build_nodes()
    xyz = f.node_xyz()
    q = G.my_p4est_node_neighbors_t(f).get_neighbors()
    n = int(np.where((xyz[:, 0] == 0.5) & (xyz[:, 1] == 0.25))[0][0])
    rec = q[n]
    assert rec["d"][1] == 0.5 and rec["d"][0] == 0.25
    assert tuple(rec["dt"][1]) == (0.25, 0.25)
    pm = [tuple(xyz[i]) for i in rec["nb"][1]]
    assert pm == [(1.0, 0.0), (1.0, 0.5)]
    # -x side: two fine cells of equal level, the first (mmm, below the node) wins the tie; the node
    # is its upper corner, so the m00 neighbour is the corner (0.25, 0.25) itself
    assert tuple(rec["dt"][0]) == (0.25, 0.0)
    assert tuple(xyz[rec["nb"][0][1]]) == (0.25, 0.25)
    # the node (0.5, 0.5) is a corner of the fine cell [0.25,0.5]^2 and of the coarse cells
    m = int(np.where((xyz[:, 0] == 0.5) & (xyz[:, 1] == 0.5))[0][0])
    assert q[m]["d"][0] == 0.25 and q[m]["d"][1] == 0.5


def test_sample_matches_numpy_shapes():
    f = flower_3d(2, 4)
    xyz = f.node_xyz()
    for sh in (shapes.sphere([0.1, 0.2, -0.1], 0.4), shapes.flower([0, 0, 0], 0.5, 0.1, 5, 4, scale=(0.2, (0.1, -0.2, 0.15))),
               shapes.spheres([[0.1, 0, 0], [-0.3, 0.2, 0.1]], [0.2, 0.3], scale=(0.1, (0.1, 0.1, 0.1)))):
        np.testing.assert_allclose(f.sample(sh), shapes.numpy_eval(*sh, xyz), rtol=1e-13, atol=1e-14)


def test_ellipse_distance_is_a_distance():
    # points on the ellipse boundary have zero distance; points at the centre -min(semi-axes)
    f = G.my_p4est_brick_new([1, 1], [-1, -1], [1, 1])
    for _ in range(5):
        f.refine(np.ones(f.num_leaves, np.uint8))
    f.build_nodes()
    sh = shapes.ellipses([(0.0, 0.0, 0.5, 0.25, 0.0)])
    v = f.sample(sh)
    xyz = f.node_xyz()
    c = np.where((xyz[:, 0] == 0) & (xyz[:, 1] == 0))[0][0]
    assert abs(v[c] + 0.25) < 1e-12
    on = np.where((xyz[:, 1] == 0) & (np.abs(xyz[:, 0]) == 0.5))[0]
    assert np.all(np.abs(v[on]) < 1e-12)
    far = np.where((xyz[:, 1] == 0) & (xyz[:, 0] == 1.0))[0][0]
    assert abs(v[far] - 0.5) < 1e-12


def test_refinement_criterion_levels():
    f = circle_2d(3, 7)
    _, level, _ = f.leaves()
    assert level.min() >= 3 and level.max() == 7
    # finest cells straddle the interface
    tree, lv, xyz = f.leaves()
    ROOT = 1 << 30
    fine = lv == 7
    cx = -1 + 2 * (xyz[fine, 0] + 0.5 * (ROOT >> 7)) / ROOT
    cy = -1 + 2 * (xyz[fine, 1] + 0.5 * (ROOT >> 7)) / ROOT
    r = np.sqrt(cx ** 2 + cy ** 2)
    assert np.max(np.abs(r - 0.5)) < 0.1
