"""Host regrid of the semi-Lagrangian step: splitting_criteria_tag_t::refine_and_coarsen
(src/my_p4est_refine_coarsen.cpp:422-479, 1170-1205) against a numpy restatement of the same rule,
plus leaf import and forest copies."""
import numpy as np
import pytest

import casl_p4est_gb300 as G

from grids import brick_3d, circle_2d, flower_3d


def expected_leaves(f, phi, min_lvl, max_lvl, lip):
    """numpy restatement: tag every leaf from its corner values, coarsen complete families tagged
    for coarsening, then refine the surviving leaves tagged for refinement."""
    dim = f.dim
    CH = 1 << dim
    maxl = 30 if dim == 2 else 19
    root = 1 << maxl
    tree, level, xyz = f.leaves()
    ln = f.local_nodes()
    fv = phi[ln]  # (nleaves, CH)
    span = (np.array(f.xyz_max[:dim]) - np.array(f.xyz_min[:dim])) / np.array(f.n_xyz[:dim])
    dmin = (root >> level).astype(np.float64) / root
    d = np.sqrt(np.sum((span[None, :] * dmin[:, None]) ** 2, axis=1))
    sign_change = np.any((fv[:, 1:] > 0) != (fv[:, :1] > 0), axis=1)
    refine = (level < max_lvl) & (np.any(np.abs(fv) <= 0.5 * lip * d[:, None], axis=1) | sign_change)
    coarsen = (level > min_lvl) & np.all(np.abs(fv) >= lip * d[:, None], axis=1) & ~sign_change
    tag = np.where(refine, 1, np.where(coarsen, -1, 0))
    tag[level < min_lvl] = 1
    tag[level > max_lvl] = -1
    out = []
    i, n = 0, len(level)
    while i < n:
        L = level[i]
        fam = False
        if L > 0 and i + CH <= n and all(xyz[i, a] % (root >> (L - 1)) == 0 for a in range(dim)):
            h = root >> L
            fam = True
            for c in range(CH):
                j = i + c
                if level[j] != L or tree[j] != tree[i] or tag[j] != -1:
                    fam = False
                    break
                if any(xyz[j, a] != xyz[i, a] + (h if (c >> a) & 1 else 0) for a in range(dim)):
                    fam = False
                    break
        if fam:
            out.append((tree[i], L - 1, *xyz[i, :dim]))
            i += CH
            continue
        if tag[i] == 1:
            h = root >> (L + 1)
            for c in range(CH):
                out.append((tree[i], L + 1, *[xyz[i, a] + (h if (c >> a) & 1 else 0) for a in range(dim)]))
        else:
            out.append((tree[i], L, *xyz[i, :dim]))
        i += 1
    return np.array(out, np.int64)


@pytest.mark.parametrize("make,shape", [
    (lambda: circle_2d(2, 7), G.shapes.sphere([0.13, -0.07], 0.45)),
    (lambda: flower_3d(2, 5), G.shapes.sphere([0.1, 0.05, -0.1], 0.4)),
    (lambda: brick_3d(1, 4), G.shapes.sphere([0.9, 0.4, 1.1], 0.35)),
])
def test_refine_and_coarsen_matches_restatement(make, shape):
    f = make()
    min_lvl, max_lvl = (2, 7) if f.dim == 2 else (1, 5)
    phi = f.sample(shape)
    want = expected_leaves(f, phi, min_lvl, max_lvl, 1.2)
    changed = f.refine_and_coarsen(min_lvl, max_lvl, phi, lip=1.2)
    tree, level, xyz = f.leaves()
    got = np.column_stack([tree, level, xyz[:, :f.dim]]).astype(np.int64)
    assert changed
    assert np.array_equal(got, want)


def test_regrid_converges_to_a_fixed_point():
    f = circle_2d(2, 6)
    shape = G.shapes.sphere([0.2, 0.1], 0.5)
    for _ in range(12):
        f.build_nodes()
        if not f.refine_and_coarsen(2, 6, f.sample(shape)):
            break
    else:
        pytest.fail("the regrid did not converge")
    f.build_nodes()  # nodes kept valid by an unchanged pass
    assert not f.refine_and_coarsen(2, 6, f.sample(shape))


def test_copy_and_set_leaves():
    f = flower_3d(2, 5)
    c = f.copy()
    assert c.num_nodes == f.num_nodes
    c.refine(np.ones(c.num_leaves, np.uint8))
    assert c.num_leaves == 8 * f.num_leaves and f.num_leaves == len(f.leaves()[0])
    d = G.my_p4est_brick_new([1, 1, 1], [-1, -1, -1], [1, 1, 1])
    t, l, x = f.leaves()
    d.set_leaves(t, l, x)
    d.build_nodes()
    assert np.array_equal(d.node_xyz(), f.node_xyz())
    with pytest.raises(G.LsgInvalidArgument):
        d.set_leaves(t[1:], l[1:], x[1:])
    bad = x.copy()
    bad[3, 0] += 1
    with pytest.raises(G.LsgInvalidArgument):
        d.set_leaves(t, l, bad)
