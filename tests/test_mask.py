"""Reinitialisation with a mask (reinitialize_2nd_order_with_mask, src/my_p4est_level_set.h:487-525):
nodes where the mask is 0 are left out of the update lists and keep their value, while their neighbours
still read it. CPU: the oracle keeps masked nodes bit for bit, a mask of ones changes nothing, and a
mask changes the unmasked nodes next to it. GPU: FP64 bit-identical to the oracle in every order
(host and device arrays); mixed keeps masked nodes exactly and stays within the band tolerance."""
import numpy as np
import pytest

import casl_p4est_gb300 as G
import oracle as O

from grids import brick_2d, brick_3d, circle_2d, flower_3d

GRIDS = {
    "circle2d": lambda: circle_2d(3, 7),
    "brick2d": lambda: brick_2d(1, 6),
    "flower3d": lambda: flower_3d(3, 5),
    "brick3d": lambda: brick_3d(1, 5),
}


def case(f):
    x = f.node_xyz()
    phi = (np.sqrt(np.sum((x - 0.07) ** 2, axis=1)) - 0.45) * (1.0 + 0.3 * x[:, 0])
    mask = np.where(x[:, 1] > 0.2, 0.0, 1.0)  # nodes of the upper part are frozen
    return phi, mask


def test_oracle_mask():
    f = circle_2d(3, 7)
    og = O.OracleGrid.from_forest(f)
    phi, mask = case(f)
    a = phi.copy()
    og.reinitialize_with_mask(a, mask, iterations=10)
    assert np.array_equal(a[mask == 0], phi[mask == 0])
    b = phi.copy()
    og.reinitialize_with_mask(b, np.ones_like(mask), iterations=10)
    c = phi.copy()
    og.reinitialize(c, iterations=10)
    assert np.array_equal(b, c)
    assert not np.array_equal(a[mask != 0], c[mask != 0])


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(GRIDS))
def test_gpu_mask_fp64_bitwise(name):
    import torch
    from casl_p4est_gb300 import _lib as L
    f = GRIDS[name]()
    og = O.OracleGrid.from_forest(f)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    phi, mask = case(f)
    want = phi.copy()
    og.reinitialize_with_mask(want, mask, iterations=8)
    got = phi.copy()
    ls.reinitialize_2nd_order_with_mask(got, mask, int((mask == 0).sum()), 8)
    assert np.array_equal(got, want)
    for os_, ot in ((1, 1), (1, 2), (2, 1)):
        w = phi.copy()
        og.reinitialize_with_mask(w, mask, os_, ot, 0.3, -0.2, 6)
        g = phi.copy()
        L.check(L.load().lsg_reinitialize_with_mask(ls.handle, L.dptr(g), L.dptr(mask), os_, ot, 0.3, -0.2, 6, L.LSG_FP64))
        assert np.array_equal(g, w), (os_, ot)
    ls.set_stream(torch.cuda.current_stream().cuda_stream)
    t = torch.from_numpy(phi).cuda()
    ls.reinitialize_2nd_order_with_mask(t, torch.from_numpy(mask).cuda(), 0, 8)
    torch.cuda.synchronize()
    assert np.array_equal(t.cpu().numpy(), want)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["circle2d", "flower3d"])
def test_gpu_mask_mixed(name):
    f = GRIDS[name]()
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    phi, mask = case(f)
    ref = phi.copy()
    ls.reinitialize_2nd_order_with_mask(ref, mask, 0, 10)
    got = phi.copy()
    ls.reinitialize_2nd_order_with_mask(got, mask, 0, 10, precision="mixed")
    assert np.array_equal(got[mask == 0], phi[mask == 0])
    _, dmin, _ = f.dxyz_min()
    band = np.abs(ref) < 3 * dmin
    assert np.max(np.abs(got[band] - ref[band])) <= 1e-4 * dmin
