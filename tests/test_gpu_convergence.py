"""Convergence order of the GPU paths: mixed precision keeps FP64's order.

The shape of examples/reinitialization/main_2d.cpp:103-116, 234, 254-262 (circle r = 0.5 times
1 + 0.5 sin(5x) cos(4y), reinitialize_2nd_order, error max |phi - phi_exact| over |phi| < 3 diag_min) and its
3D form (1 + 0.5 sin(5(x+z)) cos(4(y-z))), at three levels. The mixed path (FP32 stencil and RK, FP64 subcell
step) must converge at the FP64 path's order (within 0.1), and both above 1.5; the FP64 GPU result is the
oracle's bit for bit."""
import numpy as np
import pytest

import casl_p4est_gb300 as G
import oracle as O
from casl_p4est_gb300 import shapes

from grids import band_error

pytestmark = pytest.mark.gpu


def errors(dim, lmax, iters=50, check_oracle=False):
    if dim == 2:
        f = G.my_p4est_brick_new([1, 1], [-1, -1], [1, 1])
        f.refine_levelset(shapes.sphere([0, 0], 0.5), 0, lmax, lip=1.2)
    else:
        f = G.my_p4est_brick_new([1, 1, 1], [-1, -1, -1], [1, 1, 1])
        f.refine_levelset(shapes.sphere([0, 0, 0], 0.5), 0, lmax, lip=1.2)
    f.build_nodes()
    x = f.node_xyz()
    exact = 0.5 - np.sqrt((x ** 2).sum(1))
    if dim == 2:
        phi0 = exact * (1 + 0.5 * np.sin(5 * x[:, 0]) * np.cos(4 * x[:, 1]))
    else:
        phi0 = exact * (1 + 0.5 * np.sin(5 * (x[:, 0] + x[:, 2])) * np.cos(4 * (x[:, 1] - x[:, 2])))
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f))
    p64 = phi0.copy()
    ls.reinitialize_2nd_order(p64, iters, precision="fp64")
    p32 = phi0.copy()
    ls.reinitialize_2nd_order(p32, iters, precision="mixed")
    if check_oracle:
        ref = phi0.copy()
        O.OracleGrid.from_forest(f).reinitialize(ref, iterations=iters)
        assert np.array_equal(p64, ref)
    _, dmin, diag = f.dxyz_min(lmax)
    e64 = band_error(p64, exact, 3 * diag)
    e32 = band_error(p32, exact, 3 * diag)
    # mixed stays within 1e-4 dx_min of FP64 in the band
    band = np.abs(p64) < 3 * dmin
    assert float(np.max(np.abs(p32[band] - p64[band]))) <= 1e-4 * dmin
    return e64, e32


@pytest.mark.parametrize("dim,levels", [(2, (6, 7, 8)), (3, (5, 6, 7))])
def test_mixed_converges_at_the_fp64_order(dim, levels):
    res = [errors(dim, l, check_oracle=(l == levels[0])) for l in levels]
    e64 = [r[0] for r in res]
    e32 = [r[1] for r in res]
    o64 = [np.log2(e64[i] / e64[i + 1]) for i in range(2)]
    o32 = [np.log2(e32[i] / e32[i + 1]) for i in range(2)]
    print(f"{dim}D levels {levels}: FP64 errors {e64} orders {o64}; mixed errors {e32} orders {o32}")
    assert min(o64) > 1.5 and min(o32) > 1.5, (o64, o32)
    assert max(abs(a - b) for a, b in zip(o64, o32)) < 0.1, (o64, o32)
