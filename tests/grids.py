"""Grid builders shared by the tests (small versions of the benchmark workloads)."""
import numpy as np

import casl_p4est_gb300 as G
from casl_p4est_gb300 import shapes


def circle_2d(lmin=3, lmax=7, center=(0.0, 0.0), r=0.5, lip=2.4):
    """Workload 1 shape: refined where |sqrt(x^2+y^2)-0.5| < 1.2 diag."""
    f = G.my_p4est_brick_new([1, 1], [-1, -1], [1, 1])
    f.refine_levelset(shapes.sphere(center, r), lmin, lmax, lip=lip)
    f.build_nodes()
    return f


def phi0_circle_2d(f):
    """(sqrt(x^2+y^2) - 0.5)*(0.1 + (x-0.2)^2 + (y-0.3)^2), zero set the circle r = 0.5."""
    return f.sample(shapes.sphere_scaled([0, 0], 0.5, 0.1, [0.2, 0.3]))


def flower_3d(lmin=3, lmax=6, lip=2.4):
    f = G.my_p4est_brick_new([1, 1, 1], [-1, -1, -1], [1, 1, 1])
    f.refine_levelset(shapes.flower([0, 0, 0], 0.5, 0.1, 5, 4), lmin, lmax, lip=lip)
    f.build_nodes()
    return f


def phi0_flower_3d(f):
    return f.sample(shapes.flower([0, 0, 0], 0.5, 0.1, 5, 4, scale=(0.2, (0.1, -0.2, 0.15))))


def brick_2d(lmin=1, lmax=6):
    f = G.my_p4est_brick_new([3, 2], [-1, -1], [2, 1])
    f.refine_levelset(shapes.sphere([0.3, 0.1], 0.6), lmin, lmax, lip=1.2)
    f.build_nodes()
    return f


def brick_3d(lmin=1, lmax=5):
    f = G.my_p4est_brick_new([2, 1, 2], [0, 0, 0], [2, 1, 2])
    f.refine_levelset(shapes.sphere([0.7, 0.5, 0.9], 0.3), lmin, lmax, lip=1.2)
    f.build_nodes()
    return f


def brick_2d_odd(lmin=1, lmax=6):
    """3 x 2 trees of size 1/3 x 0.35: no cell size or neighbour distance is a power of two."""
    f = G.my_p4est_brick_new([3, 2], [0, 0], [1, 0.7])
    f.refine_levelset(shapes.sphere([0.45, 0.35], 0.2), lmin, lmax, lip=1.2)
    f.build_nodes()
    return f


def brick_3d_odd(lmin=1, lmax=5):
    """3 x 1 x 2 trees of size 1/3 x 0.3 x 0.25: x and y spacings are not powers of two, z spacings are."""
    f = G.my_p4est_brick_new([3, 1, 2], [0, 0, 0], [1, 0.3, 0.5])
    f.refine_levelset(shapes.sphere([0.5, 0.15, 0.25], 0.1), lmin, lmax, lip=1.2)
    f.build_nodes()
    return f


def band_error(phi, exact, band):
    m = np.abs(phi) < band
    return float(np.max(np.abs(phi[m] - exact[m]))) if m.any() else 0.0
