"""Analytic level-set shapes (kind + flat parameter vector) understood by the native grid builder.

Each constructor returns ``(kind, params)`` for ``Forest.refine_levelset`` / ``Forest.sample``; the
formulas are documented in ``csrc/shapes.h``. ``numpy_eval`` evaluates the same functions in numpy
(used by tests to cross-check the native sampler).
"""
from __future__ import annotations

import numpy as np

SPHERE, SPHERE_SCALED, FLOWER, SPHERES, ELLIPSES = range(5)


def sphere(center, radius):
    c = list(center) + [0.0] * (3 - len(center))
    return SPHERE, np.array(c + [radius], dtype=np.float64)


def sphere_scaled(center, radius, a, p):
    c = list(center) + [0.0] * (3 - len(center))
    pp = list(p) + [0.0] * (3 - len(p))
    return SPHERE_SCALED, np.array(c + [radius, a] + pp, dtype=np.float64)


def flower(center, r0, amp, k_theta, k_phi=0.0, scale=None):
    """r - (r0 + amp sin(k_theta*theta) [sin(k_phi*phi)]), optionally times (a + |x - p|^2)."""
    c = list(center) + [0.0] * (3 - len(center))
    if scale is None:
        a, p, on = 0.0, [0.0, 0.0, 0.0], 0.0
    else:
        a, p = scale
        p = list(p) + [0.0] * (3 - len(p))
        on = 1.0
    return FLOWER, np.array(c + [r0, amp, k_theta, k_phi, a] + p + [on], dtype=np.float64)


def spheres(centers, radii, scale=None):
    centers = np.asarray(centers, dtype=np.float64)
    n = len(radii)
    if scale is None:
        a, p, on = 0.0, [0.0, 0.0, 0.0], 0.0
    else:
        a, p = scale
        p = list(p) + [0.0] * (3 - len(p))
        on = 1.0
    body = []
    for i in range(n):
        c = list(centers[i]) + [0.0] * (3 - centers.shape[1])
        body += c + [float(radii[i])]
    return SPHERES, np.array([n, a] + p + [on] + body, dtype=np.float64)


def ellipses(items, scale=None):
    """items: list of (cx, cy, ax, ay, angle); scale: (a, (px, py), s) -> times (a + s|x-p|^2)."""
    if scale is None:
        a, p, s, on = 0.0, (0.0, 0.0), 0.0, 0.0
    else:
        a, p, s = scale
        on = 1.0
    body = []
    for it in items:
        body += [float(v) for v in it]
    return ELLIPSES, np.array([len(items), a, p[0], p[1], s, on] + body, dtype=np.float64)


def numpy_eval(kind: int, params: np.ndarray, xyz: np.ndarray) -> np.ndarray:
    """Same functions in numpy (except ELLIPSES); xyz is (n, dim)."""
    x = np.asarray(xyz, dtype=np.float64)
    dim = x.shape[1]
    p = params
    if kind == SPHERE:
        return np.sqrt(((x - p[:dim]) ** 2).sum(1)) - p[3]
    if kind == SPHERE_SCALED:
        return (np.sqrt(((x - p[:dim]) ** 2).sum(1)) - p[3]) * (p[4] + ((x - p[5:5 + dim]) ** 2).sum(1))
    if kind == FLOWER:
        rel = x - p[:dim]
        r = np.sqrt((rel ** 2).sum(1))
        theta = np.arctan2(rel[:, 1], rel[:, 0])
        if dim == 3:
            with np.errstate(invalid="ignore", divide="ignore"):
                phi = np.where(r > 0, np.arccos(np.clip(rel[:, 2] / np.where(r > 0, r, 1), -1, 1)), 0.0)
            rs = p[3] + p[4] * np.sin(p[5] * theta) * np.sin(p[6] * phi)
        else:
            rs = p[3] + p[4] * np.sin(p[5] * theta)
        v = r - rs
        if p[11] != 0:
            v = v * (p[7] + ((x - p[8:8 + dim]) ** 2).sum(1))
        return v
    if kind == SPHERES:
        n = int(p[0])
        body = p[6:].reshape(n, 4)
        d = np.min(np.sqrt(((x[:, None, :] - body[None, :, :dim]) ** 2).sum(2)) - body[None, :, 3], axis=1)
        if p[5] != 0:
            d = d * (p[1] + ((x - p[2:2 + dim]) ** 2).sum(1))
        return d
    raise NotImplementedError(kind)
