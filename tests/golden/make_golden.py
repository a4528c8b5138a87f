"""Generate the fixtures in this folder from the reference itself (run from the repository root, where the
reference tree is present):

    python tests/golden/make_golden.py [name ...]   (default: every fixture)

Each fixture holds small grids leaf by leaf (tree, level, logical corner), so Forest.set_leaves rebuilds them
exactly, the input fields, and the outputs of the reference's own code (oracle/_ref, compiled from the
reference sources by `make -C oracle ref`): second derivatives, reinitialisation (four order pairs, a phi_0
limit), normal advection, node interpolation (five methods), the semi-Lagrangian step with one velocity and
the two-velocity second-order step across three grids. Every value is also checked equal to the restatement
(oracle/) before it is written. The GPU tests compare the CUDA path with these numbers on machines without
the reference tree.

circle2d_L4-9_config1 is the 2D configuration as stated: [-1,1]^2, levels 4-9, refined where
|phi| <= 1.2 diag (lip 2.4), phi0 = (r - 0.5)(0.1 + (x-0.2)^2 + (y-0.3)^2), reinitialize_2nd_order for 20
iterations.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import casl_p4est_gb300 as G  # noqa: E402
import oracle as O  # noqa: E402
import ref as R  # noqa: E402
from casl_p4est_gb300 import shapes  # noqa: E402
from grids import brick_2d, brick_3d_odd, circle_2d, flower_3d, phi0_circle_2d, phi0_flower_3d  # noqa: E402

DBL_MAX = np.finfo(np.float64).max


def same(a, b, what):
    if not np.array_equal(a, b):
        raise SystemExit(f"restatement differs from the reference: {what}")
    return a


def grid_arrays(prefix, f):
    tree, level, xyz = f.leaves()
    return {prefix + "tree": tree, prefix + "level": level, prefix + "lxyz": xyz}


def velocity(x, dim, s):
    return np.stack([-x[:, 1] + 0.1 * s, x[:, 0] * s] + ([0.3 * x[:, 0] - 0.2 * x[:, 1]] if dim == 3 else []))


def make(name, f, phi0, f_nm1=None, f_np1=None):
    rg = R.RefGrid.from_forest(f)
    og = O.OracleGrid.from_forest(f)
    x = f.node_xyz()
    out = {"n_xyz": np.array(f.n_xyz, np.int32), "xyz_min": np.array(f.xyz_min), "xyz_max": np.array(f.xyz_max),
           "dim": np.int32(f.dim), "node_xyz": x, "phi0": phi0}
    tree, level, xyz = f.leaves()
    out.update({"tree": tree, "level": level, "lxyz": xyz})
    out["dd"] = same(rg.second_derivatives(phi0), og.compute_derivatives(phi0), "second derivatives")
    for os_, ot in [(2, 2), (1, 1), (1, 2), (2, 1)]:
        p = phi0.copy()
        og.reinitialize(p, os_, ot, iterations=8)
        out[f"reinit_{os_}{ot}"] = same(rg.reinitialize(phi0, os_, ot, DBL_MAX, -DBL_MAX, 8), p, f"reinit {os_}{ot}")
    lim = phi0.copy()
    og.reinitialize(lim, 2, 2, limit_high=0.3, limit_low=-0.2, iterations=8)
    out["reinit_22_limited"] = same(rg.reinitialize(phi0, 2, 2, 0.3, -0.2, 8), lim, "reinit limited")
    vn = 1.0 + 0.5 * np.sin(3 * x[:, 0])
    dt = 0.4 * og.advect_cfl_dt(vn)
    adv = out["reinit_22"].copy()
    og.advect_in_normal_direction(vn, adv, dt)
    out["vn"] = vn
    out["advect_dt"] = np.float64(dt)
    out["advect"] = same(rg.advect_in_normal_direction(vn, out["reinit_22"], dt)[0], adv, "normal advection")
    rng = np.random.default_rng(11)
    lo, hi = np.array(f.xyz_min[:f.dim]) - 0.02, np.array(f.xyz_max[:f.dim]) + 0.02
    pts = np.concatenate([lo + (hi - lo) * rng.random((400, f.dim)), x[::7]])
    out["points"] = pts
    for m in range(5):
        out[f"interp_{m}"] = same(rg.interpolate(m, out["reinit_22"], pts), og.interpolate(m, out["reinit_22"], pts), f"interp {m}")
    v = velocity(x, f.dim, 1.0)
    vxx = np.stack([rg.second_derivatives(v[c]) for c in range(f.dim)])
    pdd = rg.second_derivatives(out["reinit_22"])
    out["velocity"] = v
    out["sl"] = same(rg.sl_advect(0.05, v, vxx, out["reinit_22"], pdd), og.sl_advect(x, 0.05, v, out["reinit_22"]), "SL step")
    if f_nm1 is not None:
        # two-velocity step: velocity n on this grid, velocity n-1 on f_nm1, new grid f_np1
        r_nm1, r_np1 = R.RefGrid.from_forest(f_nm1), R.RefGrid.from_forest(f_np1)
        vnm1 = velocity(f_nm1.node_xyz(), f.dim, 0.8)
        vxx_nm1 = np.stack([r_nm1.second_derivatives(vnm1[c]) for c in range(f.dim)])
        out.update(grid_arrays("nm1_", f_nm1))
        out.update(grid_arrays("np1_", f_np1))
        out["vnm1"] = vnm1
        for vm in (4, 1):
            out[f"sl2_{vm}"] = r_np1.sl_advect2(rg, r_nm1, 0.04, 0.05, vnm1, vxx_nm1, v, vxx, out["reinit_22"], pdd, vm, vm)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(name, f.num_nodes, "nodes")


def make_config1():
    """The 2D configuration: reinitialize_2nd_order, 20 iterations, FP64; the reference's result and its error
    max |phi - (r - 0.5)| in |phi| < 3 dx_min."""
    f = circle_2d(4, 9)
    phi0 = phi0_circle_2d(f)
    rg = R.RefGrid.from_forest(f)
    og = O.OracleGrid.from_forest(f)
    p = phi0.copy()
    og.reinitialize(p, 2, 2, iterations=20)
    out = same(rg.reinitialize_2nd_order(phi0, 20), p, "configuration 1")
    x = f.node_xyz()
    exact = np.sqrt(x[:, 0] ** 2 + x[:, 1] ** 2) - 0.5
    dmin = 2.0 / (1 << 9)
    band = np.abs(out) < 3 * dmin
    err = float(np.max(np.abs(out[band] - exact[band])))
    tree, level, xyz = f.leaves()
    np.savez_compressed(os.path.join(HERE, "circle2d_L4-9_config1.npz"), n_xyz=np.array(f.n_xyz, np.int32),
                        xyz_min=np.array(f.xyz_min), xyz_max=np.array(f.xyz_max), dim=np.int32(2), tree=tree, level=level, lxyz=xyz,
                        node_xyz=x, phi0=phi0, reinit_20=out, band_error=np.float64(err), dx_min=np.float64(dmin))
    print("circle2d_L4-9_config1", f.num_nodes, "nodes, band error", err, "=", err / dmin, "dx_min")


def fixtures():
    def circle():
        f2 = circle_2d(3, 6)
        make("circle2d_L3-6", f2, phi0_circle_2d(f2), circle_2d(3, 5, center=(0.05, -0.03)), circle_2d(3, 6, center=(0.02, 0.01)))

    def flower():
        f3 = flower_3d(2, 4)
        make("flower3d_L2-4", f3, phi0_flower_3d(f3), flower_3d(2, 3), flower_3d(2, 5))

    def brick():
        fb = brick_2d(1, 5)
        make("brick2d_3x2_L1-5", fb, fb.sample(shapes.sphere_scaled([0.3, 0.1], 0.6, 0.1, [0.2, 0.3])))

    def brick_odd():
        # tree sizes 1/3 x 0.3 x 0.25: neighbour distances that are not powers of two
        fo = brick_3d_odd(1, 4)
        make("brick3d_odd_L1-4", fo, fo.sample(shapes.sphere_scaled([0.5, 0.15, 0.25], 0.1, 0.1, [0.3, 0.1, 0.2])))

    return {"circle2d_L3-6": circle, "flower3d_L2-4": flower, "brick2d_3x2_L1-5": brick, "brick3d_odd_L1-4": brick_odd,
            "circle2d_L4-9_config1": make_config1}


if __name__ == "__main__":
    todo = fixtures()
    for name in (sys.argv[1:] or list(todo)):
        todo[name]()
