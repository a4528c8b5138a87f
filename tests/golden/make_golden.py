"""Generate the regression fixtures in this folder (run from the repository root):

    python tests/golden/make_golden.py

Each fixture holds a small grid leaf by leaf (tree, level, logical corner) so it is rebuilt exactly by
Forest.set_leaves, the input fields, and the oracle's FP64 outputs: second derivatives, reinitialisation
(four order pairs), normal advection, node interpolation (five methods) and a semi-Lagrangian step.
The reference itself cannot run here (p4est, PETSc and MPI are absent) and its tests hold no value-level
vectors for this path, so these fixtures pin the oracle and the CUDA path to each other across changes,
not to reference binaries."""
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
from grids import circle_2d, flower_3d, phi0_circle_2d, phi0_flower_3d  # noqa: E402


def make(name, f, phi0):
    og = O.OracleGrid.from_forest(f)
    tree, level, xyz = f.leaves()
    x = f.node_xyz()
    out = {"n_xyz": np.array(f.n_xyz, np.int32), "xyz_min": np.array(f.xyz_min), "xyz_max": np.array(f.xyz_max),
           "dim": np.int32(f.dim), "tree": tree, "level": level, "lxyz": xyz, "node_xyz": x, "phi0": phi0}
    out["dd"] = og.compute_derivatives(phi0)
    for os_, ot in [(2, 2), (1, 1), (1, 2), (2, 1)]:
        p = phi0.copy()
        og.reinitialize(p, os_, ot, iterations=8)
        out[f"reinit_{os_}{ot}"] = p
    lim = phi0.copy()
    og.reinitialize(lim, 2, 2, limit_high=0.3, limit_low=-0.2, iterations=8)
    out["reinit_22_limited"] = lim
    vn = 1.0 + 0.5 * np.sin(3 * x[:, 0])
    adv = out["reinit_22"].copy()
    og.advect_in_normal_direction(vn, adv, 0.4 * og.advect_cfl_dt(vn))
    out["vn"] = vn
    out["advect"] = adv
    rng = np.random.default_rng(11)
    pts = np.concatenate([rng.uniform(-1.02, 1.02, (400, f.dim)), x[::7]])
    out["points"] = pts
    for m in range(5):
        out[f"interp_{m}"] = og.interpolate(m, out["reinit_22"], pts)
    v = np.stack([-x[:, 1], x[:, 0]] + ([0.3 * x[:, 0]] if f.dim == 3 else []))
    out["velocity"] = v
    out["sl"] = og.sl_advect(x, 0.05, v, out["reinit_22"])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(name, f.num_nodes, "nodes")


if __name__ == "__main__":
    f2 = circle_2d(3, 6)
    make("circle2d_L3-6", f2, phi0_circle_2d(f2))
    f3 = flower_3d(2, 4)
    make("flower3d_L2-4", f3, phi0_flower_3d(f3))
