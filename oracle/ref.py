"""ORACLE — test infrastructure only: the reference's own level-set code, run on this machine's CPU.

ctypes binding of oracle/_ref/libref{2,3}d.so, built by `make -C oracle ref` from the reference sources where
they lie (src/casl_math.cpp, src/my_p4est_{utils,hierarchy,cell_neighbors,node_neighbors,
quad_neighbor_nodes_of_node,level_set,interpolation,interpolation_nodes,semi_lagrangian}.cpp,
src/my_p4est_tools.c) with single-process stand-ins for p4est, PETSc and MPI (oracle/ref_stubs/) and the
p4est structures built by oracle/ref_harness.cpp. It pins the restatement (oracle.py) to the reference
itself; it exists only where the reference tree is present (available() is False elsewhere).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_TREE = os.environ.get("CASL_REFERENCE_TREE", "/root/reference")
_P, _I, _I64, _D = C.c_void_p, C.c_int, C.c_int64, C.c_double
_DP = C.POINTER(C.c_double)
_SIG = {
    "last_error": (C.c_char_p, []),
    "dim": (_I, []),
    "record_bytes": (C.c_size_t, []),
    "create": (_I, [C.POINTER(_I), _DP, _DP, _I64, _P, _P, _P, C.POINTER(_P)]),
    "destroy": (None, [_P]),
    "num_nodes": (_I64, [_P]),
    "nodes": (_I, [_P, _P, _P]),
    "local_nodes": (_I, [_P, _P]),
    "node_xyz": (_I, [_P, _DP]),
    "wall_mask": (_I, [_P, _P]),
    "export_qnnn": (_I, [_P, _P]),
    "second_derivatives": (_I, [_P, _DP, _DP]),
    "first_derivatives": (_I, [_P, _DP, _DP]),
    "reinitialize": (_I, [_P, _DP, _I, _I, _D, _D, _I]),
    "reinitialize_2nd_order": (_I, [_P, _DP, _I]),
    "reinitialize_with_mask": (_I, [_P, _DP, _DP, _I, _D]),
    "advect_in_normal_direction": (_I, [_P, _DP, _DP, _DP, _D, _DP, _DP]),
    "interpolate": (_I, [_P, _I, _I, _DP, _DP, _I64, _DP, _DP]),
    "sl_advect": (_I, [_P, _D, _DP, _DP, _DP, _DP, _I, _I, _DP]),
    "sl_advect2": (_I, [_P, _P, _P, _D, _D, _DP, _DP, _DP, _DP, _DP, _DP, _I, _I, _DP]),
    "interface_location": (_D, [_D, _D, _D, _D]),
    "interface_location_2nd": (_D, [_D, _D, _D, _D, _D, _D]),
    "minmod": (_D, [_D, _D]),
}
_libs = {}


def lib_path(dim):
    return os.path.join(HERE, "_ref", f"libref{dim}d.so")


def available() -> bool:
    """True when the reference tree is present (the libraries can be built) or they were built already."""
    return os.path.isdir(os.path.join(REF_TREE, "src")) or (os.path.exists(lib_path(2)) and os.path.exists(lib_path(3)))


def build():
    if os.path.isdir(os.path.join(REF_TREE, "src")):
        subprocess.run(["make", "-s", "-C", HERE, f"-j{os.cpu_count() or 4}", "ref", f"REF={REF_TREE}"], check=True,
                       stdout=subprocess.DEVNULL)
    return lib_path(2), lib_path(3)


class _Lib:
    def __init__(self, dim):
        path = lib_path(dim)
        if not os.path.exists(path):
            build()
        self.dim = dim
        self.so = C.CDLL(path)
        self.prefix = f"refh{dim}_"
        for k, (r, a) in _SIG.items():
            f = getattr(self.so, self.prefix + k)
            f.restype = r
            f.argtypes = a

    def __getattr__(self, name):
        return getattr(self.so, self.prefix + name)


def load(dim) -> _Lib:
    if dim not in _libs:
        _libs[dim] = _Lib(dim)
    return _libs[dim]


def _chk(lib, code):
    if code != 0:
        raise RuntimeError("reference: " + lib.last_error().decode())


def _dp(a):
    return None if a is None else a.ctypes.data_as(_DP)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, np.float64)


class RefGrid:
    """The reference's node neighbourhood (my_p4est_node_neighbors_t) of one grid given leaf by leaf."""

    def __init__(self, dim, n_xyz, xyz_min, xyz_max, tree, level, xyz):
        self.dim = dim
        self.lib = load(dim)
        tree = np.ascontiguousarray(tree, np.int32)
        level = np.ascontiguousarray(level, np.int32)
        xyz = np.ascontiguousarray(xyz, np.int32).reshape(-1, 3)
        n = (C.c_int * 3)(*(list(n_xyz) + [1] * (3 - len(n_xyz))))
        lo = (C.c_double * 3)(*(list(xyz_min) + [0.0] * (3 - len(xyz_min))))
        hi = (C.c_double * 3)(*(list(xyz_max) + [0.0] * (3 - len(xyz_max))))
        h = C.c_void_p()
        _chk(self.lib, self.lib.create(n, lo, hi, len(tree), tree.ctypes.data, level.ctypes.data, xyz.ctypes.data, C.byref(h)))
        self._h = h
        self.N = int(self.lib.num_nodes(h))

    @classmethod
    def from_forest(cls, forest):
        tree, level, xyz = forest.leaves()
        return cls(forest.dim, forest.n_xyz[:forest.dim], forest.xyz_min[:forest.dim], forest.xyz_max[:forest.dim], tree, level, xyz)

    def __del__(self):
        if getattr(self, "_h", None) is not None:
            self.lib.destroy(self._h)
            self._h = None

    def nodes(self):
        tree = np.empty(self.N, np.int32)
        xyz = np.empty((self.N, 3), np.int32)
        _chk(self.lib, self.lib.nodes(self._h, tree.ctypes.data, xyz.ctypes.data))
        return tree, xyz

    def local_nodes(self, nleaves):
        out = np.empty((nleaves, 1 << self.dim), np.int32)
        _chk(self.lib, self.lib.local_nodes(self._h, out.ctypes.data))
        return out

    def node_xyz(self):
        out = np.empty((self.N, self.dim), np.float64)
        _chk(self.lib, self.lib.node_xyz(self._h, _dp(out)))
        return out

    def wall_mask(self):
        out = np.empty(self.N, np.uint8)
        _chk(self.lib, self.lib.wall_mask(self._h, out.ctypes.data))
        return out

    def qnnn(self, dtype):
        assert dtype.itemsize == self.lib.record_bytes()
        out = np.zeros(self.N, dtype=dtype)
        _chk(self.lib, self.lib.export_qnnn(self._h, out.ctypes.data))
        return out

    def second_derivatives(self, f):
        out = np.empty((self.dim, self.N), np.float64)
        _chk(self.lib, self.lib.second_derivatives(self._h, _dp(_f64(f)), _dp(out)))
        return out

    def first_derivatives(self, f):
        out = np.empty((self.dim, self.N), np.float64)
        _chk(self.lib, self.lib.first_derivatives(self._h, _dp(_f64(f)), _dp(out)))
        return out

    def reinitialize(self, phi, order_space=2, order_pseudotime=2, limit_high=np.finfo(np.float64).max,
                     limit_low=-np.finfo(np.float64).max, iterations=50):
        """Returns the reinitialised copy of phi."""
        out = np.array(phi, np.float64, copy=True)
        _chk(self.lib, self.lib.reinitialize(self._h, _dp(out), order_space, order_pseudotime, limit_high, limit_low, iterations))
        return out

    def reinitialize_2nd_order(self, phi, iterations=50):
        out = np.array(phi, np.float64, copy=True)
        _chk(self.lib, self.lib.reinitialize_2nd_order(self._h, _dp(out), iterations))
        return out

    def reinitialize_2nd_order_with_mask(self, phi, mask, iterations=50, limit=np.finfo(np.float64).max):
        out = np.array(phi, np.float64, copy=True)
        _chk(self.lib, self.lib.reinitialize_with_mask(self._h, _dp(out), _dp(_f64(mask)), iterations, limit))
        return out

    def advect_in_normal_direction(self, vn, phi, dt, vn_np1=None, phi_dd=None):
        """Returns (phi after the step, the dt the reference returns). phi_dd (float64, (D, N)) is updated in place
        as the reference updates the caller's derivative Vecs."""
        out = np.array(phi, np.float64, copy=True)
        r = C.c_double()
        if phi_dd is not None:
            assert phi_dd.dtype == np.float64 and phi_dd.flags.c_contiguous
        _chk(self.lib, self.lib.advect_in_normal_direction(self._h, _dp(_f64(vn)), _dp(_f64(vn_np1)), _dp(out), float(dt),
                                                           _dp(phi_dd), C.byref(r)))
        return out, r.value

    def interpolate(self, method, F, xyz, Fdd=None):
        F = _f64(F)
        single = F.ndim == 1
        F2 = F.reshape(1, -1) if single else F
        pts = np.ascontiguousarray(xyz, np.float64).reshape(-1, self.dim)
        out = np.empty((F2.shape[0], len(pts)), np.float64)
        _chk(self.lib, self.lib.interpolate(self._h, int(method), F2.shape[0], _dp(F2), _dp(_f64(Fdd)), len(pts), _dp(pts), _dp(out)))
        return out[0] if single else out

    def sl_advect(self, dt, v, vxx, phi, phi_xx, velo_method=4, phi_method=4):
        """advect_from_n_to_np1 with the new grid equal to this one: v (D, N), vxx (D, D, N), phi_xx (D, N)."""
        out = np.empty(self.N, np.float64)
        _chk(self.lib, self.lib.sl_advect(self._h, float(dt), _dp(_f64(v)), _dp(_f64(vxx)), _dp(_f64(phi)), _dp(_f64(phi_xx)),
                                          int(velo_method), int(phi_method), _dp(out)))
        return out

    def sl_advect2(self, grid_n, grid_nm1, dt_nm1, dt_n, vnm1, vxx_nm1, vn, vxx_n, phi_n, phi_xx_n, velo_method=4, phi_method=4):
        """Two-velocity step onto this grid; vn, vxx_n, phi_n, phi_xx_n on grid_n; vnm1, vxx_nm1 on grid_nm1."""
        out = np.empty(self.N, np.float64)
        _chk(self.lib, self.lib.sl_advect2(self._h, grid_n._h, grid_nm1._h, float(dt_nm1), float(dt_n), _dp(_f64(vnm1)),
                                           _dp(_f64(vxx_nm1)), _dp(_f64(vn)), _dp(_f64(vxx_n)), _dp(_f64(phi_n)), _dp(_f64(phi_xx_n)),
                                           int(velo_method), int(phi_method), _dp(out)))
        return out


def interface_location(dim, a, b, fa, fb):
    return load(dim).interface_location(a, b, fa, fb)


def interface_location_2nd(dim, a, b, fa, fb, fxxa, fxxb):
    return load(dim).interface_location_2nd(a, b, fa, fb, fxxa, fxxb)


def minmod(dim, a, b):
    return load(dim).minmod(a, b)
