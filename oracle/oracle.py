"""ORACLE — test infrastructure only (tests/, smoke() and the benchmark's CPU baseline).

ctypes binding of oracle/_build/liboracle.so, the CPU restatement of parCASL's level-set loops
(oracle.cpp). Used as the checker of the CUDA path; never imported by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

_P, _I, _I64, _D = C.c_void_p, C.c_int, C.c_int64, C.c_double
_DP = C.POINTER(C.c_double)
SIG = {
    "ora_last_error": (C.c_char_p, []),
    "ora_qnnn_record_bytes": (C.c_size_t, [_I]),
    "ora_grid_from_leaves": (_I, [_I, C.POINTER(_I), _DP, _DP, _I64, _P, _P, _P, C.POINTER(_P)]),
    "ora_grid_from_qnnn": (_I, [_I, _I64, _P, _P, _DP, C.POINTER(_P)]),
    "ora_grid_destroy": (None, [_P]),
    "ora_grid_num_nodes": (_I64, [_P]),
    "ora_zero_distance_threshold": (_D, [_P]),
    "ora_grid_nodes": (_I, [_P, _P, _P]),
    "ora_grid_export_qnnn": (_I, [_P, _P]),
    "ora_grid_wall_mask": (_I, [_P, _P]),
    "ora_compute_derivatives": (_I, [_P, _DP, _DP, _I]),
    "ora_reinitialize": (_I, [_P, _DP, _I, _I, _D, _D, _I, _I]),
    "ora_reinitialize_masked": (_I, [_P, _DP, _DP, _I, _I, _D, _D, _I, _I]),
    "ora_advect_in_normal_direction": (_I, [_P, _DP, _DP, _DP, _D, _DP, _I]),
    "ora_advect_cfl_dt": (_I, [_P, _DP, _DP]),
    "ora_interpolate": (_I, [_P, _I, _I, _DP, _DP, _I64, _DP, _DP, _I]),
    "ora_locate": (_I, [_P, _I64, _DP, _P]),
    "ora_sl_advect": (_I, [_P, _I64, _DP, _D, _DP, _DP, _DP, _DP, _I, _I, _DP, _I]),
    "ora_sl_advect_vortex": (_I, [_P, _I64, _DP, _D, _D, _DP, _DP, _I, _DP, _I]),
    "ora_compute_derivatives_range": (_I, [_P, _DP, _DP, _I64, _I64, _I]),
    "ora_reinit_stage_range": (_I, [_P, _DP, _DP, _DP, _D, _D, _DP, _DP, _I64, _I64, _I]),
    "ora_advect_stage_range": (_I, [_P, _DP, _D, _DP, _DP, _DP, _I64, _I64, _I]),
    "ora_sl_advect2": (_I, [_P, _P, _I64, _DP, _D, _D, _DP, _DP, _DP, _DP, _DP, _DP, _I, _I, _DP, _I]),
    "ora_vortex": (_I, [_I, _I64, _DP, _D, _DP]),
    "ora_first_derivatives": (_I, [_P, _DP, _DP, _I]),
    "ora_compute_normals": (_I, [_P, _DP, _DP, _I]),
    "ora_mean_curvature_from_normals": (_I, [_P, _DP, _DP, _I]),
    "ora_normals_and_mean_curvature": (_I, [_P, _DP, _DP, _DP, _I]),
    "ora_extend_over_interface": (_I, [_P, _DP, _DP, _DP, _I, _I, _D, _D, _DP, _I]),
    "ora_extend_over_interface_ex": (_I, [_P, _DP, _DP, _DP, _I, _I, _D, _D, _DP, _I, _DP, _DP, _I]),
    "ora_extend_from_interface": (_I, [_P, _DP, _DP, _DP, _I, _DP, _D, _D, _DP, _I, _I]),
    "ora_extend_from_interface_cf": (_I, [_P, _DP, _DP, _DP, _I, _P, _P, _DP, _I]),
    "ora_interface_location": (_D, [_D, _D, _D, _D]),
    "ora_interface_location_2nd": (_D, [_D, _D, _D, _D, _D, _D]),
}
_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        lib = C.CDLL(LIB)
        for k, (r, a) in SIG.items():
            f = getattr(lib, k)
            f.restype = r
            f.argtypes = a
        _lib = lib
    return _lib


def _chk(code):
    if code != 0:
        raise RuntimeError("oracle: " + load().ora_last_error().decode())


def _dp(a):
    return a.ctypes.data_as(_DP) if a is not None else None


class OracleGrid:
    """CPU restatement of the grid-side objects and the level-set loops."""

    def __init__(self, handle, dim):
        self._h = handle
        self.dim = dim
        self.N = int(load().ora_grid_num_nodes(handle))
        self.zero_distance_threshold = float(load().ora_zero_distance_threshold(handle))

    @classmethod
    def from_forest(cls, forest):
        """Build nodes, cell tree and neighbours from the leaves of a product Forest (own numbering)."""
        tree, level, xyz = forest.leaves()
        n = (C.c_int * 3)(*forest.n_xyz)
        lo = (C.c_double * 3)(*forest.xyz_min)
        hi = (C.c_double * 3)(*forest.xyz_max)
        h = C.c_void_p()
        _chk(load().ora_grid_from_leaves(forest.dim, n, lo, hi, len(tree), tree.ctypes.data, level.ctypes.data, xyz.ctypes.data,
                                         C.byref(h)))
        return cls(h, forest.dim)

    @classmethod
    def from_records(cls, dim, qnnn_records, wall, tree_dims):
        qn = np.ascontiguousarray(qnnn_records)
        w = np.ascontiguousarray(wall, dtype=np.uint8)
        td = np.ascontiguousarray(list(tree_dims) + [1.0] * (3 - len(tree_dims)), dtype=np.float64)
        h = C.c_void_p()
        _chk(load().ora_grid_from_qnnn(dim, len(qn), qn.ctypes.data, w.ctypes.data, _dp(td), C.byref(h)))
        g = cls(h, dim)
        g._records = qn  # the library borrows the records
        return g

    def __del__(self):
        if getattr(self, "_h", None) is not None:
            load().ora_grid_destroy(self._h)
            self._h = None

    def nodes(self):
        tree = np.empty(self.N, np.int32)
        xyz = np.empty((self.N, 3), np.int64)
        _chk(load().ora_grid_nodes(self._h, tree.ctypes.data, xyz.ctypes.data))
        return tree, xyz

    def qnnn(self, dtype):
        out = np.zeros(self.N, dtype=dtype)
        _chk(load().ora_grid_export_qnnn(self._h, out.ctypes.data))
        return out

    def wall_mask(self):
        out = np.empty(self.N, np.uint8)
        _chk(load().ora_grid_wall_mask(self._h, out.ctypes.data))
        return out

    def compute_derivatives(self, f, nthreads=1):
        f = np.ascontiguousarray(f, np.float64)
        out = np.empty((self.dim, self.N), np.float64)
        _chk(load().ora_compute_derivatives(self._h, _dp(f), _dp(out), nthreads))
        return out

    def compute_derivatives_range(self, f, out, first, count, nthreads=1):
        """compute_derivatives over the nodes [first, first + count) only; out (D, N) updated there."""
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == self.dim * self.N
        _chk(load().ora_compute_derivatives_range(self._h, _dp(np.ascontiguousarray(f, np.float64)), _dp(out), int(first), int(count),
                                                  nthreads))

    def reinit_stage_range(self, phi_np1, phi_0, phi_n, limit_high, limit_low, dd0, ddc, first, count, nthreads=1):
        """One reinitialize_one_iteration stage over the nodes [first, first + count) only (dd0/ddc None: first
        order in space); phi_np1 (N) updated there."""
        assert phi_np1.dtype == np.float64 and phi_np1.flags.c_contiguous and phi_np1.size == self.N
        f = lambda a: None if a is None else np.ascontiguousarray(a, np.float64)
        _chk(load().ora_reinit_stage_range(self._h, _dp(phi_np1), _dp(f(phi_0)), _dp(f(phi_n)), float(limit_high), float(limit_low),
                                           _dp(f(dd0)), _dp(f(ddc)), int(first), int(count), nthreads))

    def reinitialize(self, phi, order_space=2, order_pseudotime=2, limit_high=np.finfo(np.float64).max,
                     limit_low=-np.finfo(np.float64).max, iterations=50, nthreads=1):
        """In place on a float64 numpy array."""
        assert phi.dtype == np.float64 and phi.flags.c_contiguous and phi.size == self.N
        _chk(load().ora_reinitialize(self._h, _dp(phi), order_space, order_pseudotime, limit_high, limit_low, iterations, nthreads))

    def reinitialize_with_mask(self, phi, mask, order_space=2, order_pseudotime=2, limit_high=np.finfo(np.float64).max,
                               limit_low=-np.finfo(np.float64).max, iterations=50, nthreads=1):
        """In place; nodes where mask == 0 are not updated."""
        assert phi.dtype == np.float64 and phi.flags.c_contiguous and phi.size == self.N
        mask = np.ascontiguousarray(mask, np.float64)
        _chk(load().ora_reinitialize_masked(self._h, _dp(phi), _dp(mask), order_space, order_pseudotime, limit_high, limit_low,
                                            iterations, nthreads))

    def advect_in_normal_direction(self, vn, phi, dt, vn_np1=None, phi_dd=None, nthreads=1):
        _chk(load().ora_advect_in_normal_direction(self._h, _dp(vn), _dp(vn_np1), _dp(phi), dt, _dp(phi_dd), nthreads))

    def advect_stage_range(self, vn, dt, dd, phi_n, phi_np1, first, count, nthreads=1):
        """One normal-advection sweep over the nodes [first, first + count); phi_np1 (N,) updated there."""
        assert phi_np1.dtype == np.float64 and phi_np1.flags.c_contiguous and phi_np1.size == self.N
        _chk(load().ora_advect_stage_range(self._h, _dp(np.ascontiguousarray(vn, np.float64)), float(dt),
                                           _dp(np.ascontiguousarray(dd, np.float64)), _dp(np.ascontiguousarray(phi_n, np.float64)),
                                           _dp(phi_np1), int(first), int(count), nthreads))

    def advect_cfl_dt(self, vn):
        out = C.c_double()
        _chk(load().ora_advect_cfl_dt(self._h, _dp(np.ascontiguousarray(vn, np.float64)), C.byref(out)))
        return out.value

    # ---- first derivatives, normals, curvature ------------------------------------------------
    def first_derivatives(self, f, nthreads=1):
        f = np.ascontiguousarray(f, np.float64)
        out = np.empty((self.dim, self.N), np.float64)
        _chk(load().ora_first_derivatives(self._h, _dp(f), _dp(out), nthreads))
        return out

    def compute_normals(self, phi, nthreads=1):
        phi = np.ascontiguousarray(phi, np.float64)
        out = np.empty((self.dim, self.N), np.float64)
        _chk(load().ora_compute_normals(self._h, _dp(phi), _dp(out), nthreads))
        return out

    def mean_curvature_from_normals(self, normals, nthreads=1):
        nrm = np.ascontiguousarray(normals, np.float64)
        out = np.empty(self.N, np.float64)
        _chk(load().ora_mean_curvature_from_normals(self._h, _dp(nrm), _dp(out), nthreads))
        return out

    def normals_and_mean_curvature(self, phi, nthreads=1):
        phi = np.ascontiguousarray(phi, np.float64)
        nrm = np.empty((self.dim, self.N), np.float64)
        kappa = np.empty(self.N, np.float64)
        _chk(load().ora_normals_and_mean_curvature(self._h, _dp(phi), _dp(nrm), _dp(kappa), nthreads))
        return nrm, kappa

    def extend_over_interface_tvd(self, phi, q, iterations=20, order=2, band_use=-np.finfo(np.float64).max,
                                  band_extend=np.finfo(np.float64).max, normals=None, mask=None, nthreads=1,
                                  use_nonzero_guess=False, q_n=None, q_nn=None):
        """In place on q (float64, node order); q_n / q_nn (optional, in place): the normal derivatives."""
        phi = np.ascontiguousarray(phi, np.float64)
        assert q.dtype == np.float64 and q.flags.c_contiguous and q.size == self.N
        for v in (q_n, q_nn):
            assert v is None or (v.dtype == np.float64 and v.flags.c_contiguous and v.size == self.N)
        nrm = None if normals is None else np.ascontiguousarray(normals, np.float64)
        msk = None if mask is None else np.ascontiguousarray(mask, np.float64)
        _chk(load().ora_extend_over_interface_ex(self._h, _dp(phi), _dp(msk), _dp(q), int(iterations), int(order), float(band_use),
                                                 float(band_extend), _dp(nrm), int(bool(use_nonzero_guess)), _dp(q_n), _dp(q_nn),
                                                 nthreads))

    def extend_from_interface_to_whole_domain_tvd(self, phi, qi, iterations=20, mask=None, band_zero=2.0, band_smooth=10.0,
                                                  grad_phi=None, method=4, nthreads=1):
        """Returns q (float64, node order): qi's interface values extended along the normals."""
        phi = np.ascontiguousarray(phi, np.float64)
        qi = np.ascontiguousarray(qi, np.float64)
        q = np.empty(self.N, np.float64)
        msk = None if mask is None else np.ascontiguousarray(mask, np.float64)
        g = None if grad_phi is None else np.ascontiguousarray(grad_phi, np.float64)
        _chk(load().ora_extend_from_interface(self._h, _dp(phi), _dp(qi), _dp(q), int(iterations), _dp(msk), float(band_zero),
                                              float(band_smooth), _dp(g), int(method), nthreads))
        return q

    def extend_from_interface_to_whole_domain_tvd_cf(self, phi, qi, cf, iterations=20, grad_phi=None, nthreads=1):
        """cf(node, dir, dist) -> interface value, called once per crossing in the reference's order."""
        phi = np.ascontiguousarray(phi, np.float64)
        qi = np.ascontiguousarray(qi, np.float64)
        q = np.empty(self.N, np.float64)
        g = None if grad_phi is None else np.ascontiguousarray(grad_phi, np.float64)
        proto = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_double),
                            C.POINTER(C.c_double))

        def tramp(ctx, count, nodes, dirs, dists, values):
            for k in range(count):
                values[k] = float(cf(int(nodes[k]), int(dirs[k]), float(dists[k])))
            return 0

        cb = proto(tramp)
        _chk(load().ora_extend_from_interface_cf(self._h, _dp(phi), _dp(qi), _dp(q), int(iterations), C.cast(cb, C.c_void_p), None,
                                                 _dp(g), nthreads))
        return q

    # ---- node interpolation and the semi-Lagrangian step ------------------------------------
    def interpolate(self, method, F, xyz, Fdd=None, nthreads=1):
        """F: (nf, N) or (N,); xyz: (np, dim); Fdd: (nf, dim, N) or None. Returns (nf, np) or (np,)."""
        F = np.ascontiguousarray(F, np.float64)
        single = F.ndim == 1
        F2 = F.reshape(1, -1) if single else F
        pts = np.ascontiguousarray(xyz, np.float64).reshape(-1, self.dim)
        dd = None if Fdd is None else np.ascontiguousarray(Fdd, np.float64)
        out = np.empty((F2.shape[0], len(pts)), np.float64)
        _chk(load().ora_interpolate(self._h, int(method), F2.shape[0], _dp(F2), _dp(dd), len(pts), _dp(pts), _dp(out), nthreads))
        return out[0] if single else out

    def locate(self, xyz):
        pts = np.ascontiguousarray(xyz, np.float64).reshape(-1, self.dim)
        out = np.empty(len(pts), np.int32)
        _chk(load().ora_locate(self._h, len(pts), _dp(pts), out.ctypes.data))
        return out

    def sl_advect(self, xyz_np1, dt, v, phi, vdd=None, phi_dd=None, velo_method=4, phi_method=4, nthreads=1):
        pts = np.ascontiguousarray(xyz_np1, np.float64).reshape(-1, self.dim)
        v = np.ascontiguousarray(v, np.float64)
        phi = np.ascontiguousarray(phi, np.float64)
        vdd = None if vdd is None else np.ascontiguousarray(vdd, np.float64)
        phi_dd = None if phi_dd is None else np.ascontiguousarray(phi_dd, np.float64)
        out = np.empty(len(pts), np.float64)
        _chk(load().ora_sl_advect(self._h, len(pts), _dp(pts), float(dt), _dp(v), _dp(vdd), _dp(phi), _dp(phi_dd), int(velo_method),
                                  int(phi_method), _dp(out), nthreads))
        return out

    def sl_advect2(self, grid_nm1, xyz_np1, dt_nm1, dt_n, vnm1, vn, phi, vnm1_dd=None, vn_dd=None, phi_dd=None, velo_method=4, phi_method=4,
                   nthreads=1):
        """Two-velocity second-order step: vn, phi on this grid (time n), vnm1 on grid_nm1, departure from the
        points xyz_np1 (the new grid's nodes)."""
        pts = np.ascontiguousarray(xyz_np1, np.float64).reshape(-1, self.dim)
        f = lambda a: None if a is None else np.ascontiguousarray(a, np.float64)
        out = np.empty(len(pts), np.float64)
        _chk(load().ora_sl_advect2(self._h, grid_nm1._h, len(pts), _dp(pts), float(dt_nm1), float(dt_n), _dp(f(vnm1)), _dp(f(vnm1_dd)),
                                   _dp(f(vn)), _dp(f(vn_dd)), _dp(f(phi)), _dp(f(phi_dd)), int(velo_method), int(phi_method),
                                   _dp(out), nthreads))
        return out

    def sl_advect_vortex(self, xyz_np1, dt, vscale, phi, phi_dd=None, phi_method=4, nthreads=1):
        pts = np.ascontiguousarray(xyz_np1, np.float64).reshape(-1, self.dim)
        phi = np.ascontiguousarray(phi, np.float64)
        phi_dd = None if phi_dd is None else np.ascontiguousarray(phi_dd, np.float64)
        out = np.empty(len(pts), np.float64)
        _chk(load().ora_sl_advect_vortex(self._h, len(pts), _dp(pts), float(dt), float(vscale), _dp(phi), _dp(phi_dd),
                                         int(phi_method), _dp(out), nthreads))
        return out


def vortex(dim, xyz, vscale=1.0):
    """Single-vortex velocity at points (np, dim) -> (dim, np)."""
    pts = np.ascontiguousarray(xyz, np.float64).reshape(-1, dim)
    out = np.empty((dim, len(pts)), np.float64)
    _chk(load().ora_vortex(dim, len(pts), _dp(pts), float(vscale), _dp(out)))
    return out
