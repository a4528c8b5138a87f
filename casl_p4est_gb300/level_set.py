"""my_p4est_level_set_t on the GPU (src/my_p4est_level_set.h:203-848, reinit + normal advection).

Same method names, argument meaning and error behaviour as the reference class. A "Vec" is a numpy
float64 array in node order (host; copied to the device inside each call) or a CUDA tensor with a
``data_ptr()`` (device-resident; used in place). ``precision`` selects the FP64 path (evaluates the
reference's expressions in the same order) or the mixed FP32/FP64 path.
"""
from __future__ import annotations

import ctypes as C
import sys

import numpy as np

from . import _lib as L
from .forest import my_p4est_node_neighbors_t

DBL_MAX = sys.float_info.max
PRECISIONS = {"fp64": L.LSG_FP64, "mixed": L.LSG_MIXED}


def _is_device(v) -> bool:
    return hasattr(v, "data_ptr") and getattr(getattr(v, "device", None), "type", "cpu") == "cuda"


def _host_f64(v, n, name):
    if not isinstance(v, np.ndarray) or v.dtype != np.float64 or not v.flags.c_contiguous:
        raise TypeError(f"{name} must be a C-contiguous float64 numpy array (or a CUDA tensor)")
    if v.size != n:
        raise ValueError(f"{name} has {v.size} entries, the grid has {n} nodes")
    return v


class my_p4est_level_set_t:
    def __init__(self, ngbd: my_p4est_node_neighbors_t, precision: str = "fp64", device_build: bool = False):
        """device_build: build the node-neighbour tables on the GPU (same results, no host table work)."""
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {list(PRECISIONS)}")
        self.ngbd = ngbd
        self.precision = precision
        self.device_build = bool(device_build)
        self._h = None
        self._build(ngbd)

    def _build(self, ngbd):
        h = C.c_void_p()
        L.check(L.load().lsg_level_set_create_ex(ngbd.forest.handle, L.LSG_BUILD_ON_DEVICE if self.device_build else 0,
                                                 C.byref(h)))
        self._h = h
        self.num_nodes = int(L.load().lsg_level_set_num_nodes(h))
        self.zero_distance_threshold = float(L.load().lsg_level_set_zero_distance_threshold(h))

    def update(self, ngbd: my_p4est_node_neighbors_t):
        """my_p4est_level_set_t::update (src/my_p4est_level_set.h:416-422): rebuild the device tables."""
        self._free()
        self.ngbd = ngbd
        self._build(ngbd)

    def _free(self):
        if self._h is not None and self._h.value:
            L.load().lsg_level_set_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self._free()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr: int | None):
        L.check(L.load().lsg_level_set_set_stream(self._h, C.c_void_p(stream_ptr or 0)))

    @property
    def stream(self) -> int:
        return int(L.load().lsg_level_set_stream(self._h) or 0)

    def _prec(self, precision):
        return PRECISIONS[precision or self.precision]

    # ---- reinitialisation -------------------------------------------------------------------
    def reinitialize_within_range_of_phi_0(self, phi, order_space, order_pseudotime, phi_0_limit_high, phi_0_limit_low,
                                           number_of_iterations, precision=None):
        if order_space not in (1, 2) or order_pseudotime not in (1, 2):
            raise ValueError("my_p4est_level_set_t::reinitialize_within_range_of_phi_0: valid orders of orders of accuracy "
                             "for space and pseudotime are 1 and 2 only!")
        p = self._prec(precision)
        if _is_device(phi):
            L.check(L.load().lsg_reinitialize_device(self._h, C.c_void_p(phi.data_ptr()), order_space, order_pseudotime,
                                                     float(phi_0_limit_high), float(phi_0_limit_low), int(number_of_iterations), p))
        else:
            _host_f64(phi, self.num_nodes, "phi")
            L.check(L.load().lsg_reinitialize(self._h, L.dptr(phi), order_space, order_pseudotime, float(phi_0_limit_high),
                                              float(phi_0_limit_low), int(number_of_iterations), p))

    def reinitialize_1st_order(self, phi, number_of_iterations=50, limit_absolute_value_phi_0=DBL_MAX, precision=None):
        self.reinitialize_within_range_of_phi_0(phi, 1, 1, limit_absolute_value_phi_0, -limit_absolute_value_phi_0,
                                                number_of_iterations, precision)

    def reinitialize_1st_order_above_threshold(self, phi, threshold, number_of_iterations=50, upper_limit_phi_0=DBL_MAX,
                                               precision=None):
        self.reinitialize_within_range_of_phi_0(phi, 1, 1, upper_limit_phi_0, threshold, number_of_iterations, precision)

    def reinitialize_2nd_order(self, phi, number_of_iterations=50, limit_absolute_value_phi_0=DBL_MAX, precision=None):
        self.reinitialize_within_range_of_phi_0(phi, 2, 2, limit_absolute_value_phi_0, -limit_absolute_value_phi_0,
                                                number_of_iterations, precision)

    def reinitialize_2nd_order_with_mask(self, phi, mask, number_of_masked=0, number_of_iterations=50,
                                         limit_absolute_value_phi_0=DBL_MAX, precision=None):
        """reinitialize_2nd_order_with_mask (src/my_p4est_level_set.h:487-525): nodes where mask == 0 keep
        their value (number_of_masked is the reference's reservation hint and is not needed here)."""
        p = self._prec(precision)
        lim = float(limit_absolute_value_phi_0)
        if _is_device(phi):
            L.check(L.load().lsg_reinitialize_with_mask_device(self._h, C.c_void_p(phi.data_ptr()), C.c_void_p(mask.data_ptr()), 2, 2,
                                                               lim, -lim, int(number_of_iterations), p))
            return
        _host_f64(phi, self.num_nodes, "phi")
        m = _host_f64(np.ascontiguousarray(mask, np.float64), self.num_nodes, "mask")
        L.check(L.load().lsg_reinitialize_with_mask(self._h, L.dptr(phi), L.dptr(m), 2, 2, lim, -lim, int(number_of_iterations), p))

    def reinitialize_2nd_order_above_threshold(self, phi, threshold, number_of_iterations=50, upper_limit_phi_0=DBL_MAX,
                                               precision=None):
        self.reinitialize_within_range_of_phi_0(phi, 2, 2, upper_limit_phi_0, threshold, number_of_iterations, precision)

    def reinitialize_2nd_order_time_1st_order_space(self, phi, number_of_iterations=50, limit_absolute_value_phi_0=DBL_MAX,
                                                    precision=None):
        self.reinitialize_within_range_of_phi_0(phi, 1, 2, limit_absolute_value_phi_0, -limit_absolute_value_phi_0,
                                                number_of_iterations, precision)

    def reinitialize_1st_order_time_2nd_order_space(self, phi, number_of_iterations=50, limit_absolute_value_phi_0=DBL_MAX,
                                                    precision=None):
        self.reinitialize_within_range_of_phi_0(phi, 2, 1, limit_absolute_value_phi_0, -limit_absolute_value_phi_0,
                                                number_of_iterations, precision)

    # ---- normal-direction advection ----------------------------------------------------------
    def advect_in_normal_direction(self, vn, phi, dt=None, phi_xx=None, vn_np1=None, precision=None):
        """Forms of the reference (src/my_p4est_level_set.h:632-659):
        - advect_in_normal_direction(vn_cf, phi[, phi_xx]) with vn a callable of node coordinates:
          dt from CFL 0.8, returned;
        - advect_in_normal_direction(vn, phi, dt[, phi_xx]) with node-sampled vn: returns dt;
        - advect_in_normal_direction(vn, phi, dt, vn_np1=...) two-velocity form.
        phi_xx, if given, is a (dim, N) float64 array overwritten with the derivatives of the
        intermediate stage, as the reference does."""
        p = self._prec(precision)
        lib = L.load()
        if callable(vn):
            xyz = self.ngbd.forest.node_xyz()
            vn_arr = np.ascontiguousarray(vn(xyz), dtype=np.float64)
            dtv = C.c_double()
            L.check(lib.lsg_advect_cfl_dt(self._h, L.dptr(vn_arr), C.byref(dtv)))
            self.advect_in_normal_direction(vn_arr, phi, dtv.value, phi_xx=phi_xx, precision=precision)
            return dtv.value
        if dt is None:
            raise ValueError("advect_in_normal_direction: dt is required with a node-sampled velocity")
        if _is_device(phi):
            L.check(lib.lsg_advect_in_normal_direction_device(
                self._h, C.c_void_p(vn.data_ptr()), C.c_void_p(vn_np1.data_ptr() if vn_np1 is not None else 0),
                C.c_void_p(phi.data_ptr()), float(dt), C.c_void_p(phi_xx.data_ptr() if phi_xx is not None else 0), p))
            return dt
        n = self.num_nodes
        _host_f64(phi, n, "phi")
        _host_f64(vn, n, "vn")
        if vn_np1 is not None:
            _host_f64(vn_np1, n, "vn_np1")
        if phi_xx is not None:
            if not (isinstance(phi_xx, np.ndarray) and phi_xx.dtype == np.float64 and phi_xx.flags.c_contiguous
                    and phi_xx.size == self.ngbd.dim * n):
                raise TypeError("phi_xx must be a C-contiguous float64 array of shape (dim, N)")
        L.check(lib.lsg_advect_in_normal_direction(self._h, L.dptr(vn), L.dptr(vn_np1) if vn_np1 is not None else None,
                                                   L.dptr(phi), float(dt), L.dptr(phi_xx) if phi_xx is not None else None, p))
        return dt

    def compute_derivatives(self, phi) -> np.ndarray:
        """second_derivatives_central of phi: returns (dim, N) (a CUDA tensor for a CUDA tensor phi)."""
        n = self.num_nodes
        if _is_device(phi):
            out = phi.new_empty((self.ngbd.dim, n))
            L.check(L.load().lsg_second_derivatives_device(self._h, C.c_void_p(phi.data_ptr()), C.c_void_p(out.data_ptr())))
            return out
        _host_f64(phi, n, "phi")
        out = np.empty((self.ngbd.dim, n), np.float64)
        L.check(L.load().lsg_second_derivatives(self._h, L.dptr(phi), L.dptr(out)))
        return out

    # ---- first derivatives, normals, curvature (FP64) ----------------------------------------------
    def first_derivatives_central(self, f) -> np.ndarray:
        """Gradient of f, (dim, N) (my_p4est_node_neighbors_t::first_derivatives_central)."""
        f = _host_f64(np.ascontiguousarray(f, np.float64), self.num_nodes, "f")
        out = np.empty((self.ngbd.dim, self.num_nodes), np.float64)
        L.check(L.load().lsg_first_derivatives(self._h, L.dptr(f), L.dptr(out)))
        return out

    def compute_normals(self, phi) -> np.ndarray:
        phi = _host_f64(np.ascontiguousarray(phi, np.float64), self.num_nodes, "phi")
        out = np.empty((self.ngbd.dim, self.num_nodes), np.float64)
        L.check(L.load().lsg_compute_normals(self._h, L.dptr(phi), L.dptr(out)))
        return out

    def compute_mean_curvature(self, normals) -> np.ndarray:
        nrm = np.ascontiguousarray(normals, np.float64)
        if nrm.size != self.ngbd.dim * self.num_nodes:
            raise ValueError("normals must be (dim, N)")
        out = np.empty(self.num_nodes, np.float64)
        L.check(L.load().lsg_compute_mean_curvature(self._h, L.dptr(nrm), L.dptr(out)))
        return out

    def compute_normals_and_mean_curvature(self, phi):
        phi = _host_f64(np.ascontiguousarray(phi, np.float64), self.num_nodes, "phi")
        nrm = np.empty((self.ngbd.dim, self.num_nodes), np.float64)
        kappa = np.empty(self.num_nodes, np.float64)
        L.check(L.load().lsg_compute_normals_and_mean_curvature(self._h, L.dptr(phi), L.dptr(nrm), L.dptr(kappa)))
        return nrm, kappa

    def extend_Over_Interface_TVD(self, phi, q, iterations=20, order=2, band_use=-DBL_MAX, band_extend=DBL_MAX,
                                  normal=None, mask=None, bc=None, use_nonzero_guess=False, q_n=None, q_nn=None):
        """Extend q (updated in place) from phi < 0 (or mask < 0) along the normals (FP64). normal: (dim, N).
        q_n / q_nn (optional, N each, in place): starting guesses where no normal derivative can be
        computed, and on return the extended first / second normal derivatives. bc (boundary conditions of
        the Poisson solvers) is not supported."""
        if order not in (0, 1, 2):
            raise ValueError("[CASL_ERROR]: my_p4est_level_set_t->extend_Over_Interface_TVD: order must be 0, 1 or 2.")
        if bc is not None:
            raise ValueError("extend_Over_Interface_TVD: boundary conditions are not supported")
        n = self.num_nodes
        if _is_device(phi):
            ptr = lambda t: None if t is None else C.c_void_p(t.data_ptr())
            L.check(L.load().lsg_extend_over_interface_tvd_ex_device(self._h, ptr(phi), ptr(q), int(iterations), int(order),
                                                                     float(band_use), float(band_extend), ptr(normal), ptr(mask),
                                                                     int(bool(use_nonzero_guess)), ptr(q_n), ptr(q_nn)))
            return
        phi = _host_f64(np.ascontiguousarray(phi, np.float64), n, "phi")
        _host_f64(q, n, "q")
        for v, name in ((q_n, "q_n"), (q_nn, "q_nn")):
            if v is not None:
                _host_f64(v, n, name)
        nrm = None if normal is None else np.ascontiguousarray(normal, np.float64)
        msk = None if mask is None else _host_f64(np.ascontiguousarray(mask, np.float64), n, "mask")
        opt = lambda a: L.dptr(a) if a is not None else None
        L.check(L.load().lsg_extend_over_interface_tvd_ex(self._h, L.dptr(phi), L.dptr(q), int(iterations), int(order), float(band_use),
                                                          float(band_extend), opt(nrm), opt(msk), int(bool(use_nonzero_guess)),
                                                          opt(q_n), opt(q_nn)))

    interpolation_on_interface = 4  # quadratic_non_oscillatory_continuous_v2 (src/my_p4est_level_set.h:389)

    def set_interpolation_on_interface(self, method):
        """set_interpolation_on_interface (src/my_p4est_level_set.h:843)."""
        if int(method) not in range(5):
            raise ValueError("unknown interpolation_method")
        self.interpolation_on_interface = int(method)

    def extend_from_interface_to_whole_domain_TVD(self, phi, q_interface, q=None, iterations=20, mask=None, band_zero=2.0,
                                                  band_smooth=10.0, cf=None, grad_phi_in=None):
        """q = the interface values of q_interface extended in the normal direction on both sides (FP64).

        q_interface: (N,) or (nfields, N) (the reference's blocksize, components as blocks); q: output of the
        same shape (allocated and returned when None; must not overlap q_interface); grad_phi_in: (dim, N).
        cf: the interface values given by the caller instead of interpolated, as a vectorised function
        cf(nodes, dirs, dists) -> values over the crossing grid lines (host arrays, one field, no mask)."""
        if cf is not None:
            if mask is not None:
                raise ValueError("No mask and cf simultaneously at the moment")
            n = self.num_nodes
            phi_h = _host_f64(np.ascontiguousarray(phi, np.float64), n, "phi")
            qi = _host_f64(np.ascontiguousarray(q_interface, np.float64).reshape(-1), n, "q_interface")
            out = np.empty(n, np.float64) if q is None else q
            _host_f64(out, n, "q")
            g = None if grad_phi_in is None else np.ascontiguousarray(grad_phi_in, np.float64)
            failure = []

            def tramp(ctx, count, nodes, dirs, dists, values):
                try:
                    nd = np.ctypeslib.as_array(nodes, shape=(count,)).copy()
                    dr = np.ctypeslib.as_array(dirs, shape=(count,)).copy()
                    ds = np.ctypeslib.as_array(dists, shape=(count,)).copy()
                    np.ctypeslib.as_array(values, shape=(count,))[:] = np.asarray(cf(nd, dr, ds), np.float64).reshape(count)
                    return 0
                except Exception as e:
                    failure.append(e)
                    return 1

            cb = L.INTERFACE_VALUES_FN(tramp)
            code = L.load().lsg_extend_from_interface_to_whole_domain_tvd_cf(self._h, L.dptr(phi_h), L.dptr(qi), L.dptr(out),
                                                                             int(iterations), C.cast(cb, C.c_void_p), None,
                                                                             L.dptr(g) if g is not None else None)
            if failure:
                raise failure[0]
            L.check(code)
            return out
        if _is_device(phi):
            if q is None:
                q = q_interface.new_empty(q_interface.shape)
            nf = 1 if q_interface.dim() == 1 else int(q_interface.shape[0])
            ptr = lambda t: None if t is None else C.c_void_p(t.data_ptr())
            L.check(L.load().lsg_extend_from_interface_to_whole_domain_tvd_device(
                self._h, ptr(phi), ptr(q_interface), ptr(q), nf, int(iterations), ptr(mask), float(band_zero), float(band_smooth),
                ptr(grad_phi_in), self.interpolation_on_interface))
            return q
        n = self.num_nodes
        phi = _host_f64(np.ascontiguousarray(phi, np.float64), n, "phi")
        qi = np.ascontiguousarray(q_interface, np.float64)
        nf = 1 if qi.ndim == 1 else qi.shape[0]
        if qi.size != nf * n:
            raise ValueError(f"q_interface has {qi.size} entries, expected {nf} x {n}")
        out = np.empty_like(qi) if q is None else q
        if not (isinstance(out, np.ndarray) and out.dtype == np.float64 and out.flags.c_contiguous and out.size == qi.size):
            raise TypeError("q must be a C-contiguous float64 numpy array shaped like q_interface")
        msk = None if mask is None else _host_f64(np.ascontiguousarray(mask, np.float64), n, "mask")
        g = None if grad_phi_in is None else np.ascontiguousarray(grad_phi_in, np.float64)
        L.check(L.load().lsg_extend_from_interface_to_whole_domain_tvd(
            self._h, L.dptr(phi), L.dptr(qi), L.dptr(out), nf, int(iterations), L.dptr(msk) if msk is not None else None,
            float(band_zero), float(band_smooth), L.dptr(g) if g is not None else None, self.interpolation_on_interface))
        return out

    def band_linf(self, a, b, band):
        """FP64 max |a - b| over |b| < band on the device (CUDA tensors); returns (value, band node count)."""
        if not (_is_device(a) and _is_device(b)):
            raise TypeError("band_linf takes CUDA tensors")
        out = C.c_double()
        cnt = C.c_int64()
        L.check(L.load().lsg_band_linf_device(self._h, C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), float(band),
                                              C.byref(out), C.byref(cnt)))
        return out.value, cnt.value

    def interface_location_error(self, a, b):
        """FP64 max distance between the zero crossings of a and b along the grid edges b cuts (CUDA tensors);
        returns (value, cut edges, edges a does not cut)."""
        if not (_is_device(a) and _is_device(b)):
            raise TypeError("interface_location_error takes CUDA tensors")
        out = C.c_double()
        edges = C.c_int64()
        mis = C.c_int64()
        L.check(L.load().lsg_interface_location_error_device(self._h, C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
                                                             C.byref(out), C.byref(edges), C.byref(mis)))
        return out.value, edges.value, mis.value

    def table_stats(self):
        """Sizes of the mixed tables: nodes, regular, uniform, irregular, extended set, classes, corrections."""
        out = np.zeros(7, np.int64)
        L.check(L.load().lsg_level_set_table_stats(self._h, out.ctypes.data_as(C.POINTER(C.c_int64))))
        keys = ("nodes", "regular", "uniform", "irregular", "extended_regular", "classes", "corrections")
        return {k: int(v) for k, v in zip(keys, out)}

    # ---- launch shape of the mixed stage -----------------------------------------------------------
    def autotune(self, phi, trials=3):
        """Time candidate launch shapes of the mixed stage on phi (host) and keep the fastest."""
        return _autotune(self._h, phi, trials)

    @property
    def stage_config(self):
        return _stage_config(self._h)

    @stage_config.setter
    def stage_config(self, cfg):
        _set_stage_config(self._h, cfg)

    def set_wait_limit(self, cycles=0):
        """Bound of the bulk-copy stage kernel's waits in SM clock cycles (0: the default, about a second).
        A wait that runs out makes the call raise LsgTimeout; the next call starts clean."""
        L.check(L.load().lsg_level_set_set_wait_limit(self._h, int(cycles)))

    def perturb_level_set_function(self, phi, epsilon):
        _host_f64(phi, self.num_nodes, "phi")
        L.check(L.load().lsg_perturb_level_set_function(self._h, L.dptr(phi), float(epsilon)))


def _cfg_dict(cfg):
    return {"threads_per_block": int(cfg[0]), "uniform_blocks": int(cfg[1]), "regular_blocks": int(cfg[2]),
            "uniform_depth": int(cfg[3]), "window_halo": int(cfg[4]), "streams": int(cfg[5]),
            "priority": int(cfg[6])}


def _autotune(handle, phi, trials):
    phi = np.ascontiguousarray(phi, np.float64)
    cfg = np.zeros(7, np.int32)
    L.check(L.load().lsg_level_set_autotune(handle, L.dptr(phi), int(trials), L.i32ptr(cfg)))
    return _cfg_dict(cfg)


def _stage_config(handle):
    cfg = np.zeros(7, np.int32)
    L.check(L.load().lsg_level_set_stage_config(handle, L.i32ptr(cfg)))
    return _cfg_dict(cfg)


def _set_stage_config(handle, cfg):
    arr = np.array([cfg["threads_per_block"], cfg["uniform_blocks"], cfg["regular_blocks"], cfg.get("uniform_depth", 5),
                    cfg.get("window_halo", 512), cfg.get("streams", 2), cfg.get("priority", 2)], np.int32)
    L.check(L.load().lsg_level_set_set_stage_config(handle, L.i32ptr(arr)))


class my_p4est_level_set_batch_t:
    """Many level-set fields on separate grids (same dimension and tree size) reinitialised together.

    The grids' tables are concatenated on the device; reinitialize_2nd_order runs every stage kernel
    once over all grids, grid k for its own iteration count, the loop captured as a CUDA graph."""

    def __init__(self, forests, device_build: bool = False):
        """device_build: build the grids' tables on the GPU (same results, no host table work)."""
        self.forests = list(forests)  # kept alive: the batch borrows them
        arr = (C.c_void_p * len(self.forests))(*[f.handle.value for f in self.forests])
        h = C.c_void_p()
        L.check(L.load().lsg_batch_create_ex(len(self.forests), C.cast(arr, C.POINTER(C.c_void_p)),
                                             L.LSG_BUILD_ON_DEVICE if device_build else 0, C.byref(h)))
        self._h = h
        self.count = int(L.load().lsg_batch_count(h))
        off = np.zeros(self.count + 1, np.int64)
        L.check(L.load().lsg_batch_offsets(h, off.ctypes.data_as(C.POINTER(C.c_int64))))
        self.offsets = off
        self.num_nodes = int(off[-1])

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                L.load().lsg_level_set_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr):
        L.check(L.load().lsg_level_set_set_stream(self._h, C.c_void_p(stream_ptr or 0)))

    def split(self, phi):
        return [phi[self.offsets[k]:self.offsets[k + 1]] for k in range(self.count)]

    def concat(self, phis):
        return np.ascontiguousarray(np.concatenate([np.asarray(p, np.float64) for p in phis]))

    def reinitialize_2nd_order(self, phi, number_of_iterations=50, use_graph=True):
        """phi: concatenated float64 host array (updated in place) or CUDA tensor; number_of_iterations:
        one count for all grids or one per grid."""
        its = np.full(self.count, number_of_iterations, np.int32) if np.isscalar(number_of_iterations) else \
            np.ascontiguousarray(number_of_iterations, np.int32)
        if its.size != self.count:
            raise ValueError("one iteration count per grid is required")
        if _is_device(phi):
            L.check(L.load().lsg_batch_reinitialize_device(self._h, C.c_void_p(phi.data_ptr()), L.i32ptr(its), int(use_graph)))
            return
        _host_f64(phi, self.num_nodes, "phi")
        L.check(L.load().lsg_batch_reinitialize(self._h, L.dptr(phi), L.i32ptr(its), int(use_graph)))

    def autotune(self, phi, trials=3):
        return _autotune(self._h, phi, trials)

    @property
    def stage_config(self):
        return _stage_config(self._h)

    @stage_config.setter
    def stage_config(self, cfg):
        _set_stage_config(self._h, cfg)
