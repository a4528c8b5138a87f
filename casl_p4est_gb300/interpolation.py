"""Node interpolation and the semi-Lagrangian step on the GPU (FP64).

Mirrors my_p4est_interpolation_nodes_t (src/my_p4est_interpolation_nodes.h:33-103, set_input /
add_point / interpolate) and my_p4est_semi_lagrangian_t::advect_from_n_to_np1 / update_p4est, with one
velocity (src/my_p4est_semi_lagrangian.cpp:108-223, 321-529) and with two (:225-319, 779-939). Arrays are numpy float64 in node order (host, copied
inside each call) or CUDA tensors (device-resident).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .level_set import _is_device, my_p4est_level_set_t

# interpolation_method, src/my_p4est_utils.h:332-338
linear = 0
quadratic = 1
quadratic_non_oscillatory = 2
quadratic_non_oscillatory_continuous_v1 = 3
quadratic_non_oscillatory_continuous_v2 = 4
METHODS = (linear, quadratic, quadratic_non_oscillatory, quadratic_non_oscillatory_continuous_v1,
           quadratic_non_oscillatory_continuous_v2)


def _ptr(a):
    if a is None:
        return None
    if _is_device(a):
        return C.c_void_p(a.data_ptr())
    return L.dptr(a)


def _f64(a, name, size=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if size is not None and a.size != size:
        raise ValueError(f"{name} has {a.size} entries, expected {size}")
    return a


class my_p4est_interpolation_nodes_t:
    """Interpolation of node fields of one grid at arbitrary points.

    ``ls`` is the grid's my_p4est_level_set_t (it owns the device image of the node neighbours)."""

    def __init__(self, ls: my_p4est_level_set_t):
        self.ls = ls
        self.dim = ls.ngbd.dim
        self.clear()
        self._F = None

    def clear(self):
        self._idx = []
        self._pts = []

    def add_point(self, node_idx_on_output, xyz):
        self._idx.append(int(node_idx_on_output))
        self._pts.append(np.asarray(xyz, np.float64).reshape(self.dim))

    def add_points(self, xyz):
        """Vectorised add_point for points 0..np-1 (xyz: (np, dim))."""
        xyz = np.asarray(xyz, np.float64).reshape(-1, self.dim)
        base = len(self._idx)
        self._idx.extend(range(base, base + len(xyz)))
        self._pts.extend(xyz)

    def set_input(self, F, method, Fxxyyzz=None):
        """F: (N,) or (nf, N); Fxxyyzz: (dim, N) or (nf, dim, N) second derivatives, or None to compute them."""
        if method not in METHODS:
            raise ValueError("unknown interpolation_method")
        self._F, self._Fdd, self.method = F, Fxxyyzz, method

    def interpolate(self, out=None):
        if self._F is None:
            raise RuntimeError("set_input was not called")
        pts = np.ascontiguousarray(np.array(self._pts, np.float64).reshape(-1, self.dim))
        vals = self.interpolate_points(pts, self._F, self.method, self._Fdd)
        if out is None:
            out = np.empty(vals.shape[:-1] + (max(self._idx) + 1 if self._idx else 0,), np.float64)
        out[..., np.asarray(self._idx, np.int64)] = vals
        return out

    def interpolate_points(self, xyz, F, method, Fdd=None):
        """Direct form: F (N,) or (nf, N) host arrays at points (np, dim); returns (np,) or (nf, np)."""
        N = self.ls.num_nodes
        F = _f64(F, "F")
        single = F.ndim == 1
        F2 = F.reshape(-1, N)
        nf = F2.shape[0]
        pts = _f64(xyz, "xyz").reshape(-1, self.dim)
        dd = None if (Fdd is None or method == linear) else _f64(Fdd, "Fdd", nf * self.dim * N)
        out = np.empty((nf, len(pts)), np.float64)
        L.check(L.load().lsg_interpolate_nodes(self.ls.handle, L.dptr(pts), len(pts), L.dptr(F2), nf, _ptr(dd), int(method),
                                               L.dptr(out)))
        return out[0] if single else out

    def interpolate_device(self, xyz, F, nf, method, out, Fdd=None):
        """Device form: CUDA tensors xyz (np*dim), F (nf*N), out (nf*np), Fdd (nf*dim*N) or None."""
        npts = xyz.numel() // self.dim
        L.check(L.load().lsg_interpolate_nodes_device(self.ls.handle, _ptr(xyz), npts, _ptr(F), int(nf), _ptr(Fdd), int(method),
                                                      _ptr(out)))


class VortexVelocity:
    """Single-vortex velocity of examples/level_set_advection/main_2d.cpp:116-181, scaled by
    `scale` (the example's direction sign, or cos(pi t/T))."""

    def __init__(self, scale=1.0):
        self.scale = float(scale)


class my_p4est_semi_lagrangian_t:
    """advect_from_n_to_np1 from the grid at time n (ls_n) onto the nodes of the grid at n+1.

    splitting: (min_lvl, max_lvl, lip) of the grid's splitting criterion (the reference reads it from
    p4est->user_pointer), used by update_p4est. ls_nm1: the grid at n-1 (the reference's ngbd_nm1), needed
    by the two-velocity forms."""

    def __init__(self, forest_np1, ls_n: my_p4est_level_set_t, splitting=None, ls_nm1: my_p4est_level_set_t = None):
        self.forest_np1 = forest_np1
        self.ls_n = ls_n
        self.ls_nm1 = ls_nm1
        self.splitting = splitting
        self.dim = ls_n.ngbd.dim
        self.velo_interpolation = quadratic_non_oscillatory_continuous_v2
        self.phi_interpolation = quadratic_non_oscillatory_continuous_v2

    def set_velo_interpolation(self, method):
        if method not in METHODS:
            raise ValueError("unknown interpolation_method")
        self.velo_interpolation = method

    def set_phi_interpolation(self, method):
        if method not in METHODS:
            raise ValueError("unknown interpolation_method")
        self.phi_interpolation = method

    def advect_from_n_to_np1(self, *args, **kw):
        """advect_from_n_to_np1(dt, v, phi_n, vxx=None, phi_xx_n=None, xyz_np1=None), or the two-velocity
        form advect_from_n_to_np1(dt_nm1, dt_n, vnm1, vn, phi_n, vxx_nm1=None, vxx_n=None, phi_xx_n=None,
        xyz_np1=None), told apart as the reference's overloads are, by the arguments: a number in second
        place is dt_n."""
        if len(args) >= 2 and isinstance(args[1], (int, float, np.floating)):
            return self._advect2(*args, **kw)
        return self._advect1(*args, **kw)

    def _advect2(self, dt_nm1, dt_n, vnm1, vn, phi_n, vxx_nm1=None, vxx_n=None, phi_xx_n=None, xyz_np1=None):
        """The two-velocity second-order step (src/my_p4est_semi_lagrangian.cpp:225-319): vn (dim, N_n) and
        phi_n on ls_n's grid, vnm1 (dim, N_nm1) on ls_nm1's; vxx_* (dim, dim, N) and phi_xx_n (dim, N_n) may be
        omitted (computed as the reference's update_p4est does). numpy arrays (copied in and out) or CUDA
        tensors (device-resident; xyz_np1 then a (npts, dim) CUDA tensor, default forest_np1's nodes on the
        device). Returns phi at the nodes of forest_np1."""
        if self.ls_nm1 is None:
            raise ValueError("the two-velocity step needs the grid at n-1 (ls_nm1)")
        lib = L.load()
        d = self.dim
        Nn, Nm = self.ls_n.num_nodes, self.ls_nm1.num_nodes
        if _is_device(phi_n):
            import torch
            xyz = xyz_np1 if xyz_np1 is not None else self.forest_np1.node_xyz_device()
            npts = xyz.shape[0]
            for name, a, n in (("vn", vn, d * Nn), ("vnm1", vnm1, d * Nm), ("phi_n", phi_n, Nn)):
                if not _is_device(a) or a.dtype != torch.float64 or a.numel() != n or not a.is_contiguous():
                    raise ValueError(f"{name} must be a contiguous float64 CUDA tensor of {n} values")
            out = torch.empty(npts, dtype=torch.float64, device=phi_n.device)
            L.check(lib.lsg_semi_lagrangian_advect2_device(self.ls_n.handle, self.ls_nm1.handle, _ptr(xyz), npts, float(dt_nm1),
                                                           float(dt_n), _ptr(vnm1), _ptr(vxx_nm1), _ptr(vn), _ptr(vxx_n),
                                                           _ptr(phi_n), _ptr(phi_xx_n), int(self.velo_interpolation),
                                                           int(self.phi_interpolation), _ptr(out)))
            return out
        xyz = xyz_np1 if xyz_np1 is not None else self.forest_np1.node_xyz()
        xyz = _f64(xyz, "xyz_np1").reshape(-1, d)
        vn = _f64(vn, "vn", d * Nn)
        vnm1 = _f64(vnm1, "vnm1", d * Nm)
        phi_n = _f64(phi_n, "phi_n", Nn)
        vxn = None if vxx_n is None else _f64(vxx_n, "vxx_n", d * d * Nn)
        vxm = None if vxx_nm1 is None else _f64(vxx_nm1, "vxx_nm1", d * d * Nm)
        pdd = None if phi_xx_n is None else _f64(phi_xx_n, "phi_xx_n", d * Nn)
        out = np.empty(len(xyz), np.float64)
        L.check(lib.lsg_semi_lagrangian_advect2(self.ls_n.handle, self.ls_nm1.handle, L.dptr(xyz), len(xyz), float(dt_nm1), float(dt_n),
                                                L.dptr(vnm1), _ptr(vxm), L.dptr(vn), _ptr(vxn), L.dptr(phi_n), _ptr(pdd),
                                                int(self.velo_interpolation), int(self.phi_interpolation), L.dptr(out)))
        return out

    def _advect1(self, dt, v, phi_n, vxx=None, phi_xx_n=None, xyz_np1=None):
        """v: (dim, N_n) node velocities, a VortexVelocity, or a callable velocity(xyz) -> (dim, npts)
        evaluated on the host at points xyz (npts, dim) (the CF overload). Returns phi at the nodes of
        forest_np1 (host arrays)."""
        lib = L.load()
        N = self.ls_n.num_nodes
        xyz = xyz_np1 if xyz_np1 is not None else self.forest_np1.node_xyz()
        xyz = _f64(xyz, "xyz_np1").reshape(-1, self.dim)
        phi_n = _f64(phi_n, "phi_n", N)
        pdd = None if phi_xx_n is None else _f64(phi_xx_n, "phi_xx_n", self.dim * N)
        out = np.empty(len(xyz), np.float64)
        if callable(v) and not isinstance(v, VortexVelocity):
            dim = self.dim
            failure = []

            def trampoline(ctx, npts, pts, vout):
                try:
                    p = np.ctypeslib.as_array(pts, shape=(npts, dim))
                    val = np.asarray(v(p.copy()), np.float64).reshape(dim, npts)
                    np.ctypeslib.as_array(vout, shape=(npts, dim))[:] = val.T
                    return 0
                except Exception as e:  # reported after the call
                    failure.append(e)
                    return 1

            cb = L.VELOCITY_FN(trampoline)
            code = lib.lsg_semi_lagrangian_advect_callback(self.ls_n.handle, L.dptr(xyz), len(xyz), float(dt), cb, None, L.dptr(phi_n),
                                                           _ptr(pdd), int(self.phi_interpolation), L.dptr(out))
            if failure:
                raise failure[0]
            L.check(code)
            return out
        if isinstance(v, VortexVelocity):
            par = np.array([v.scale], np.float64)
            L.check(lib.lsg_semi_lagrangian_advect_cf(self.ls_n.handle, L.dptr(xyz), len(xyz), float(dt), L.LSG_VELOCITY_VORTEX,
                                                      L.dptr(par), 1, L.dptr(phi_n), _ptr(pdd), int(self.phi_interpolation),
                                                      L.dptr(out)))
            return out
        v = _f64(v, "v", self.dim * N)
        vdd = None if vxx is None else _f64(vxx, "vxx", self.dim * self.dim * N)
        L.check(lib.lsg_semi_lagrangian_advect(self.ls_n.handle, L.dptr(xyz), len(xyz), float(dt), L.dptr(v), _ptr(vdd),
                                               L.dptr(phi_n), _ptr(pdd), int(self.velo_interpolation), int(self.phi_interpolation),
                                               L.dptr(out)))
        return out

    def update_p4est(self, *args, **kw):
        """update_p4est(v, dt, phi, phi_xx=None, vxx=None), or the two-velocity form update_p4est(vnm1, vn,
        dt_nm1, dt_n, phi, phi_xx=None, phi_add_refine=None) (a number in third place is dt_nm1)."""
        if len(args) >= 3 and isinstance(args[2], (int, float, np.floating)):
            return self._update_p4est2(*args, **kw)
        return self._update_p4est1(*args, **kw)

    def _update_p4est2(self, vnm1, vn, dt_nm1, dt_n, phi, phi_xx=None, phi_add_refine=None):
        """update_p4est(vnm1, vn, dt_nm1, dt_n, phi, phi_xx, phi_add_refine) (src/my_p4est_semi_lagrangian.cpp:779-939):
        the second derivatives of both velocities (and of phi unless given) once, then the two-velocity step
        onto forest_np1 and splitting_criteria_tag_t::refine_and_coarsen from the advected values (or from
        min(|phi_np1|, |phi_add_refine|), phi_add_refine on grid n interpolated linearly), until the grid
        stops changing. numpy arrays or CUDA tensors. Returns phi at the nodes of the final forest_np1
        (modified in place)."""
        if self.splitting is None:
            raise ValueError("update_p4est needs the splitting criterion (min_lvl, max_lvl, lip)")
        if self.ls_nm1 is None:
            raise ValueError("the two-velocity update_p4est needs the grid at n-1 (ls_nm1)")
        min_lvl, max_lvl, lip = self.splitting
        d = self.dim
        dev = _is_device(phi)
        if dev:
            import torch
            stream = torch.cuda.current_stream().cuda_stream
            self.ls_n.set_stream(stream)
            self.ls_nm1.set_stream(stream)
            stack = lambda xs: torch.stack(xs)
            vn = vn.contiguous()
            vnm1 = vnm1.contiguous()
            row = lambda a, k: a[k].contiguous()
        else:
            stack = np.stack
            vn = _f64(vn, "vn", d * self.ls_n.num_nodes).reshape(d, -1)
            vnm1 = _f64(vnm1, "vnm1", d * self.ls_nm1.num_nodes).reshape(d, -1)
            phi = _f64(phi, "phi", self.ls_n.num_nodes)
            row = lambda a, k: np.ascontiguousarray(a[k])
        vxx_n = stack([self.ls_n.compute_derivatives(row(vn, k)) for k in range(d)])
        vxx_nm1 = stack([self.ls_nm1.compute_derivatives(row(vnm1, k)) for k in range(d)])
        if phi_xx is None:
            phi_xx = self.ls_n.compute_derivatives(phi)
        f = self.forest_np1
        self.iterations = 0
        while True:
            xyz = f.node_xyz_device() if dev else f.node_xyz()
            phi_np1 = self._advect2(dt_nm1, dt_n, vnm1, vn, phi, vxx_nm1=vxx_nm1, vxx_n=vxx_n, phi_xx_n=phi_xx, xyz_np1=xyz)
            self.iterations += 1
            eff = phi_np1
            if phi_add_refine is not None:
                add = my_p4est_interpolation_nodes_t(self.ls_n)
                if dev:
                    extra = torch.empty_like(phi_np1)
                    add.interpolate_device(xyz, phi_add_refine, 1, linear, extra)
                    eff = torch.minimum(extra.abs(), phi_np1.abs())
                else:
                    extra = add.interpolate_points(xyz, phi_add_refine, linear)
                    eff = np.minimum(np.abs(extra), np.abs(phi_np1))
            if not f.refine_and_coarsen(min_lvl, max_lvl, eff, lip=lip):
                return phi_np1
            if dev:
                f.build_nodes(device=True)
            else:
                f.build_nodes()

    def _update_p4est1(self, v, dt, phi, phi_xx=None, vxx=None):
        """update_p4est(v, dt, phi[, phi_xx]) (src/my_p4est_semi_lagrangian.cpp:321-392 for an analytic
        velocity, :394-529 for node velocities): advect phi onto forest_np1, regrid it with
        splitting_criteria_tag_t::refine_and_coarsen from the advected values, and repeat until the grid
        stops changing. Second derivatives on the grid at n are computed once. Returns phi at the
        nodes of the final forest_np1 (which is modified in place)."""
        if self.splitting is None:
            raise ValueError("update_p4est needs the splitting criterion (min_lvl, max_lvl, lip)")
        if _is_device(phi):
            return self._update_p4est_device(v, dt, phi, phi_xx, vxx)
        min_lvl, max_lvl, lip = self.splitting
        N = self.ls_n.num_nodes
        phi = _f64(phi, "phi", N)
        if phi_xx is None and self.phi_interpolation != linear:
            phi_xx = self.ls_n.compute_derivatives(phi)
        if not isinstance(v, VortexVelocity):
            v = _f64(v, "v", self.dim * N).reshape(self.dim, N)
            if vxx is None and self.velo_interpolation != linear:
                vxx = np.stack([self.ls_n.compute_derivatives(np.ascontiguousarray(v[k])) for k in range(self.dim)])
        f = self.forest_np1
        self.iterations = 0
        while True:
            phi_np1 = self.advect_from_n_to_np1(dt, v, phi, vxx=vxx, phi_xx_n=phi_xx)
            self.iterations += 1
            if not f.refine_and_coarsen(min_lvl, max_lvl, phi_np1, lip=lip):
                return phi_np1
            f.build_nodes()

    def _update_p4est_device(self, v, dt, phi, phi_xx, vxx):
        """update_p4est with every field on the GPU (phi a CUDA tensor; v a VortexVelocity or a (dim, N)
        CUDA tensor): node numbering, node coordinates, the semi-Lagrangian step and the refinement tags
        run on the device, on the current torch stream (which ls_n is switched to); only one byte per
        leaf goes to the host for each coarsening/refinement pass. Returns phi at the nodes of the final
        forest_np1 as a CUDA tensor."""
        import torch
        min_lvl, max_lvl, lip = self.splitting
        stream = torch.cuda.current_stream().cuda_stream
        self.ls_n.set_stream(stream)
        lib = L.load()
        N = self.ls_n.num_nodes
        if phi.dtype != torch.float64 or phi.numel() != N:
            raise ValueError("phi must be a float64 tensor with one value per node of grid n")
        phi = phi.contiguous()
        if phi_xx is None and self.phi_interpolation != linear:
            phi_xx = self.ls_n.compute_derivatives(phi)
        vortex = isinstance(v, VortexVelocity)
        if not vortex:
            v = v.contiguous()
            if vxx is None and self.velo_interpolation != linear:
                vxx = torch.stack([self.ls_n.compute_derivatives(v[k].contiguous()) for k in range(self.dim)])
        f = self.forest_np1
        self.iterations = 0
        while True:
            xyz = f.node_xyz_device()
            out = torch.empty(f.num_nodes, dtype=torch.float64, device=phi.device)
            if vortex:
                par = np.array([v.scale], np.float64)
                L.check(lib.lsg_semi_lagrangian_advect_cf_device(self.ls_n.handle, _ptr(xyz), f.num_nodes, float(dt), L.LSG_VELOCITY_VORTEX,
                                                                 L.dptr(par), 1, _ptr(phi), _ptr(phi_xx), int(self.phi_interpolation),
                                                                 _ptr(out)))
            else:
                L.check(lib.lsg_semi_lagrangian_advect_device(self.ls_n.handle, _ptr(xyz), f.num_nodes, float(dt), _ptr(v), _ptr(vxx),
                                                              _ptr(phi), _ptr(phi_xx), int(self.velo_interpolation),
                                                              int(self.phi_interpolation), _ptr(out)))
            self.iterations += 1
            if not f.refine_and_coarsen(min_lvl, max_lvl, out, lip=lip):
                return out
            f.build_nodes(device=True)
