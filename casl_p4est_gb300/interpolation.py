"""Node interpolation and the semi-Lagrangian step on the GPU (FP64).

Mirrors my_p4est_interpolation_nodes_t (src/my_p4est_interpolation_nodes.h:33-103, set_input /
add_point / interpolate) and my_p4est_semi_lagrangian_t::advect_from_n_to_np1
(src/my_p4est_semi_lagrangian.cpp:108-223). Arrays are numpy float64 in node order (host, copied
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
    p4est->user_pointer), used by update_p4est."""

    def __init__(self, forest_np1, ls_n: my_p4est_level_set_t, splitting=None):
        self.forest_np1 = forest_np1
        self.ls_n = ls_n
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

    def advect_from_n_to_np1(self, dt, v, phi_n, vxx=None, phi_xx_n=None, xyz_np1=None):
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

    def update_p4est(self, v, dt, phi, phi_xx=None, vxx=None):
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
