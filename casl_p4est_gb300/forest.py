"""Host grid: the p4est objects parCASL's level-set path reads, built natively (see csrc/forest.hpp).

Python names mirror the parCASL calls a driver makes (examples/reinitialization/main_2d.cpp:157-188):

    forest = my_p4est_brick_new(n_xyz, xyz_min, xyz_max, periodic)     # + my_p4est_new (one root per tree)
    for _ in range(lmax): forest.refine_levelset(shape, lmin, lmax, lip) # my_p4est_refine(refine_levelset_cf)
    forest.build_nodes()                                               # my_p4est_nodes_new
    ngbd = my_p4est_node_neighbors_t(forest); ngbd.init_neighbors()
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def _is_cuda(v) -> bool:
    return hasattr(v, "data_ptr") and getattr(getattr(v, "device", None), "type", "cpu") == "cuda"


class Forest:
    """p4est_t + p4est_nodes_t for one process (brick of trees, non-periodic)."""

    def __init__(self, dim, n_xyz, xyz_min, xyz_max, periodic=None):
        lib = L.load()
        self.dim = int(dim)
        n = (C.c_int * 3)(*(list(n_xyz) + [1] * (3 - len(n_xyz))))
        lo = (C.c_double * 3)(*(list(xyz_min) + [0.0] * (3 - len(xyz_min))))
        hi = (C.c_double * 3)(*(list(xyz_max) + [1.0] * (3 - len(xyz_max))))
        per = (C.c_int * 3)(*((list(periodic) if periodic is not None else [0, 0, 0]) + [0] * 3)[:3])
        h = C.c_void_p()
        L.check(lib.lsg_forest_create(self.dim, n, lo, hi, per, C.byref(h)))
        self._h = h
        self.n_xyz = tuple(n[:3])
        self.xyz_min = tuple(lo[:3])
        self.xyz_max = tuple(hi[:3])
        self.max_lvl_requested = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                L.load().lsg_forest_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    # ---- leaves -------------------------------------------------------------------------------
    @property
    def num_leaves(self) -> int:
        return int(L.load().lsg_forest_num_leaves(self._h))

    def leaves(self):
        n = self.num_leaves
        tree = np.empty(n, np.int32)
        level = np.empty(n, np.int32)
        xyz = np.empty((n, 3), np.int32)
        L.check(L.load().lsg_forest_leaves(self._h, L.i32ptr(tree), L.i32ptr(level), L.i32ptr(xyz)))
        return tree, level, xyz

    def refine(self, tags):
        tags = np.ascontiguousarray(tags, dtype=np.uint8)
        L.check(L.load().lsg_forest_refine(self._h, L.u8ptr(tags), tags.size))

    def coarsen(self, tags):
        tags = np.ascontiguousarray(tags, dtype=np.uint8)
        L.check(L.load().lsg_forest_coarsen(self._h, L.u8ptr(tags), tags.size))

    def tag_levelset(self, shape, min_lvl, max_lvl, lip=1.2, band=0.0):
        kind, params = shape
        params = np.ascontiguousarray(params, np.float64)
        tags = np.empty(self.num_leaves, np.uint8)
        L.check(L.load().lsg_forest_tag_levelset(self._h, min_lvl, max_lvl, lip, band, kind, L.dptr(params), params.size,
                                                 L.u8ptr(tags)))
        return tags

    def refine_levelset(self, shape, min_lvl, max_lvl, lip=1.2, band=0.0, passes=None):
        """Repeated my_p4est_refine(refine_levelset_cf) passes (default: max_lvl passes, as the examples)."""
        kind, params = shape
        params = np.ascontiguousarray(params, np.float64)
        passes = max_lvl if passes is None else passes
        self.max_lvl_requested = max(self.max_lvl_requested, max_lvl)
        L.check(L.load().lsg_forest_refine_levelset(self._h, min_lvl, max_lvl, lip, band, kind, L.dptr(params), params.size,
                                                    passes))

    def copy(self) -> "Forest":
        """p4est_copy: an independent forest with the same leaves (and nodes, if built)."""
        h = C.c_void_p()
        L.check(L.load().lsg_forest_copy(self._h, C.byref(h)))
        c = Forest.__new__(Forest)
        c._h = h
        c.dim, c.n_xyz, c.xyz_min, c.xyz_max = self.dim, self.n_xyz, self.xyz_min, self.xyz_max
        c.max_lvl_requested = self.max_lvl_requested
        return c

    def set_leaves(self, tree, level, xyz):
        """Adopt a complete forest given leaf by leaf in tree-major Morton order (e.g. from p4est)."""
        tree = np.ascontiguousarray(tree, np.int32)
        level = np.ascontiguousarray(level, np.int32)
        xyz3 = np.zeros((len(tree), 3), np.int32)
        xyz = np.asarray(xyz, np.int32).reshape(len(tree), -1)
        xyz3[:, :xyz.shape[1]] = xyz
        L.check(L.load().lsg_forest_set_leaves(self._h, len(tree), L.i32ptr(tree), L.i32ptr(level), L.i32ptr(xyz3)))
        self.max_lvl_requested = max(self.max_lvl_requested, int(level.max()))

    def refine_and_coarsen(self, min_lvl, max_lvl, phi, lip=1.2, band=0.0) -> bool:
        """splitting_criteria_tag_t(min_lvl, max_lvl, lip).refine_and_coarsen(p4est, nodes, phi): one
        coarsening and one refinement pass tagged from the node values phi. Returns whether the grid
        changed; the nodes must be rebuilt. With phi a CUDA tensor the tags are evaluated on the GPU
        (on the tensor's current stream) and only one byte per leaf comes back to the host."""
        if _is_cuda(phi):
            import torch
            if phi.dtype != torch.float64 or not phi.is_contiguous() or phi.numel() != self.num_nodes:
                raise ValueError("phi must be a contiguous float64 tensor with one value per node")
            changed = C.c_int(0)
            L.check(L.load().lsg_forest_refine_and_coarsen_device(self._h, int(min_lvl), int(max_lvl), float(lip), float(band),
                                                                  C.c_void_p(phi.data_ptr()), C.byref(changed),
                                                                  C.c_void_p(torch.cuda.current_stream().cuda_stream)))
            self.max_lvl_requested = max(self.max_lvl_requested, int(max_lvl))
            return bool(changed.value)
        phi = np.ascontiguousarray(phi, np.float64)
        if phi.size != self.num_nodes:
            raise ValueError("phi must hold one value per node")
        changed = C.c_int(0)
        L.check(L.load().lsg_forest_refine_and_coarsen(self._h, int(min_lvl), int(max_lvl), float(lip), float(band), L.dptr(phi),
                                                       C.byref(changed)))
        self.max_lvl_requested = max(self.max_lvl_requested, int(max_lvl))
        return bool(changed.value)

    # ---- nodes --------------------------------------------------------------------------------
    def build_nodes(self, device=False):
        """my_p4est_nodes_new. device=True: the numbering is computed on the GPU (same result) and a
        device copy of the leaves and nodes stays with the forest for node_xyz_device, device tagging and
        level sets built on the device."""
        if device:
            import torch
            L.check(L.load().lsg_forest_build_nodes_device(self._h, C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        else:
            L.check(L.load().lsg_forest_build_nodes(self._h))
        return self

    def node_xyz_device(self):
        """Node coordinates as a (N, dim) float64 CUDA tensor, computed on the GPU."""
        import torch
        out = torch.empty((self.num_nodes, self.dim), dtype=torch.float64, device="cuda")
        L.check(L.load().lsg_forest_node_xyz_device(self._h, C.c_void_p(out.data_ptr()),
                                                    C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        return out

    @property
    def num_nodes(self) -> int:
        n = int(L.load().lsg_forest_num_nodes(self._h))
        if n < 0:
            L.check(L.LSG_ESTATE)
        return n

    def node_xyz(self) -> np.ndarray:
        out = np.empty((self.num_nodes, self.dim), np.float64)
        L.check(L.load().lsg_forest_node_xyz(self._h, L.dptr(out)))
        return out

    def nodes(self):
        n = self.num_nodes
        tree = np.empty(n, np.int32)
        xyz = np.empty((n, 3), np.int32)
        L.check(L.load().lsg_forest_nodes(self._h, L.i32ptr(tree), L.i32ptr(xyz)))
        return tree, xyz

    def local_nodes(self) -> np.ndarray:
        out = np.empty((self.num_leaves, 1 << self.dim), np.int32)
        L.check(L.load().lsg_forest_local_nodes(self._h, L.i32ptr(out)))
        return out

    def sample(self, shape) -> np.ndarray:
        """sample_cf_on_nodes for an analytic shape."""
        kind, params = shape
        params = np.ascontiguousarray(params, np.float64)
        out = np.empty(self.num_nodes, np.float64)
        L.check(L.load().lsg_forest_sample_shape(self._h, kind, L.dptr(params), params.size, L.dptr(out)))
        return out

    def wall_mask(self) -> np.ndarray:
        out = np.empty(self.num_nodes, np.uint8)
        L.check(L.load().lsg_forest_wall_mask(self._h, L.u8ptr(out)))
        return out

    def dxyz_min(self, max_lvl=None):
        """get_dxyz_min (src/my_p4est_utils.cpp:1148-1173) for the splitting criterion's max level."""
        lvl = self.max_lvl_requested if max_lvl is None else max_lvl
        dx = [(self.xyz_max[a] - self.xyz_min[a]) / self.n_xyz[a] / (1 << lvl) for a in range(self.dim)]
        return np.array(dx), min(dx), float(np.sqrt(sum(v * v for v in dx)))


def qnnn_dtype(dim: int) -> np.dtype:
    """numpy layout of one quad_neighbor_nodes_of_node_t record as exported by the library."""
    h = 1 << (dim - 1)
    dt = np.dtype([("node_000", np.int32), ("nb", np.int32, (2 * dim, h)), ("d", np.float64, (2 * dim,)),
                   ("dt", np.float64, (2 * dim, 2 * (dim - 1))), ("inverse_d_max", np.float64)], align=True)
    assert dt.itemsize == L.load().lsg_qnnn_record_bytes(dim), "record layout mismatch"
    return dt


def my_p4est_brick_new(n_xyz, xyz_min, xyz_max, periodic=None) -> Forest:
    return Forest(len(n_xyz), n_xyz, xyz_min, xyz_max, periodic)


class my_p4est_node_neighbors_t:
    """Node neighbourhood of a forest (quad_neighbor_nodes_of_node_t per node)."""

    def __init__(self, forest: Forest):
        if forest.num_nodes <= 0:
            raise ValueError("forest has no nodes")
        self.forest = forest
        self.dim = forest.dim
        self._initialized = False

    def init_neighbors(self):
        self._initialized = True

    def neighbors_are_initialized(self) -> bool:
        return self._initialized

    def get_neighbors(self, first=0, count=None) -> np.ndarray:
        n = self.forest.num_nodes
        count = n - first if count is None else count
        dt = qnnn_dtype(self.dim)
        out = np.zeros(count, dtype=dt)
        L.check(L.load().lsg_forest_export_qnnn(self.forest.handle, first, count, out.ctypes.data_as(C.c_void_p), dt.itemsize))
        return out
