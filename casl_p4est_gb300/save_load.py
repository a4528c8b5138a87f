"""On-disk formats: VTK output (my_p4est_vtk_write_all, src/my_p4est_vtk.h:132-135), PETSc binary
vectors (VecDump, src/my_p4est_save_load.cpp:77-98) and the forest-and-data folder layout of
my_p4est_save_forest_and_data (src/my_p4est_save_load.cpp:350-380): <folder>/<forest_filename> for
the grid (this library's leaf-list format; p4est's own forest format is not written) and
<folder>/<name>.petscbin per group of node vectors, in the PETSc binary format one process writes."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib as L
from .forest import Forest


def _f64_rows(vals, n, what):
    out = []
    for v in vals:
        a = np.ascontiguousarray(v, np.float64).reshape(-1)
        if a.size != n:
            raise ValueError(f"{what} has {a.size} values, expected {n}")
        out.append(a)
    return out


def my_p4est_vtk_write_all(forest: Forest, filename: str, point_data=None, cell_data=None, write_tree=True, binary=False):
    """Write <filename>.pvtu and <filename>.vtu/0000.vtu: nodes as points, leaves as pixels/voxels,
    point_data / cell_data as {name: values} (one value per node / per leaf)."""
    point_data = dict(point_data or {})
    cell_data = dict(cell_data or {})
    pv = _f64_rows(point_data.values(), forest.num_nodes, "point data")
    cv = _f64_rows(cell_data.values(), forest.num_leaves, "cell data")
    pn = (C.c_char_p * max(1, len(pv)))(*[k.encode() for k in point_data])
    cn = (C.c_char_p * max(1, len(cv)))(*[k.encode() for k in cell_data])
    pp = (C.c_void_p * max(1, len(pv)))(*[a.ctypes.data for a in pv])
    cp = (C.c_void_p * max(1, len(cv)))(*[a.ctypes.data for a in cv])
    L.check(L.load().lsg_vtk_write_all(forest.handle, filename.encode(), int(bool(write_tree)), len(pv), pn, pp, len(cv), cn, cp,
                                       int(bool(binary))))


def VecDump(fname: str, vecs, petsc_int64=False):
    """PETSc binary Vec records of the given vectors (one file, in order)."""
    vecs = [np.ascontiguousarray(v, np.float64).reshape(-1) for v in vecs]
    n = vecs[0].size
    if any(v.size != n for v in vecs):
        raise ValueError("VecDump: the vectors of one group must have the same size")
    ptrs = (C.c_void_p * len(vecs))(*[v.ctypes.data for v in vecs])
    L.check(L.load().lsg_vec_dump(fname.encode(), len(vecs), ptrs, n, int(bool(petsc_int64))))


def VecLoad(fname: str, n: int, nvecs=1, petsc_int64=False):
    """Read nvecs PETSc binary Vec records of n values; returns a (nvecs, n) array."""
    out = np.empty((nvecs, n), np.float64)
    ptrs = (C.c_void_p * nvecs)(*[out[k].ctypes.data for k in range(nvecs)])
    L.check(L.load().lsg_vec_load(fname.encode(), int(nvecs), ptrs, int(n), int(bool(petsc_int64))))
    return out


def forest_save(forest: Forest, fname: str):
    L.check(L.load().lsg_forest_save(forest.handle, fname.encode()))


def forest_load(fname: str) -> Forest:
    """A forest saved by forest_save (nodes not built)."""
    h = C.c_void_p()
    L.check(L.load().lsg_forest_load(fname.encode(), C.byref(h)))
    head = np.fromfile(fname, dtype=np.uint8, count=8 + 4 + 12 + 48 + 8)
    dim = int(head[8:12].view("<i4")[0])
    f = Forest.__new__(Forest)
    f._h = h
    f.dim = dim
    f.n_xyz = tuple(int(v) for v in head[12:24].view("<i4"))
    f.xyz_min = tuple(float(v) for v in head[24:48].view("<f8"))
    f.xyz_max = tuple(float(v) for v in head[48:72].view("<f8"))
    f.max_lvl_requested = int(f.leaves()[1].max()) if f.num_leaves else 0
    return f


def my_p4est_save_forest_and_data(folder: str, forest: Forest, forest_filename: str, elements):
    """elements: [(name, [vec, ...]), ...] node vectors; each group goes to <folder>/<name>.petscbin."""
    if not os.path.isdir(folder):
        raise ValueError("my_p4est_save_forest_and_data: invalid path to exportation folder")
    forest_save(forest, os.path.join(folder, forest_filename))
    for name, vecs in elements:
        VecDump(os.path.join(folder, name + ".petscbin"), vecs)


def my_p4est_load_forest_and_data(folder: str, forest_filename: str, elements):
    """elements: [(name, nvecs), ...]. Returns (forest with nodes built, {name: (nvecs, N) array})."""
    forest = forest_load(os.path.join(folder, forest_filename)).build_nodes()
    data = {name: VecLoad(os.path.join(folder, name + ".petscbin"), forest.num_nodes, nvecs) for name, nvecs in elements}
    return forest, data
