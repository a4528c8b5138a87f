"""casl_p4est_gb300: the level-set hot path of parCASL (UCSB-CASL/casl_p4est) on GB300.

Reinitialisation (reinitialize_2nd_order and its siblings), normal-direction advection and
semi-Lagrangian node interpolation on quadtree/octree grids, as CUDA kernels for sm_103a behind a
C ABI (include/lsgpu.h). The Python classes mirror the reference's C++ class API.
"""
from . import shapes
from ._lib import LSG_FP64, LSG_MIXED, LsgError, LsgInvalidArgument, LsgTimeout, load


def device_cache_bytes() -> int:
    """Device memory released by level sets and grids and kept for reuse, in bytes."""
    return int(load().lsg_device_cache_bytes())


def release_device_cache() -> None:
    """Give the device memory kept for reuse back to the driver (synchronises the device)."""
    from ._lib import check
    check(load().lsg_device_cache_release())


from .forest import Forest, my_p4est_brick_new, my_p4est_node_neighbors_t, qnnn_dtype
from .level_set import DBL_MAX, my_p4est_level_set_batch_t, my_p4est_level_set_t
from .interpolation import VortexVelocity, my_p4est_interpolation_nodes_t, my_p4est_semi_lagrangian_t
from . import interpolation, save_load
from .save_load import (VecDump, VecLoad, my_p4est_load_forest_and_data, my_p4est_save_forest_and_data,
                        my_p4est_vtk_write_all)

__all__ = [
    "shapes", "load", "LsgError", "LsgInvalidArgument", "LsgTimeout", "LSG_FP64", "LSG_MIXED", "Forest", "my_p4est_brick_new",
    "my_p4est_node_neighbors_t", "qnnn_dtype", "my_p4est_level_set_t", "DBL_MAX", "interpolation",
    "my_p4est_interpolation_nodes_t", "my_p4est_semi_lagrangian_t", "VortexVelocity", "my_p4est_level_set_batch_t",
    "save_load", "VecDump", "VecLoad", "my_p4est_save_forest_and_data", "my_p4est_load_forest_and_data",
    "my_p4est_vtk_write_all", "device_cache_bytes", "release_device_cache",
]
