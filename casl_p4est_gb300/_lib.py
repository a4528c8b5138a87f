"""ctypes binding of liblsgpu.so (the C ABI declared in include/lsgpu.h).

The library is loaded from the package's ``_lib`` directory; nothing here falls back to Python
arithmetic: if the library is missing, importing the bindings raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "liblsgpu.so")

LSG_OK, LSG_EINVAL, LSG_ENOMEM, LSG_EDEVICE, LSG_ETIMEOUT, LSG_ENAN, LSG_ESTATE = range(7)
LSG_FP64, LSG_MIXED = 0, 1
LSG_BUILD_ON_DEVICE = 1
# int (*lsg_velocity_fn)(void* ctx, int64_t npts, const double* xyz, double* v)
# int (*lsg_interface_values_fn)(void* ctx, int64_t count, const int32_t* nodes, const int32_t* dirs, const double* dists, double* values)
INTERFACE_VALUES_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                  C.POINTER(C.c_double))
VELOCITY_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double))
LSG_VELOCITY_VORTEX = 0

_P = C.c_void_p
_I = C.c_int
_I64 = C.c_int64
_D = C.c_double
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
_I32P = C.POINTER(C.c_int32)
_U8P = C.POINTER(C.c_uint8)

# name: (restype, argtypes)
SIGNATURES = {
    "lsg_last_error": (C.c_char_p, []),
    "lsg_version": (_I, []),
    "lsg_forest_create": (_I, [_I, _IP, _DP, _DP, _IP, C.POINTER(_P)]),
    "lsg_forest_destroy": (_I, [_P]),
    "lsg_forest_dim": (_I, [_P]),
    "lsg_forest_num_leaves": (_I64, [_P]),
    "lsg_forest_leaves": (_I, [_P, _I32P, _I32P, _I32P]),
    "lsg_forest_copy": (_I, [_P, C.POINTER(_P)]),
    "lsg_forest_set_leaves": (_I, [_P, _I64, _I32P, _I32P, _I32P]),
    "lsg_forest_refine_and_coarsen": (_I, [_P, _I, _I, _D, _D, _DP, C.POINTER(_I)]),
    "lsg_forest_refine": (_I, [_P, _U8P, _I64]),
    "lsg_forest_coarsen": (_I, [_P, _U8P, _I64]),
    "lsg_forest_tag_levelset": (_I, [_P, _I, _I, _D, _D, _I, _DP, _I, _U8P]),
    "lsg_forest_refine_levelset": (_I, [_P, _I, _I, _D, _D, _I, _DP, _I, _I]),
    "lsg_forest_build_nodes": (_I, [_P]),
    "lsg_forest_build_nodes_device": (_I, [_P, _P]),
    "lsg_vtk_write_all": (_I, [_P, C.c_char_p, _I, _I, _P, _P, _I, _P, _P, _I]),
    "lsg_vec_dump": (_I, [C.c_char_p, _I, _P, _I64, _I]),
    "lsg_vec_load": (_I, [C.c_char_p, _I, _P, _I64, _I]),
    "lsg_forest_save": (_I, [_P, C.c_char_p]),
    "lsg_forest_load": (_I, [C.c_char_p, C.POINTER(_P)]),
    "lsg_forest_node_xyz_device": (_I, [_P, _P, _P]),
    "lsg_forest_refine_and_coarsen_device": (_I, [_P, _I, _I, _D, _D, _P, C.POINTER(C.c_int), _P]),
    "lsg_forest_num_nodes": (_I64, [_P]),
    "lsg_forest_node_xyz": (_I, [_P, _DP]),
    "lsg_forest_nodes": (_I, [_P, _I32P, _I32P]),
    "lsg_forest_local_nodes": (_I, [_P, _I32P]),
    "lsg_forest_sample_shape": (_I, [_P, _I, _DP, _I, _DP]),
    "lsg_qnnn_record_bytes": (C.c_size_t, [_I]),
    "lsg_forest_export_qnnn": (_I, [_P, _I64, _I64, _P, C.c_size_t]),
    "lsg_forest_wall_mask": (_I, [_P, _U8P]),
    "lsg_forest_dxyz_min": (_I, [_P, _DP]),
    "lsg_level_set_create": (_I, [_P, C.POINTER(_P)]),
    "lsg_level_set_create_ex": (_I, [_P, _I, C.POINTER(_P)]),
    "lsg_level_set_destroy": (_I, [_P]),
    "lsg_level_set_set_stream": (_I, [_P, _P]),
    "lsg_level_set_stream": (_P, [_P]),
    "lsg_level_set_num_nodes": (_I64, [_P]),
    "lsg_level_set_zero_distance_threshold": (_D, [_P]),
    "lsg_reinitialize": (_I, [_P, _DP, _I, _I, _D, _D, _I, _I]),
    "lsg_reinitialize_device": (_I, [_P, _P, _I, _I, _D, _D, _I, _I]),
    "lsg_reinitialize_with_mask": (_I, [_P, _DP, _DP, _I, _I, _D, _D, _I, _I]),
    "lsg_reinitialize_with_mask_device": (_I, [_P, _P, _P, _I, _I, _D, _D, _I, _I]),
    "lsg_reinitialize_device_noalloc": (_I, [_P, _P, _I, _I, _D, _D, _I]),
    "lsg_reinit_2nd": (_I, [_P, _DP, _I, _D, _I]),
    "lsg_advect_in_normal_direction": (_I, [_P, _DP, _DP, _DP, _D, _DP, _I]),
    "lsg_advect_in_normal_direction_device": (_I, [_P, _P, _P, _P, _D, _P, _I]),
    "lsg_advect_cfl_dt": (_I, [_P, _DP, _DP]),
    "lsg_second_derivatives": (_I, [_P, _DP, _DP]),
    "lsg_second_derivatives_device": (_I, [_P, _P, _P]),
    "lsg_perturb_level_set_function": (_I, [_P, _DP, _D]),
    "lsg_level_set_enable_kernel_timing": (_I, [_P, _I]),
    "lsg_first_derivatives": (_I, [_P, _DP, _DP]),
    "lsg_first_derivatives_device": (_I, [_P, _P, _P]),
    "lsg_compute_normals": (_I, [_P, _DP, _DP]),
    "lsg_compute_normals_device": (_I, [_P, _P, _P]),
    "lsg_compute_mean_curvature": (_I, [_P, _DP, _DP]),
    "lsg_compute_mean_curvature_device": (_I, [_P, _P, _P]),
    "lsg_compute_normals_and_mean_curvature": (_I, [_P, _DP, _DP, _DP]),
    "lsg_compute_normals_and_mean_curvature_device": (_I, [_P, _P, _P, _P]),
    "lsg_extend_over_interface_tvd": (_I, [_P, _DP, _DP, _I, _I, _D, _D, _DP, _DP]),
    "lsg_extend_over_interface_tvd_device": (_I, [_P, _P, _P, _I, _I, _D, _D, _P, _P]),
    "lsg_extend_over_interface_tvd_ex": (_I, [_P, _DP, _DP, _I, _I, _D, _D, _DP, _DP, _I, _DP, _DP]),
    "lsg_extend_over_interface_tvd_ex_device": (_I, [_P, _P, _P, _I, _I, _D, _D, _P, _P, _I, _P, _P]),
    "lsg_extend_from_interface_to_whole_domain_tvd": (_I, [_P, _DP, _DP, _DP, _I, _I, _DP, _D, _D, _DP, _I]),
    "lsg_extend_from_interface_to_whole_domain_tvd_device": (_I, [_P, _P, _P, _P, _I, _I, _P, _D, _D, _P, _I]),
    "lsg_extend_from_interface_to_whole_domain_tvd_cf": (_I, [_P, _DP, _DP, _DP, _I, _P, _P, _DP]),
    "lsg_interpolate_nodes": (_I, [_P, _DP, _I64, _DP, _I, _DP, _I, _DP]),
    "lsg_interpolate_nodes_device": (_I, [_P, _P, _I64, _P, _I, _P, _I, _P]),
    "lsg_locate_points_device": (_I, [_P, _P, _I64, _P]),
    "lsg_semi_lagrangian_advect": (_I, [_P, _DP, _I64, _D, _DP, _DP, _DP, _DP, _I, _I, _DP]),
    "lsg_semi_lagrangian_advect_device": (_I, [_P, _P, _I64, _D, _P, _P, _P, _P, _I, _I, _P]),
    "lsg_semi_lagrangian_advect_cf": (_I, [_P, _DP, _I64, _D, _I, _DP, _I, _DP, _DP, _I, _DP]),
    "lsg_semi_lagrangian_advect_cf_device": (_I, [_P, _P, _I64, _D, _I, _DP, _I, _P, _P, _I, _P]),
    "lsg_semi_lagrangian_advect_callback": (_I, [_P, _DP, _I64, _D, _P, _P, _DP, _DP, _I, _DP]),
    "lsg_semi_lagrangian_advect2": (_I, [_P, _P, _DP, _I64, _D, _D, _DP, _DP, _DP, _DP, _DP, _DP, _I, _I, _DP]),
    "lsg_semi_lagrangian_advect2_device": (_I, [_P, _P, _P, _I64, _D, _D, _P, _P, _P, _P, _P, _P, _I, _I, _P]),
    "lsg_level_set_set_wait_limit": (_I, [_P, C.c_longlong]),
    "lsg_second_derivatives_range_device": (_I, [_P, _P, _P, _I64, _I64]),
    "lsg_reinit_prep_range_device": (_I, [_P, _P, _P, _I, _D, _D, _I64, _I64]),
    "lsg_reinit_stage_range_device": (_I, [_P, _I, _P, _P, _P, _P, _P, _I64, _I64]),
    "lsg_advect_stage_range_device": (_I, [_P, _P, _P, _P, _P, _D, _P, _P, _I64, _I64]),
    "lsg_mixed_split_begin_device": (_I, [_P, _P, _P, _I, _D, _D]),
    "lsg_mixed_split_stage_device": (_I, [_P, _I, _I]),
    "lsg_mixed_split_field_device": (_I, [_P, _I, C.POINTER(C.c_void_p)]),
    "lsg_mixed_split_slots_device": (_I, [_P, _P]),
    "lsg_mixed_split_end_device": (_I, [_P, _P]),
    "lsg_interface_location_error_device": (_I, [_P, _P, _P, _DP, C.POINTER(_I64), C.POINTER(_I64)]),
    "lsg_band_linf_device": (_I, [_P, _P, _P, _D, _DP, C.POINTER(_I64)]),
    "lsg_batch_create": (_I, [_I, C.POINTER(_P), C.POINTER(_P)]),
    "lsg_batch_create_ex": (_I, [_I, C.POINTER(_P), _I, C.POINTER(_P)]),
    "lsg_batch_count": (_I, [_P]),
    "lsg_batch_offsets": (_I, [_P, C.POINTER(_I64)]),
    "lsg_batch_reinitialize": (_I, [_P, _DP, _I32P, _I]),
    "lsg_batch_reinitialize_device": (_I, [_P, _P, _I32P, _I]),
    "lsg_level_set_autotune": (_I, [_P, _DP, _I, _I32P]),
    "lsg_level_set_stage_config": (_I, [_P, _I32P]),
    "lsg_level_set_set_stage_config": (_I, [_P, _I32P]),
    "lsg_level_set_table_stats": (_I, [_P, C.POINTER(_I64)]),
    "lsg_level_set_kernel_times": (_I, [_P, _DP, C.POINTER(_I64), _I, _I]),
    "lsg_level_set_launch_count": (_I64, [_P]),
    "lsg_device_cache_bytes": (_I64, []),
    "lsg_device_cache_release": (_I, []),
}

KERNEL_KINDS = ["dd64", "prep64", "stage64", "advect64", "dd32", "prep_mixed", "stage32", "advect32", "convert", "copy", "interp"]


class LsgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[lsgpu status {code}] {msg}")
        self.code = code


class LsgInvalidArgument(LsgError, ValueError):
    pass


class LsgTimeout(LsgError, TimeoutError):
    """A bounded device-side wait gave up (LSG_ETIMEOUT); the call's results are incomplete."""


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m casl_p4est_gb300.build`")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int) -> None:
    if code == LSG_OK:
        return
    msg = load().lsg_last_error().decode(errors="replace")
    if code == LSG_EINVAL:
        raise LsgInvalidArgument(code, msg)
    if code == LSG_ETIMEOUT:
        raise LsgTimeout(code, msg)
    raise LsgError(code, msg)


def dptr(a):
    return a.ctypes.data_as(_DP)


def i32ptr(a):
    return a.ctypes.data_as(_I32P)


def u8ptr(a):
    return a.ctypes.data_as(_U8P)
