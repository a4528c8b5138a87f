"""The C-ABI library loads, exports every symbol include/lsgpu.h declares, and reports bad
arguments as status codes (no GPU needed for the grid-side entry points)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import casl_p4est_gb300 as G
from casl_p4est_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "lsgpu.h")).read()
    return sorted(set(re.findall(r"\b(lsg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(L.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    assert set(declared_symbols()) <= set(L.SIGNATURES)


def test_device_cache_queries_need_no_device():
    # nothing allocated yet in this process: nothing cached, and releasing nothing succeeds
    assert G.device_cache_bytes() >= 0
    if G.device_cache_bytes() == 0:
        G.release_device_cache()
        assert G.device_cache_bytes() == 0


def test_bad_arguments_return_status_codes():
    lib = L.load()
    h = C.c_void_p()
    n = (C.c_int * 3)(1, 1, 1)
    lo = (C.c_double * 3)(0, 0, 0)
    hi = (C.c_double * 3)(1, 1, 1)
    assert lib.lsg_forest_create(4, n, lo, hi, None, C.byref(h)) == L.LSG_EINVAL
    assert "dim" in lib.lsg_last_error().decode()
    bad_hi = (C.c_double * 3)(0, 1, 1)
    assert lib.lsg_forest_create(2, n, lo, bad_hi, None, C.byref(h)) == L.LSG_EINVAL
    f = G.my_p4est_brick_new([1, 1], [0, 0], [1, 1])
    tags = np.ones(5, np.uint8)
    assert lib.lsg_forest_refine(f.handle, L.u8ptr(tags), 5) == L.LSG_EINVAL
    # nodes not built yet: level-set construction is refused before touching the device
    ls = C.c_void_p()
    assert lib.lsg_level_set_create(f.handle, C.byref(ls)) == L.LSG_ESTATE
    assert lib.lsg_forest_num_nodes(f.handle) == -1
    with pytest.raises(G.LsgInvalidArgument):
        f.refine(np.ones(3, np.uint8))


def test_record_layout_matches_python_dtype():
    for dim in (2, 3):
        assert G.qnnn_dtype(dim).itemsize == L.load().lsg_qnnn_record_bytes(dim)
