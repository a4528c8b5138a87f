"""lsg_reinitialize_device_noalloc: the FP64 reinitialisation with its work vectors in a static
device array, called through the C ABI and compared with lsg_reinitialize_device (LSG_FP64) on
two calls in a row. Both run the same FP64 kernels in the same order, so the tolerance is the
FP64 tests' one: exact equality.

Kept in its own file, collected last, so that it runs both after the other GPU tests and alone in
a fresh process (where its first call performs the per-device set-up)."""
import ctypes as C

import numpy as np
import pytest

import casl_p4est_gb300 as G
from casl_p4est_gb300 import _lib as L

from grids import circle_2d, flower_3d, phi0_circle_2d, phi0_flower_3d

pytestmark = pytest.mark.gpu

DBL_MAX = np.finfo(np.float64).max
SCRATCH_BYTES = 32 << 20


def _level_set(forest):
    import torch
    ngbd = G.my_p4est_node_neighbors_t(forest)
    ls = G.my_p4est_level_set_t(ngbd)
    ls.set_stream(torch.cuda.current_stream().cuda_stream)
    return ls


def _allocating(ls, phi, os, ot, hi, lo, iters):
    L.check(L.load().lsg_reinitialize_device(ls.handle, C.c_void_p(phi.data_ptr()), os, ot, hi, lo, iters, L.LSG_FP64))


def _noalloc(ls, phi, os, ot, hi, lo, iters):
    return L.load().lsg_reinitialize_device_noalloc(ls.handle, C.c_void_p(phi.data_ptr()), os, ot, hi, lo, iters)


CASES = {
    "flower3d": (lambda: flower_3d(3, 7), phi0_flower_3d),
    "circle2d": (lambda: circle_2d(3, 9), phi0_circle_2d),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_noalloc_matches_allocating_path_on_two_calls(name):
    import torch
    build, phi0_of = CASES[name]
    f = build()
    ls = _level_set(f)
    phi0 = torch.from_numpy(phi0_of(f)).cuda()
    ref = phi0.clone()
    got = phi0.clone()
    # two calls in a row on the same arrays, with different orders and limits
    for os, ot, hi, lo, iters in [(2, 2, DBL_MAX, -DBL_MAX, 8), (1, 2, 0.3, -0.2, 5)]:
        _allocating(ls, ref, os, ot, hi, lo, iters)
        L.check(_noalloc(ls, got, os, ot, hi, lo, iters))
        torch.cuda.synchronize()
        a, b = ref.cpu().numpy(), got.cpu().numpy()
        assert np.array_equal(a, b), f"{name} orders {(os, ot)}: max diff {np.max(np.abs(a - b))}"
    assert not np.array_equal(ref.cpu().numpy(), phi0.cpu().numpy())


def test_noalloc_leaves_free_memory_unchanged():
    import torch
    f = flower_3d(3, 6)
    ls = _level_set(f)
    phi = torch.from_numpy(phi0_flower_3d(f)).cuda()
    for _ in range(2):  # set-up and first use of every kernel variant
        L.check(_noalloc(ls, phi, 2, 2, DBL_MAX, -DBL_MAX, 2))
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    L.check(_noalloc(ls, phi, 2, 2, DBL_MAX, -DBL_MAX, 2))
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before


def test_noalloc_rejects_grids_beyond_the_scratch():
    import torch
    f = flower_3d(4, 8)  # 858,915 nodes: 114 bytes each exceed the static scratch
    assert f.num_nodes * 114 > SCRATCH_BYTES
    ls = _level_set(f)
    phi = torch.from_numpy(phi0_flower_3d(f)).cuda()
    before = phi.clone()
    assert _noalloc(ls, phi, 2, 2, DBL_MAX, -DBL_MAX, 2) == L.LSG_EINVAL
    msg = L.load().lsg_last_error().decode()
    assert "LSG_NOALLOC_SCRATCH_BYTES" in msg and str(f.num_nodes) in msg
    torch.cuda.synchronize()
    assert torch.equal(phi, before)
    assert L.load().lsg_reinitialize_device_noalloc(ls.handle, None, 2, 2, DBL_MAX, -DBL_MAX, 2) == L.LSG_EINVAL
