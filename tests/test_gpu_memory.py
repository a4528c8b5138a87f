"""The device memory cache behind every table and work vector: a destroyed level set's buffers are kept,
the next level set reuses them with unchanged results, and lsg_device_cache_release gives them back
to the driver."""
import gc

import numpy as np
import pytest

import casl_p4est_gb300 as G
from grids import flower_3d, phi0_flower_3d

pytestmark = pytest.mark.gpu


def _reinit(f, phi0, device_build):
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f), device_build=device_build)
    phi = phi0.copy()
    ls.reinitialize_2nd_order(phi, 10, precision="fp64")
    mixed = phi0.copy()
    ls.reinitialize_2nd_order(mixed, 10, precision="mixed")
    return ls, phi, mixed


@pytest.mark.parametrize("device_build", [False, True])
def test_cache_reuse_keeps_results_and_release_returns_memory(device_build):
    import torch
    f = flower_3d(3, 6)
    if device_build:
        f.build_nodes(device=True)
    phi0 = phi0_flower_3d(f)
    gc.collect()
    G.release_device_cache()
    assert G.device_cache_bytes() == 0
    # first level set: every buffer comes from the driver
    ls, fresh64, fresh32 = _reinit(f, phi0, device_build)
    del ls
    gc.collect()
    held = G.device_cache_bytes()
    assert held > 0
    # second level set on the same grid: buffers come back out of the cache, results unchanged
    ls, again64, again32 = _reinit(f, phi0, device_build)
    assert G.device_cache_bytes() < held
    np.testing.assert_array_equal(again64, fresh64)
    np.testing.assert_array_equal(again32, fresh32)
    del ls
    gc.collect()
    held = G.device_cache_bytes()
    assert held > 0
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    G.release_device_cache()
    assert G.device_cache_bytes() == 0
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after - free_before >= held // 2

