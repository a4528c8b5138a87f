"""Failure detection without a GPU fault: the bulk-copy stage kernel's bounded waits.

The kernel waits for its own cp.async.bulk copies on mbarriers, each wait bounded. With the bound set to a
single SM cycle (lsg_level_set_set_wait_limit), the first wait of every block runs out while its copies are
still on their way: the block then lets those copies land (bounded by the full limit) and stops, the call
returns LSG_ETIMEOUT (LsgTimeout here), and the next call on the same level set starts clean and gives the
same bits as before. Nothing faults, traps or hangs: every wait is bounded and every copy lands."""
import numpy as np
import pytest

import casl_p4est_gb300 as G

from grids import flower_3d, phi0_flower_3d

pytestmark = pytest.mark.gpu

BULK = {"threads_per_block": 256, "uniform_blocks": 0, "regular_blocks": 0, "uniform_depth": 3}


@pytest.fixture(scope="module")
def grid():
    f = flower_3d(3, 7)
    ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f), precision="mixed")
    return f, ls, phi0_flower_3d(f)


def test_bulk_kernel_runs_and_matches_register_pipeline(grid):
    f, ls, phi0 = grid
    assert ls.table_stats()["uniform"] > 10000
    ref = phi0.copy()
    ls.reinitialize_2nd_order(ref, 4, precision="mixed")
    cfg = ls.stage_config
    ls.stage_config = BULK
    got = phi0.copy()
    ls.reinitialize_2nd_order(got, 4, precision="mixed")
    ls.stage_config = cfg
    assert np.array_equal(got, ref)


def test_bounded_wait_gives_up_and_next_call_is_clean(grid):
    f, ls, phi0 = grid
    ref = phi0.copy()
    ls.reinitialize_2nd_order(ref, 4, precision="mixed")
    cfg = ls.stage_config
    ls.stage_config = BULK
    try:
        ls.set_wait_limit(1)
        with pytest.raises(G.LsgTimeout):
            ls.reinitialize_2nd_order(phi0.copy(), 4, precision="mixed")
        ls.set_wait_limit(0)
        again = phi0.copy()
        ls.reinitialize_2nd_order(again, 4, precision="mixed")
        assert np.array_equal(again, ref)
    finally:
        ls.set_wait_limit(0)
        ls.stage_config = cfg
    after = phi0.copy()
    ls.reinitialize_2nd_order(after, 4, precision="mixed")
    assert np.array_equal(after, ref)


def test_autotune_discards_a_candidate_that_timed_out(grid):
    """With the bound at one cycle every bulk-copy candidate gives up; the autotuner must not pick it and
    must leave no flag behind for the next call."""
    f, ls, phi0 = grid
    cfg = ls.stage_config
    try:
        ls.set_wait_limit(1)
        best = ls.autotune(phi0, trials=1)
        assert best["uniform_depth"] in (1, 2, 5)
        got = phi0.copy()
        ls.reinitialize_2nd_order(got, 4, precision="mixed")
    finally:
        ls.set_wait_limit(0)
        ls.stage_config = cfg
    ref = phi0.copy()
    ls.reinitialize_2nd_order(ref, 4, precision="mixed")
    assert np.array_equal(got, ref)


def test_calls_run_on_the_level_sets_device(grid):
    """Every call is made on the device the level set was created on (the only one here); the caller's
    current device is left as it was."""
    import torch
    f, ls, phi0 = grid
    before = torch.cuda.current_device()
    p = phi0.copy()
    ls.reinitialize_2nd_order(p, 2, precision="fp64")
    assert torch.cuda.current_device() == before
