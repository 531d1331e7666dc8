"""Failure handling on the GPU without a GPU fault: a bounded device wait is
made to run out on purpose (a barrier nothing arrives on, 1 ms limit), the
host sees TDM_ERR_TIMEOUT from tdm_device_status, and the next library call
works in the same context.  The reference has no counterpart: Marvin's
FatalError exits the process (core/marvin.hpp:132-138)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_the_context_stays_usable(tdm, oracle, cuda, scene):
    import torch
    tdm.device_status()  # start clean
    copied, timed_out, word = tdm.selftest_wait_timeout(1000)
    assert copied == 1 and word == 0x5E1F7E57  # the completed copy was waited for normally
    assert timed_out == 1
    with pytest.raises(tdm.TdmError) as e:
        tdm.device_status()
    assert e.value.status == 6  # TIMEOUT
    tdm.device_status()  # the word was cleared by the read
    # the next library call runs normally (TDF of a small fragment, bit-exact)
    pts = scene.fragment(20260003, n_points=5000)
    g = tdm.grid_from_points_host(pts)
    got = tdm.tdf(torch.from_numpy(pts).to(cuda), g).cpu().numpy()
    dim, origin = oracle.grid_setup(pts)
    occ = oracle.occupancy(pts, dim, origin, 0.01)
    assert np.array_equal(got, oracle.tdf(occ, dim, 0.01, np.float32(0.01) * np.float32(5)))
    tdm.device_status()


def test_selftest_rejects_out_of_range_budgets(tdm, cuda):
    import torch
    out = torch.zeros(3, dtype=torch.int32, device=cuda)
    assert tdm.lib().tdm_selftest_wait_timeout(0, out.data_ptr(), None) == 1
    assert tdm.lib().tdm_selftest_wait_timeout(2_000_000, out.data_ptr(), None) == 1
    assert tdm.lib().tdm_selftest_wait_timeout(1000, None, None) == 1
