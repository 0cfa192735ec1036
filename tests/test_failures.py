"""Failure detection without a GPU fault: errors are reported as status
codes or counters and the system (or device) stays usable.  Capacity
exhaustion and corrupt scene files are covered beside the features they
belong to (test_gpu_parity.py, test_scene.py)."""
import numpy as np
import pytest

import granular_gpu_gb300 as gg
from granular_gpu_gb300 import abi, workloads


@pytest.mark.gpu
def test_bounded_wait_gives_up_and_reports():
    # a wait on a barrier phase nothing completes: bounded, reported, and
    # the device keeps working afterwards
    assert gg.lib().gg_selftest_bounded_wait(0, 2000) == abi.GG_ERR_TIMEOUT
    assert gg.lib().gg_selftest_bounded_wait(0, 1) == abi.GG_ERR_TIMEOUT
    desc = workloads.box_drop(n_side=6)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    s.step(3)
    assert np.isfinite(s.read(gg.FIELD_POS)).all()
    s.close()


def test_bounded_wait_rejects_bad_limits_without_a_gpu():
    assert gg.lib().gg_selftest_bounded_wait(0, 0) == abi.GG_ERR_INVALID_ARGUMENT
    assert gg.lib().gg_selftest_bounded_wait(0, 1 << 21) == abi.GG_ERR_INVALID_ARGUMENT


@pytest.mark.gpu
def test_injected_nan_is_counted_and_contained():
    desc = workloads.box_drop(n_side=8, substeps=4, iters=3)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    p = s.read(gg.FIELD_POS)
    p[17] = (np.nan, 0.5, 0.5)
    s.write(gg.FIELD_POS, p)
    s.step(5)
    # the NaN particle hashes to cell 0 and fails every contact test
    # (comparisons with NaN are false), so it stays the only one
    st = s.stats()
    assert st["nonfinite"] == 1
    q = s.read(gg.FIELD_POS)
    assert np.isfinite(q).sum(1).tolist().count(3) == len(q) - 1
    s.close()
