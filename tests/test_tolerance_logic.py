"""The raster and trajectory criteria themselves (CPU)."""
import numpy as np
import pytest

from tolerance import assert_rasters_match, trajectory_errors


def test_raster_shift_accepted_only_at_small_margin():
    ref = {(t, j): 1.0 for t, j in [(10, 1), (20, 2), (30, 3)]} | {(40, 4): 0.001}
    assert assert_rasters_match(set(ref), ref) == 0
    got = set(ref) - {(40, 4)} | {(41, 4)}
    assert assert_rasters_match(got, ref, max_frac=0.5) == 1
    with pytest.raises(AssertionError):   # same shift, but the crossing was not marginal
        assert_rasters_match(set(ref) - {(30, 3)} | {(31, 3)}, ref, max_frac=0.5)
    with pytest.raises(AssertionError):   # a spike the oracle does not have
        assert_rasters_match(set(ref) | {(50, 5)}, ref)
    with pytest.raises(AssertionError):   # shifted by two steps
        assert_rasters_match(set(ref) - {(40, 4)} | {(42, 4)}, ref, max_frac=0.5)


def test_trajectory_criterion_separates_steep_neurons():
    ref = np.array([[-65.0, -10.0], [0.05, 0.6], [0.6, 0.3], [0.3, 0.5]])
    prev = ref.copy()
    prev[0, 1] = -12.0                    # 200 mV/ms: in a spike
    got = ref.copy()
    got[0, 1] += 0.1                      # within a 1 us shift at 200 mV/ms
    assert trajectory_errors(got, ref, prev, 0.01)["violations"] == 0
    got[0, 0] += 0.01                     # 1.5e-4 relative at rest: violation
    assert trajectory_errors(got, ref, prev, 0.01)["violations"] == 1
