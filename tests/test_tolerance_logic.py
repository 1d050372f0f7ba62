"""The raster and trajectory criteria themselves (CPU)."""
import numpy as np
import pytest

from tolerance import assert_rasters_match, assert_trajectory, perturbed_neurons, trajectory_errors


def test_raster_shift_accepted_only_at_small_margin():
    ref = {(t, j): 1.0 for t, j in [(10, 1), (20, 2), (30, 3)]} | {(40, 4): 0.001}
    assert assert_rasters_match(set(ref), ref) == []
    got = set(ref) - {(40, 4)} | {(41, 4)}
    assert assert_rasters_match(got, ref, max_frac=0.5) == [(40, 4)]
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


def test_perturbed_neurons_are_held_to_the_wider_bound():
    rp = np.array([0, 2, 2, 3])
    col = np.array([1, 2, 0])
    mask = perturbed_neurons([(10, 0)], rp, col, 3)
    assert mask.tolist() == [True, True, True]
    mask = perturbed_neurons([(10, 1)], rp, col, 3)
    assert mask.tolist() == [False, True, False]
    ref = np.array([[-65.0, -60.0, -70.0], [0.05] * 3, [0.6] * 3, [0.3] * 3])
    got = ref.copy()
    got[0, 1] += 0.5                        # 1e-2 relative on a perturbed neuron
    assert_trajectory(got, ref, ref, 0.01, exclude=mask)
    with pytest.raises(AssertionError):
        assert_trajectory(got, ref, ref, 0.01)
    got[0, 1] += 10.0                       # beyond the 5e-2 bound
    with pytest.raises(AssertionError):
        assert_trajectory(got, ref, ref, 0.01, exclude=mask)


def test_cascade_of_a_root_shift_is_explained_only_downstream():
    from oracle.parity import compare_rasters
    # neuron 1 -> targets 2, 3; neuron 4 -> target 5
    row_ptr = np.array([0, 0, 2, 2, 2, 3, 3])
    col = np.array([2, 3, 5])
    ref = {(10, 1): 0.001, (15, 2): 1.0, (15, 4): 1.0, (20, 5): 1.0}
    got = {(11, 1), (16, 2), (15, 4), (20, 5)}
    r = compare_rasters(got, ref, row_ptr=row_ptr, col=col)
    assert r["shifted"] == [(10, 1)] and r["cascade"] == [(15, 2)]
    assert not r["unexplained_oracle"] and not r["unexplained_device"]
    assert r["perturbed"] == [1, 2, 3]
    # without the network the downstream shift is unexplained
    r = compare_rasters(got, ref)
    assert r["unexplained_oracle"] == [(15, 2)]
    # a shift of a neuron no difference reaches stays unexplained
    r = compare_rasters({(11, 1), (15, 2), (16, 4), (20, 5)}, ref, row_ptr=row_ptr, col=col)
    assert r["unexplained_oracle"] == [(15, 4)]
    # a spike missing on the device entirely, downstream of the root shift
    r = compare_rasters({(11, 1), (15, 4), (20, 5)}, ref, row_ptr=row_ptr, col=col)
    assert r["cascade"] == [(15, 2)] and not r["unexplained_oracle"]
