"""Trajectory and raster tolerance shared by the parity tests.

The criteria live in oracle/parity.py (also used by bench.py's parity
report); this module turns them into assertions.

* Trajectories: |dV/dt| < 20 mV/ms at the checkpoint (not in a spike): every
  variable within ``rtol`` = 1e-4 relative, floors 1 mV for V and 1e-3 for
  gates; steep neurons (in a spike): within their rate of change times a
  spike-time shift of 1 us, plus the 1e-4-relative allowance.
* Rasters: identical (step, neuron) sets, with one stated relaxation of
  "identical spike rasters": a spike may sit one step earlier or later when
  the FP64 oracle's threshold crossing lies within 0.01 mV of the step
  boundary, for at most 0.5 % of the spikes.  Such a crossing is decided by
  the last bits of the FP32 potential, whose rounding the FP64 oracle does not
  share.
"""
from __future__ import annotations

import numpy as np

from oracle.parity import (FLOORS, MARGIN_MV, SHIFT_MS, STEEP_MV_PER_MS, compare_rasters,  # noqa: F401
                           perturbed_neurons, trajectory_errors)


def assert_trajectory(got, ref, ref_prev, dt_ms, rtol=1e-4, exclude=None, exclude_bound=5e-2):
    """exclude: neurons perturbed by an accepted one-step spike shift (the
    shifted neurons and their postsynaptic targets, which received that input
    one step apart); they are held to exclude_bound relative instead."""
    got, ref, ref_prev = (np.asarray(a, np.float64) for a in (got, ref, ref_prev))
    if exclude is not None and np.any(exclude):
        keep = ~np.asarray(exclude, bool)
        floors = np.array(FLOORS)[:, None]
        rel_ex = np.abs(got[:, ~keep] - ref[:, ~keep]) / (np.abs(ref[:, ~keep]) + floors)
        assert rel_ex.max() < exclude_bound, rel_ex.max()
        got, ref, ref_prev = got[:, keep], ref[:, keep], ref_prev[:, keep]
    e = trajectory_errors(got, ref, ref_prev, dt_ms, rtol)
    assert e["violations"] == 0, e
    return e


def assert_rasters_match(got: set, ref_margins: dict, max_frac: float = 0.005) -> list:
    """Spike rasters as sets of (step, neuron): identical except for spikes
    shifted by exactly one step whose FP64 threshold crossing lies within
    MARGIN_MV of the step boundary, at most max_frac of the spikes (no
    cascades: the windows these tests use are checked without the network).
    Returns the shifted oracle spikes."""
    r = compare_rasters(got, ref_margins)
    assert not r["unexplained_oracle"], f"oracle spikes missing on the device: {r['unexplained_oracle'][:5]}"
    assert not r["unexplained_device"], f"device spikes without an oracle counterpart: {r['unexplained_device'][:5]}"
    assert len(r["shifted"]) <= max_frac * max(len(ref_margins), 1), (len(r["shifted"]), len(ref_margins))
    return r["shifted"]
