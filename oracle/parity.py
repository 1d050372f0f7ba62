"""Parity criteria of the simulation step against the FP64 oracle.  TEST
INFRASTRUCTURE ONLY: used by tests/ (through tests/tolerance.py, which turns
them into assertions) and by bench.py's CPU-baseline leg, which reports them.

FP32 device state against the FP64 oracle: rounding differences of ~1e-7 are
amplified only at spike initiation, where the upstroke is unstable; a neuron
caught mid-spike at the checkpoint can differ by ~1e-3 relative although its
spike time agrees to well under a microsecond.  The trajectory criterion is
therefore stated per neuron:

* |dV/dt| < 20 mV/ms at the checkpoint (not in a spike): every variable within
  ``rtol`` = 1e-4 relative, with floors of 1 mV for V and 1e-3 for gates;
* steep neurons (in a spike): each variable's difference below its rate of
  change times a spike-time shift of 1 us (|dx/dt| * 1e-3 ms), plus the
  1e-4-relative allowance.

Rasters, as sets of (step, neuron): identical, except that a spike may sit
one step earlier or later when the FP64 oracle's threshold crossing lies within
MARGIN_MV = 0.01 mV of the step boundary (V before or after the crossing step
within 0.01 mV of the threshold).  This relaxes "identical rasters": a
crossing that close to the boundary is decided by the last bits of an FP32
potential, whose rounding the FP64 oracle does not share.  Shifted spikes are
counted and bounded (0.5 % of the spikes in the tests).  In a window long
enough for a shifted spike to reach its targets (delays >= 1 step), the
targets' input arrives one step apart and their own spikes may move too: with
the network given, such differences downstream of an accepted one are counted
as its cascade, and every neuron they reach leaves the trajectory check.
"""
from __future__ import annotations

import numpy as np

STEEP_MV_PER_MS = 20.0
SHIFT_MS = 1e-3
MARGIN_MV = 0.01
FLOORS = (1.0, 1e-3, 1e-3, 1e-3)


def trajectory_errors(got: np.ndarray, ref: np.ndarray, ref_prev: np.ndarray, dt_ms: float,
                      rtol: float = 1e-4) -> dict:
    """got/ref/ref_prev: (4, n) arrays of V, m, h, n.  Returns violation counts
    and the error statistics used in reports."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    rate = np.abs(ref - np.asarray(ref_prev, np.float64)) / dt_ms
    steep = rate[0] >= STEEP_MV_PER_MS
    floors = np.array(FLOORS)[:, None]
    err = np.abs(got - ref)
    rel = err / (np.abs(ref) + floors)
    allow = rtol * (np.abs(ref) + floors)
    allow_steep = allow + rate * SHIFT_MS
    bad_flat = (err > allow) & ~steep[None, :]
    bad_steep = (err > allow_steep) & steep[None, :]
    return {
        "violations": int(bad_flat.sum() + bad_steep.sum()),
        "steep_neurons": int(steep.sum()),
        "max_rel_flat": float(rel[:, ~steep].max()) if (~steep).any() else 0.0,
        "max_rel_all": float(rel.max()),
        "median_rel": float(np.median(rel)),
    }


def compare_rasters(got: set, ref_margins: dict, margin_mv: float = MARGIN_MV, row_ptr=None, col=None) -> dict:
    """got: device raster as a set of (step, neuron); ref_margins: the
    oracle's spikes mapped to their threshold-crossing margin (mV).

    A spike present on one side only is explained when
    * it is one step from the other side's spike of the same neuron and the
      oracle's crossing lies within margin_mv of the threshold (a root
      difference: FP32 rounding decides the step), or
    * (with the network given) its neuron was perturbed before it: the neuron
      is a target of an earlier explained difference, so its input arrived one
      step apart or not at all (a cascade of a root difference).
    Explained differences perturb their neuron and its targets from then on.
    Returns the root shifts, the cascaded differences, the unexplained ones
    and the perturbed neurons."""
    ref = set(ref_margins)
    only_ref, only_got = ref - got, set(got - ref)
    perturbed_at: dict[int, int] = {}

    def perturb(j: int, t: int) -> None:
        for k in ([j] + (col[row_ptr[j]:row_ptr[j + 1]].tolist() if row_ptr is not None else [])):
            if perturbed_at.get(k, t + 1) > t:
                perturbed_at[k] = t

    def caused(j: int, t: int) -> bool:
        return j in perturbed_at and perturbed_at[j] < t

    shifted, cascade, unexplained_ref, unexplained_got = [], [], [], []
    events = sorted([(t, 0, j) for (t, j) in only_ref] + [(t, 1, j) for (t, j) in only_got])
    done = set()
    for (t, side, j) in events:
        if (t, side, j) in done:
            continue
        if side == 0:
            partner = next(((t + d, j) for d in (-1, 1) if (t + d, j) in only_got and (t + d, 1, j) not in done), None)
            if partner is not None and (ref_margins[(t, j)] < margin_mv or caused(j, min(t, partner[0]))):
                (shifted if ref_margins[(t, j)] < margin_mv else cascade).append((t, j))
                done.add((partner[0], 1, j))
                perturb(j, min(t, partner[0]))
            elif caused(j, t):
                cascade.append((t, j))
                perturb(j, t)
            else:
                unexplained_ref.append((t, j))
        else:
            partner = next(((t + d, j) for d in (-1, 1) if (t + d, j) in only_ref and (t + d, 0, j) not in done), None)
            if partner is not None and (ref_margins[partner] < margin_mv or caused(j, min(t, partner[0]))):
                (shifted if ref_margins[partner] < margin_mv else cascade).append(partner)
                done.add((partner[0], 0, j))
                perturb(j, min(t, partner[0]))
            elif caused(j, t):
                cascade.append((t, j))
                perturb(j, t)
            else:
                unexplained_got.append((t, j))
    return {"identical": not only_ref and not only_got, "spikes_device": len(got), "spikes_oracle": len(ref),
            "shifted": shifted, "cascade": cascade, "unexplained_oracle": unexplained_ref,
            "unexplained_device": unexplained_got, "perturbed": sorted(perturbed_at)}


def perturbed_neurons(shifted, row_ptr, col, n) -> np.ndarray:
    """Neurons whose spike was shifted by one step, and their targets (they
    received that input one step apart)."""
    mask = np.zeros(n, bool)
    for (_, j) in shifted:
        mask[j] = True
        mask[col[row_ptr[j]:row_ptr[j + 1]]] = True
    return mask


def find_burst(sim, period: int, n: int, max_periods: int = 150) -> int:
    """Advance a simulation by whole periods until one holds at least 1e-3 of
    the neurons in spikes, so that the next window starts inside a population
    burst.  Returns the periods advanced (max_periods when none came)."""
    _, s0 = sim.counters()
    for k in range(max_periods):
        sim.step(period)
        _, s1 = sim.counters()
        if s1 - s0 >= max(100, n // 1000):
            return k + 1
        s0 = s1
    return max_periods


def window_parity(sim, steps: int) -> dict:
    """Advance a simulation (the library's Simulation) and the FP64 oracle
    `steps` timesteps from the simulation's present state: its neuron fields,
    delay ring and step counter, the complete state a step depends on.
    Returns the comparison (rasters and per-neuron trajectories as above)
    plus the oracle object, its wall time and the spiking neurons."""
    import time

    from . import CSR, Sim
    n = sim.config.n
    rp, col, w, d, inh = sim.get_network()
    state6 = np.stack([sim.get_field(f) for f in ("V", "M", "H", "N", "GE", "GI")])
    ring = sim.get_ring()
    t0, _ = sim.counters()
    o = Sim(CSR(rp, col, w, d), inh, sim.get_field("IDRIVE"), sim.config.seed, ring.shape[0], state6)
    o.ring[:] = ring.astype(np.float64).ravel()
    o.t = t0
    prev = None
    tc = time.perf_counter()
    for q in range(steps):
        if q == steps - 1:
            prev = o.state()[:4]
        o.step()
    t_oracle = time.perf_counter() - tc
    sim.reset_raster()
    sim.step(steps)
    st, ne = sim.raster()
    got = {(int(a), int(b)) for a, b in zip(st, ne) if t0 <= a < t0 + steps}
    gpu = np.stack([sim.get_field(f) for f in ("V", "M", "H", "N")])
    ref = o.state()[:4]
    r = compare_rasters(got, o.margins, row_ptr=rp, col=col)
    excl = np.zeros(n, bool)
    excl[np.asarray(r["perturbed"], np.int64)] = True
    e = trajectory_errors(gpu[:, ~excl], ref[:, ~excl], prev[:, ~excl], 0.01)
    steep = np.abs(ref[0] - prev[0]) / 0.01 >= STEEP_MV_PER_MS
    flat = ~steep & ~excl
    rel_v = np.abs(gpu[0, flat].astype(np.float64) - ref[0, flat]) / (np.abs(ref[0, flat]) + 1.0)
    floors = np.array(FLOORS)[:, None]
    rel_ex = (np.abs(gpu[:, excl] - ref[:, excl]) / (np.abs(ref[:, excl]) + floors)).max() if excl.any() else 0.0
    return {
        "steps": steps, "start_step": int(t0),
        "spikes_gpu": r["spikes_device"], "spikes_oracle": r["spikes_oracle"],
        "raster_identical": r["identical"], "shifted_spikes": len(r["shifted"]),
        "cascade_spikes": len(r["cascade"]),
        "unexplained_spikes": len(r["unexplained_oracle"]) + len(r["unexplained_device"]),
        "max_rel_V_nonspiking": float(rel_v.max()) if flat.any() else None,
        "trajectory_violations": e["violations"], "steep_neurons": e["steep_neurons"],
        "max_rel_all": e["max_rel_all"], "excluded_neurons": int(excl.sum()),
        "max_rel_excluded": float(rel_ex),
        "_oracle": o, "_t_oracle_s": t_oracle,
    }
