"""Electrodes, synchrony measures and the Hebbian rule on the GPU against the
numpy restatements in oracle/probes.py.  Tolerances: region means 1e-5
relative (FP32 sums in a different order), firing counts and timers exact,
chi 1e-6 relative (FP64 accumulators; sub-population sums in FP32 differ in
order), Hebbian weights 1e-5 relative after 200 updates (FP32 expf and one
rounding per update on either side)."""
import numpy as np
import pytest

import neuronephys_clean_gb300 as nn
from oracle import probes as P

pytestmark = pytest.mark.gpu


def test_electrodes(ctx):
    rng = np.random.default_rng(0)
    n, R = 5000, 40
    sizes = rng.integers(1, 300, R)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    idx = rng.integers(0, n, off[-1]).astype(np.int32)           # overlapping regions allowed
    V = rng.uniform(-80, 30, n).astype(np.float32)
    fire = (rng.random(n) < 0.1).astype(np.int32)
    e = nn.ElectrodeNet(ctx, idx, off)
    avg, fir = e.do_electrode_measurements(ctx.to_device(V), ctx.to_device(fire))
    ravg, rfir = P.electrodes_measure(idx, off, V, fire)
    np.testing.assert_allclose(avg, ravg, rtol=1e-5, atol=1e-4)
    assert np.array_equal(fir, rfir)
    m = nn.ElectrodeNet.measure_average_entire_network(ctx, ctx.to_device(V), n)
    assert abs(m - V.astype(np.float64).mean()) <= 1e-5 * abs(V).max()


def _electrode_sim(ctx, n=20000, seed=3):
    c = nn.default_config(n)
    c.seed, c.max_delay, c.raster_capacity = seed, 20, 1_000_000
    s = nn.Simulation(ctx, c)
    spec = nn.default_net_spec(nn.NN_NET_GAUSS)
    spec.k, spec.dmax = 30, 20
    s.generate_network(spec)
    s.init_state(-65.0, 6.0, 12.0)
    s.set_field("V", np.random.default_rng(seed).uniform(-65, -30, n).astype(np.float32))
    return s


@pytest.mark.parametrize("every,capacity,steps", [(3, 8, 22), (1, 4, 12)])
def test_electrodes_fused_into_step(ctx, every, capacity, steps):
    """nn_sim_set_electrodes: the recording fused into the neuron update
    against the numpy restatement of ElectrodeNet::DoElectrodeMeasurements
    (oracle/probes.py) on the states and spikes of the same steps: region
    means within 1e-5 relative (FP64 sums here, the reference's sequential
    FP32 sum there), firing counts exact.
    Overlapping regions; a ring smaller than the run keeps the last
    `capacity` samples."""
    n, R = 20000, 30
    rng = np.random.default_rng(7)
    sizes = rng.integers(1, 200, R)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    idx = rng.integers(0, n, off[-1]).astype(np.int32)
    s = _electrode_sim(ctx, n)
    s.step(41)  # into the spiking
    s.set_electrodes(idx, off, every=every, capacity=capacity)
    want = {}
    for t in range(41, 41 + steps):
        s.step(1)
        if t % every == 0:
            want[t] = s.get_field("V")
    st, ne = s.raster()
    first, avg, fire = s.read_electrodes()
    sample_steps = sorted(want)[-capacity:]
    assert first == sample_steps[0] and len(avg) == len(sample_steps)
    assert sum(len(ne[st == t]) for t in sample_steps) > 0
    for k, t in enumerate(sample_steps):
        spiked = np.zeros(n, np.int32)
        spiked[ne[st == t]] = 1
        ravg, rfire = P.electrodes_measure(idx, off, want[t], spiked)
        np.testing.assert_allclose(avg[k], ravg, rtol=1e-5, atol=1e-4)
        assert np.array_equal(fire[k], rfire), t
    s.set_electrodes(idx, off, every=0)
    assert s.read_electrodes()[1].shape[0] == 0
    s.close()


def test_synchrony(ctx):
    rng = np.random.default_rng(1)
    n = 4000
    inds = rng.permutation(n)[:1000].astype(np.int32)
    sub = [10, 100, 1000]
    s = nn.SynchronyNet(ctx, inds, sub)
    o = P.SynchronyOracle(inds, sub)
    common = rng.standard_normal(60)
    for t in range(60):
        V = (-60 + 5 * common[t] + rng.standard_normal(n) * 3).astype(np.float32)
        s.measure_variances(ctx.to_device(V))
        o.measure(V)
    np.testing.assert_allclose(s.get_synchrony_measures(), o.chi(), rtol=1e-6)


def test_hebbian_matches_full_sweep(ctx):
    """The active-row update equals the reference's sweep over all synapses."""
    rng = np.random.default_rng(2)
    n, k = 2000, 50
    deg = rng.integers(0, 2 * k, n)
    off = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
    col = rng.integers(0, n, off[-1]).astype(np.int32)
    w = rng.uniform(0, 2, off[-1]).astype(np.float32)
    window, inc = 10, 0.1
    h = nn.Hebbian(ctx, window, inc, off[-1], n)
    dcol, doff, dw = ctx.to_device(col), ctx.to_device(off), ctx.to_device(w)
    rw, rt = w.copy(), np.zeros(off[-1], np.int64)
    for t in range(200):
        fire = (rng.random(n) < 0.03).astype(np.int32)
        lst = np.nonzero(fire)[0].astype(np.int32)
        h.update_weights(dcol, doff, dw, ctx.to_device(fire), ctx.to_device(lst) if len(lst) else None, len(lst))
        P.hebbian_update(col, off, rw, rt, fire, lst, window, inc)
    assert np.array_equal(h.timers(), rt)
    np.testing.assert_allclose(dw.numpy(), rw, rtol=1e-5, atol=1e-6)
    assert not np.array_equal(rw, w)
