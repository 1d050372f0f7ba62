"""The GB300 simulation step against the FP64 oracle of the same model.

Tolerances (stated per result):
* V, m, h, n after 10 ms: 1e-4 relative (floors 1 mV / 1e-3) for every neuron
  not in a spike; neurons in a spike within a 1 us spike-time shift
  (tests/tolerance.py);
* spike rasters over the first 10 ms: identical (step, neuron) sets, except
  spikes shifted by one step whose FP64 threshold crossing lies within 0.01 mV
  of the step boundary (at most 0.5 % of spikes; tests/tolerance.py);
* population spike count over 50 ms: within 1 %.
"""
import numpy as np
import pytest

import neuronephys_clean_gb300 as nn
from tolerance import assert_rasters_match, assert_trajectory, perturbed_neurons

pytestmark = pytest.mark.gpu


def make_sim(ctx, n=1000, delivery=0, seed=2024, raster=200000, grid=0, **kw):
    c = nn.default_config(n)
    c.seed = seed
    c.delivery = delivery
    c.raster_capacity = raster
    c.grid = grid
    for k, v in kw.items():
        setattr(c, k, v)
    s = nn.Simulation(ctx, c)
    spec = nn.default_net_spec(nn.NN_NET_ER)
    spec.p, spec.w_max = 0.01, 0.5
    s.generate_network(spec)
    s.init_state(-65.0, 5.0, 15.0)
    return s


def oracle_for(orc, s, seed, grid=0, vox=None):
    rp, col, w, d, inh = s.get_network()
    state = np.stack([s.get_field(k) for k in ("V", "M", "H", "N", "GE", "GI")])
    net = orc.CSR(rp, col, w, d)
    return orc.Sim(net, inh, s.get_field("IDRIVE"), seed, s.config.max_delay + 1, state,
                   vox=vox, grid_cells=grid ** 3 if grid else 0)


def gpu_state(s):
    return np.stack([s.get_field(k) for k in ("V", "M", "H", "N")])


def run_oracle(o, steps):
    """Advance the oracle; returns its raster and the state one step before the end."""
    spikes, prev = set(), None
    for t in range(steps):
        if t == steps - 1:
            prev = o.state()[:4]
        t0 = o.t
        spikes |= {(t0, int(j)) for j in o.step()}
    return spikes, prev


def perturbed(s, shifted):
    rp, col = s.get_network()[:2]
    return perturbed_neurons(shifted, rp, col, s.config.n)


def raster_set(steps, neurons):
    return set(zip(steps.tolist(), neurons.tolist()))


@pytest.mark.parametrize("delivery", [0, 1])
def test_first_10ms_parity(ctx, orc, delivery):
    seed = 2024
    s = make_sim(ctx, delivery=delivery, seed=seed)
    o = oracle_for(orc, s, seed)
    ref_spikes, prev = run_oracle(o, 1000)
    s.step(1000)
    st, ne = s.raster()
    assert len(ref_spikes) > 50
    shifted = assert_rasters_match(raster_set(st, ne), o.margins)
    assert_trajectory(gpu_state(s), o.state()[:4], prev, 0.01, exclude=perturbed(s, shifted))
    step, total = s.counters()
    assert step == 1000 and total == len(ref_spikes)


def test_population_rate_50ms(ctx, orc):
    seed = 7
    s = make_sim(ctx, seed=seed, raster=0)
    o = oracle_for(orc, s, seed)
    nref = sum(len(o.step()) for _ in range(5000))
    s.step(5000)
    _, total = s.counters()
    assert nref > 500
    assert abs(total - nref) / nref < 0.01


def test_benchmarked_configuration_parity(ctx, orc):
    """The benchmarked 1M-neuron network (Gaussian connectivity, 100
    out-edges per neuron = 1e8 synapses, lognormal(-1, 1) weights, delays
    U{1..20}, 20 % inhibitory, drive U[6, 12]) against the FP64 oracle over
    50 timesteps, started from the GPU's state (neuron fields, delay ring,
    step counter) at a period boundary inside a population burst after 2,000
    settling steps.  Tolerances as above (tests/tolerance.py), with the
    cascade rule of oracle/parity.py: in a 50-step window a one-step shift
    reaches its targets, whose inputs then arrive a step apart; differences
    downstream of an accepted shift are counted (at most 1 % of the spikes)
    and the neurons they reach (at most 1 % of the neurons) leave the
    trajectory check."""
    from oracle.parity import find_burst, window_parity
    n = 1_000_000
    c = nn.default_config(n)
    c.seed, c.max_delay, c.raster_capacity, c.grid = 1, 20, 2_000_000, 0
    s = nn.Simulation(ctx, c)
    spec = nn.default_net_spec(nn.NN_NET_GAUSS)
    spec.k, spec.sigma, spec.w_mu, spec.w_sigma, spec.dmax = 100, 0.1, -1.0, 1.0, 20
    spec.inh_fraction, spec.inh_random = 0.2, 1
    s.generate_network(spec)
    assert s.nnz == 100 * n
    s.init_state(-65.0, 6.0, 12.0)
    s.step(2000)
    find_burst(s, 50, n, max_periods=400)
    r = window_parity(s, 50)
    r.pop("_oracle")
    print({k: v for k, v in r.items() if not k.startswith("_")})
    assert r["spikes_oracle"] > 1000
    assert r["unexplained_spikes"] == 0
    assert r["shifted_spikes"] <= 0.005 * r["spikes_oracle"]
    assert r["cascade_spikes"] <= 0.01 * r["spikes_oracle"]
    assert r["excluded_neurons"] <= 0.01 * n
    assert r["trajectory_violations"] == 0, r
    s.close()


def test_push_pull_agree_and_pull_is_deterministic(ctx):
    a = make_sim(ctx, delivery=0, seed=5)
    b = make_sim(ctx, delivery=1, seed=5)
    c = make_sim(ctx, delivery=1, seed=5)
    for s in (a, b, c):
        s.step(1000)
    assert raster_set(*a.raster()) == raster_set(*b.raster())
    # the two orders of summing synaptic input differ in the last bits
    np.testing.assert_allclose(gpu_state(a), gpu_state(b), rtol=1e-3, atol=1e-3)
    assert np.array_equal(gpu_state(b), gpu_state(c))


def test_sliced_pull_matches_warp_pull(ctx, monkeypatch):
    """Pull delivery through the shared-memory bitmap (delay-sliced CSC) and
    through the warp-per-column kernel (NN_PULL_UNSLICED=1): same rasters,
    states within the last-bits spread of two summation orders; each is
    deterministic.  Gaussian network with delays 1..20, membrane potentials
    spread over [-65, -35] mV so that spikes start at once."""
    def run(unsliced):
        if unsliced:
            monkeypatch.setenv("NN_PULL_UNSLICED", "1")
        else:
            monkeypatch.delenv("NN_PULL_UNSLICED", raising=False)
        c = nn.default_config(4096)
        c.seed, c.max_delay, c.raster_capacity, c.delivery = 9, 20, 100000, 1
        s = nn.Simulation(ctx, c)
        spec = nn.default_net_spec(nn.NN_NET_GAUSS)
        spec.k, spec.dmax, spec.w_mu = 40, 20, 0.0
        s.generate_network(spec)
        assert s.pull_info()[0] == (not unsliced)
        s.init_state(-65.0, 6.0, 12.0)
        s.set_field("V", np.random.default_rng(3).uniform(-65, -35, 4096).astype(np.float32))
        s.step(400)
        return raster_set(*s.raster()), gpu_state(s), np.stack([s.get_field("GE"), s.get_field("GI")])
    a, b, u = run(False), run(False), run(True)
    assert len(a[0]) > 100
    assert a[0] == b[0] and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    assert a[0] == u[0]
    np.testing.assert_allclose(a[1], u[1], rtol=1e-3, atol=1e-3)
    np.testing.assert_allclose(a[2], u[2], rtol=1e-4, atol=1e-5)


def test_chunked_pull_many_buckets(ctx, monkeypatch):
    """The chunked pull where its (block, delay) runs fill whole chunks and
    are split by source span: 300k neurons, 100 out-edges each to uniformly
    random targets, delays U{1..3}, lognormal(-1, 1) weights.  Each gather
    block then holds ~66k entries per delay (8 full chunks of 8,192 entries)
    whose sources cover all 19 source buckets of 16,384 neurons, more than a
    chunk may span (16).  The layout facts are checked on the host from the
    network; the gather is compared with the warp-per-column kernel: same
    rasters, inputs within the spread of two summation orders, and each
    deterministic."""
    n, k, dmax = 300_000, 100, 3
    rng = np.random.default_rng(12)
    col = rng.integers(0, n, n * k).astype(np.int32)
    rp = (np.arange(n + 1, dtype=np.int64) * k)
    w = np.exp(rng.normal(-1.0, 1.0, n * k)).astype(np.float32)
    d = rng.integers(1, dmax + 1, n * k).astype(np.uint8)
    inh = (rng.random(n) < 0.2).astype(np.uint8)

    def run(unsliced):
        if unsliced:
            monkeypatch.setenv("NN_PULL_UNSLICED", "1")
        else:
            monkeypatch.delenv("NN_PULL_UNSLICED", raising=False)
        c = nn.default_config(n)
        c.seed, c.max_delay, c.raster_capacity, c.delivery = 5, dmax, 2_000_000, 1
        s = nn.Simulation(ctx, c)
        s.set_network(rp, col, w, d, inh)
        sliced, cols = s.pull_info()
        assert sliced == (not unsliced)
        s.init_state(-65.0, 6.0, 12.0)
        s.set_field("V", np.random.default_rng(4).uniform(-65, -35, n).astype(np.float32))
        s.step(100)
        return raster_set(*s.raster()), np.stack([s.get_field("GE"), s.get_field("GI")]), cols

    a = run(False)
    cols = a[2]
    # layout facts of the gather: entries per (block, delay) and the source
    # buckets they cover (the pull reads synapses by postsynaptic column)
    src = np.repeat(np.arange(n), k)
    key = (col // cols).astype(np.int64) * dmax + (d.astype(np.int64) - 1)
    per_run = np.bincount(key)
    assert per_run.min() > 8192 * 4
    buckets = np.zeros((per_run.size, (n + 16383) // 16384), bool)
    buckets[key, src // 16384] = True
    assert buckets.sum(axis=1).max() > 16
    b, u = run(False), run(True)
    assert len(a[0]) > 1000
    assert a[0] == b[0] and np.array_equal(a[1], b[1])
    assert a[0] == u[0]
    np.testing.assert_allclose(a[1], u[1], rtol=1e-4, atol=1e-5)


def test_delays_parity(ctx, orc):
    """Gaussian network with delays U{1..20}: raster and state vs the oracle."""
    n, seed = 2744, 31
    c = nn.default_config(n)
    c.seed, c.max_delay, c.raster_capacity = seed, 20, 100000
    for delivery in (0, 1):
        c.delivery = delivery
        s = nn.Simulation(ctx, c)
        spec = nn.default_net_spec(nn.NN_NET_GAUSS)
        spec.k, spec.dmax, spec.w_mu = 30, 20, 0.0
        s.generate_network(spec)
        s.init_state(-65.0, 6.0, 12.0)
        o = oracle_for(orc, s, seed)
        ref, prev = run_oracle(o, 600)
        s.step(600)
        assert len(ref) > 50
        shifted = assert_rasters_match(raster_set(*s.raster()), o.margins)
        assert_trajectory(gpu_state(s), o.state()[:4], prev, 0.01, exclude=perturbed(s, shifted))


def test_automatic_delivery_switches_and_matches_oracle(ctx, orc):
    """Automatic delivery with its threshold moved so that the periods alternate
    between push and pull.  Each change of mode carries the spikes in flight:
    the pull gather skips the ring rows of pushed steps, and leaving pull
    scatters the pulled spikes that have yet to arrive.  Raster and state
    against the oracle; raster and delay ring against a push-only run of the
    same network (same spikes, the ring's sums in another order: 1e-5)."""
    n, seed, periods = 2744, 31, 14
    sims = {}
    for delivery in (nn.NN_DELIVERY_PUSH, nn.NN_DELIVERY_AUTO):
        c = nn.default_config(n)
        c.seed, c.max_delay, c.raster_capacity, c.delivery = seed, 20, 100000, delivery
        s = nn.Simulation(ctx, c)
        spec = nn.default_net_spec(nn.NN_NET_GAUSS)
        spec.k, spec.dmax, spec.w_mu = 30, 20, 0.0
        s.generate_network(spec)
        s.init_state(-65.0, 6.0, 12.0)
        if delivery == nn.NN_DELIVERY_AUTO:
            o = oracle_for(orc, s, seed)
            ref, prev = run_oracle(o, 50 * periods)
            for k in range(periods):  # periods of 50 steps (no field)
                s.set_pull_rate(0.0 if k % 2 == 0 else 2.0)
                s.step(50)
                s.counters()  # the period's spike total is read back before the next choice
            modes, rates = s.delivery_log()
        else:
            s.step(50 * periods)
        sims[delivery] = s
    auto, push = sims[nn.NN_DELIVERY_AUTO], sims[nn.NN_DELIVERY_PUSH]
    # no rate measured for the first three periods (push); then the threshold decides
    assert modes.tolist() == [0, 0, 0] + [1 - k % 2 for k in range(3, periods)], modes
    assert (rates[:3] < 0).all() and (rates[3:] >= 0).all()
    got = raster_set(*auto.raster())
    assert len(ref) > 50
    shifted = assert_rasters_match(got, o.margins)
    assert_trajectory(gpu_state(auto), o.state()[:4], prev, 0.01, exclude=perturbed(auto, shifted))
    assert got == raster_set(*push.raster())
    np.testing.assert_allclose(auto.get_ring(), push.get_ring(), rtol=1e-5, atol=1e-5)


def test_paracrine_field(ctx, orc):
    """Deposits of 100 steps, then one 7-point backward-Euler PCG solve.  The
    membrane potentials start spread over [-65, -35] mV so spikes (and hence
    deposits) occur within the first millisecond."""
    seed, g, ts = 17, 16, 100
    s = make_sim(ctx, seed=seed, grid=g, timescale=ts, par_D=1.0, par_decay=0.5)
    s.set_field("V", np.random.default_rng(3).uniform(-65, -35, s.n).astype(np.float32))
    x, y, z = (s.get_field(k) for k in ("X", "Y", "Z"))
    ix = np.clip((x * np.float32(g)).astype(np.int32), 0, g - 1)
    iy = np.clip((y * np.float32(g)).astype(np.int32), 0, g - 1)
    iz = np.clip((z * np.float32(g)).astype(np.int32), 0, g - 1)
    vox = (ix + g * (iy + g * iz)).astype(np.int32)
    o = oracle_for(orc, s, seed, grid=g, vox=vox)
    for _ in range(ts):
        o.step()
    s.step(ts)
    src = o.src.copy()
    dt_s = ts * 0.01 * 1e-3
    alpha, beta = dt_s * 1.0 * g * g, dt_s * 0.5
    ref, it, _ = orc.pcg7(src, np.zeros(g ** 3), (g, g, g), alpha, beta, rtol=1e-12)
    got = s.density()
    st = s.solve_stats()
    assert st.converged and st.relres <= 1e-6 and st.solves == 1
    assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(ref)
    assert src.sum() > 0 and abs(src.sum() - s.counters()[1]) < 1e-6


def test_run_host_matches_device_path(ctx):
    """Bit-identical results through the host-buffer entry point (pull delivery
    is deterministic; push delivery sums with float atomics in arrival order)."""
    a = make_sim(ctx, seed=9, raster=0, delivery=1)
    b = make_sim(ctx, seed=9, raster=0, delivery=1)
    state = np.stack([a.get_field(k) for k in ("V", "M", "H", "N", "GE", "GI")]).astype(np.float32)
    out = np.empty_like(state)
    spikes = a.run_host(np.ascontiguousarray(state), 300, out)
    b.step(300)
    ref = np.stack([b.get_field(k) for k in ("V", "M", "H", "N", "GE", "GI")])
    assert np.array_equal(out, ref)
    assert spikes == b.counters()[1]


def test_non_finite_state_is_reported(ctx):
    s = make_sim(ctx, seed=1, raster=0)
    v = s.get_field("V")
    v[17] = np.nan
    s.set_field("V", v)
    s.step(2)
    with pytest.raises(nn.NNError) as e:
        s.get_field("V")
    assert e.value.status == 5


def test_invalid_network_rejected(ctx):
    c = nn.default_config(10)
    s = nn.Simulation(ctx, c)
    with pytest.raises(nn.NNError) as e:
        s.set_network(np.array([0, 1] + [1] * 9, np.int64), np.array([10], np.int32),
                      np.array([0.1], np.float32), np.array([1], np.uint8))
    assert e.value.status == 1
    with pytest.raises(nn.NNError):
        s.set_network(np.array([0, 1] + [1] * 9, np.int64), np.array([3], np.int32),
                      np.array([0.1], np.float32), np.array([2], np.uint8))  # delay > max_delay


def test_deliver_spike_list(ctx):
    """An explicit spike list pushed through the network reaches g_e / g_i of
    the targets one step later: the sum of the excitatory / inhibitory weights
    onto each neuron, decayed by one RK4 step of dg/dt = -g/tau (1e-5
    relative; FP32 sums in different orders).  The pull form runs on a
    pull-mode simulation."""
    n, mode = 3000, 0
    c = nn.default_config(n)
    c.seed, c.delivery, c.max_delay, c.raster_capacity = 4, mode, 1, 0
    c.hp.noise_sigma = 0.0
    s = nn.Simulation(ctx, c)
    spec = nn.default_net_spec(nn.NN_NET_ER)
    spec.p, spec.w_max, spec.inh_fraction = 0.02, 0.5, 0.2
    s.generate_network(spec)
    s.init_state(-65.0, 0.0, 0.0)           # at rest, no drive, no noise: no spikes of its own
    rp, col, w, d, inh = s.get_network()
    lst = np.sort(np.random.default_rng(1).choice(n, 150, replace=False)).astype(np.int32)
    s.deliver_spikes(ctx.to_device(lst), len(lst), mode)
    s.step(2)                               # step 0 reads slot 0, step 1 reads the delivered slot 1
    assert s.counters()[1] == 0
    ge = np.zeros(n)
    gi = np.zeros(n)
    for i in lst:
        tgt, wt = col[rp[i]:rp[i + 1]], w[rp[i]:rp[i + 1]].astype(np.float64)
        np.add.at(gi if inh[i] else ge, tgt, wt)
    h = c.hp.dt / c.hp.tau_exc
    decay = 1 - h + h * h / 2 - h ** 3 / 6 + h ** 4 / 24
    np.testing.assert_allclose(s.get_field("GE"), ge * decay, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(s.get_field("GI"), gi * decay, rtol=1e-5, atol=1e-6)
    c.delivery = 1
    sp = nn.Simulation(ctx, c)
    sp.generate_network(spec)
    sp.deliver_spikes(ctx.to_device(lst), len(lst), 1)
    ctx.synchronize()
    # the pull wrote the complete input of the next step into ring slot 1:
    # the same sums; the gather alone, rerun from the same bitmap, rewrites it
    # bit for bit (fixed-point sums)
    ring = sp.get_ring()
    np.testing.assert_allclose(ring[1, :, 0], ge, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(ring[1, :, 1], gi, rtol=1e-5, atol=1e-6)
    sp.pull_gather()
    assert np.array_equal(sp.get_ring(), ring)


def test_overlapped_field_solve_matches_serial(ctx):
    """With no field feedback (g_par = 0) each period's solve runs on its own
    stream while the next period's steps run; the result is bit-identical to
    solving in line (same kernels, same inputs, deterministic reductions).
    Pull delivery, whose fixed-point sums do not depend on arrival order (the
    push scatter's float atomics do, when two spikes reach one target in one
    step)."""
    out = []
    for overlap in (1, 0):
        s = make_sim(ctx, delivery=1, seed=21, grid=32, raster=0, par_overlap=overlap, timescale=100)
        s.set_field("V", np.random.default_rng(2).uniform(-65, -35, 1000).astype(np.float32))
        s.step(250)
        s.step(150)
        out.append((s.density(), gpu_state(s), s.counters(), s.solve_stats().iterations))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2] and out[0][3] == out[1][3]
    assert np.abs(out[0][0]).max() > 0
