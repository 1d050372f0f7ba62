"""Device network generators, CSC transpose and initial state against the oracle
(bit-exact for indices, delays and integer-derived values)."""
import numpy as np
import pytest

import neuronephys_clean_gb300 as nn

pytestmark = pytest.mark.gpu


def _sim(ctx, n, max_delay=1, delivery=0, **kw):
    c = nn.default_config(n)
    c.max_delay = max_delay
    c.delivery = delivery
    c.seed = kw.pop("seed", 1234)
    for k, v in kw.items():
        setattr(c, k, v)
    return nn.Simulation(ctx, c)


def test_er_generator_bit_exact(ctx, orc):
    n, p, seed = 1000, 0.01, 1234
    s = _sim(ctx, n, seed=seed)
    spec = nn.default_net_spec(nn.NN_NET_ER)
    spec.p, spec.w_max = p, 0.5
    s.generate_network(spec)
    rp, col, w, d, inh = s.get_network()
    ref = orc.gen_er(n, p, 0.5, seed)
    assert np.array_equal(rp, ref.row_ptr)
    assert np.array_equal(col, ref.col)
    assert np.array_equal(w, ref.weight)
    assert np.array_equal(d, ref.delay)
    assert inh.sum() == 200 and inh[800:].all() and not inh[:800].any()
    assert abs(len(col) / (n * (n - 1)) - p) < 0.002


def test_gauss_generator_bit_exact(ctx, orc):
    n, k, seed = 8000, 50, 99
    s = _sim(ctx, n, max_delay=20, seed=seed)
    spec = nn.default_net_spec(nn.NN_NET_GAUSS)
    spec.k, spec.sigma, spec.w_mu, spec.w_sigma, spec.dmax = k, 0.1, -1.0, 1.0, 20
    s.generate_network(spec)
    rp, col, w, d, inh = s.get_network()
    ref = orc.gen_gauss(n, k, 0.1, -1.0, 1.0, 20, seed)
    assert np.array_equal(rp, ref.row_ptr)
    assert np.array_equal(col, ref.col)
    assert np.array_equal(d, ref.delay)
    np.testing.assert_array_max_ulp(w, ref.weight, maxulp=1)
    assert d.min() >= 1 and d.max() <= 20
    assert 0.17 < inh.mean() < 0.23
    # distance dependence: mean lattice distance to targets ~ sigma * sqrt(3) * (1 - boundary effects)
    x, y, z = orc.lattice_positions(n, seed)
    src = np.repeat(np.arange(n), k)
    dist = np.sqrt((x[col] - x[src]) ** 2 + (y[col] - y[src]) ** 2 + (z[col] - z[src]) ** 2)
    assert 0.08 < dist.mean() < 0.2


def test_block_generator_structure(ctx):
    n, k = 20000, 30
    s = _sim(ctx, n, max_delay=40, seed=5)
    spec = nn.default_net_spec(nn.NN_NET_BLOCK)
    spec.k, spec.n_regions, spec.block_dmax = k, 50, 40
    s.generate_network(spec)
    rp, col, w, d, inh = s.get_network()
    assert np.array_equal(rp, np.arange(n + 1) * k)
    assert col.min() >= 0 and col.max() < n and not np.any(col == np.repeat(np.arange(n), k))
    assert d.min() >= 1 and d.max() <= 40 and np.all(w > 0)


def test_block_generator_bit_exact(ctx, orc):
    """Region-block model (the 10M-neuron workload's generator) against the
    oracle: targets and delays bit-exact, lognormal weights within 1 ulp."""
    n, k, R, seed = 12000, 40, 60, 17
    s = _sim(ctx, n, max_delay=40, seed=seed)
    spec = nn.default_net_spec(nn.NN_NET_BLOCK)
    spec.k, spec.n_regions, spec.block_dmax, spec.w_mu, spec.w_sigma = k, R, 40, -1.0, 1.0
    s.generate_network(spec)
    rp, col, w, d, _ = s.get_network()
    ref = orc.gen_block(n, k, R, spec.region_size_sigma, spec.density_sigma, 40, -1.0, 1.0, seed)
    assert np.array_equal(rp, ref.row_ptr)
    assert np.array_equal(col, ref.col)
    assert np.array_equal(d, ref.delay)
    np.testing.assert_array_max_ulp(w, ref.weight, maxulp=1)
    assert len(np.unique(d)) > 10


@pytest.mark.parametrize("kind", ["er", "gauss"])
def test_csc_bit_exact(ctx, orc, kind):
    if kind == "er":
        n = 1500
        s = _sim(ctx, n, seed=3)
        spec = nn.default_net_spec(nn.NN_NET_ER)
        spec.p = 0.02
    else:
        n = 4096
        s = _sim(ctx, n, max_delay=20, seed=3)
        spec = nn.default_net_spec(nn.NN_NET_GAUSS)
        spec.k, spec.dmax = 40, 20
    s.generate_network(spec)
    rp, col, w, d, inh = s.get_network()
    cp, src, cw, cd = s.get_csc()
    ref = orc.csr_to_csc(orc.CSR(rp, col, w, d))
    for a, b in zip((cp, src, cw, cd), ref):
        assert np.array_equal(a, b)


def test_csc_long_columns(ctx, orc):
    """Columns longer than the warp sort (1024) and the block sort paths."""
    n = 3000
    rng = np.random.default_rng(0)
    rows = [rng.integers(0, n, 40) for _ in range(n)]
    for i in range(0, n, 2):
        rows[i] = np.concatenate([rows[i], [7] * 2, [11]])   # column 7: 3000 entries, column 11: 1500
        rows[i + 1] = np.concatenate([rows[i + 1], [3] * 12])  # column 3: 18000 (rank-sort path)
    rp = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int64)
    col = np.concatenate(rows).astype(np.int32)
    w = rng.random(len(col)).astype(np.float32)
    d = np.ones(len(col), np.uint8)
    s = _sim(ctx, n)
    s.set_network(rp, col, w, d)
    got = s.get_csc()
    ref = orc.csr_to_csc(orc.CSR(rp, col, w, d))
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


def test_init_state(ctx, orc):
    n, seed = 3000, 77
    s = _sim(ctx, n, seed=seed, grid=16)
    s.init_state(-65.0, 5.0, 15.0)
    ids = s.get_field("IDRIVE")
    u = np.array([orc.philox([i, 0, 0, 2], [seed & 0xffffffff, seed >> 32])[0] for i in range(n)], np.uint32)
    u01 = (u >> 8).astype(np.float32) * np.float32(1.0 / 16777216.0)
    want = np.float32(5.0) + (np.float32(15.0) - np.float32(5.0)) * u01
    assert np.array_equal(ids, want)
    x, y, z = orc.lattice_positions(n, seed)
    assert np.array_equal(s.get_field("X"), x) and np.array_equal(s.get_field("Z"), z)
    m, h, nn_ = orc.steady_state(-65.0)
    assert np.allclose(s.get_field("M"), m, rtol=1e-6) and np.allclose(s.get_field("N"), nn_, rtol=1e-6)
    assert np.all(s.get_field("V") == -65.0)


@pytest.mark.parametrize("kind", ["er", "gauss"])
def test_init_state_drive_and_types_match_oracle(ctx, orc, kind):
    """The oracle's generators of the initial state (drive currents,
    inhibitory flags, voxels), which the CPU reference arm of the benchmark
    uses instead of the device: bit-exact against the device."""
    n, seed, g = 5000, 1, 32
    s = _sim(ctx, n, max_delay=20, seed=seed, grid=g)
    if kind == "er":
        spec = nn.default_net_spec(nn.NN_NET_ER)
        spec.p = 0.002
    else:
        spec = nn.default_net_spec(nn.NN_NET_GAUSS)
        spec.k, spec.dmax = 10, 20
    s.generate_network(spec)
    s.init_state(-65.0, 6.0, 12.0)
    assert np.array_equal(s.get_field("IDRIVE"), orc.init_drive(n, seed, 6.0, 12.0))
    assert np.array_equal(s.get_network()[4], orc.inh_flags(n, 0.2, kind == "gauss", seed))
    assert np.array_equal(s.get_vox(), orc.voxels(*orc.lattice_positions(n, seed), g))
    st = orc.rest_state(n)
    for q, f in enumerate(("V", "M", "H", "N")):
        np.testing.assert_allclose(s.get_field(f), st[q], rtol=1e-6)
