"""Batched mode: many independent networks in one simulation (block-diagonal
ER with one p per instance, per-instance paracrine grids solved by the
batched PCG), and the launch-shape autotuner.

Tolerances: generated networks bit-exact against the oracle's single-network
generator per instance; batched PCG solutions within 1e-5 (relative 2-norm)
of FP64 CG per instance, iteration counts within 3 of the single-grid
solver's; the simulated raster of the batch equal to the FP64 oracle's for
the concatenated network (margin-aware, as the single-network test); the
autotuned simulation bit-identical to an untuned twin (pull delivery)."""
import numpy as np
import pytest

import neuronephys_clean_gb300 as nn
from tolerance import assert_rasters_match

pytestmark = pytest.mark.gpu

SIZES = [300, 800, 1500, 400, 1000]
GRIDS = [8, 12, 16, 8, 12]
P = [0.05, 0.02, 0.01, 0.04, 0.015]


def batch_sim(ctx, seed=11, delivery=0, grids=True, raster=100000, overlap=1):
    n = sum(SIZES)
    c = nn.default_config(n)
    c.seed, c.delivery, c.raster_capacity, c.grid, c.timescale = seed, delivery, raster, 0, 100
    c.par_overlap = overlap
    s = nn.Simulation(ctx, c)
    off = np.concatenate([[0], np.cumsum(SIZES)])
    s.set_instances(off, GRIDS if grids else None)
    s.generate_batch_er(P, w_max=0.5, inh_fraction=0.2)
    s.init_state(-65.0, 5.0, 15.0)
    # potentials spread over [-65, -35] mV so spikes (and deposits) start at once
    s.set_field("V", np.random.default_rng(seed).uniform(-65, -35, n).astype(np.float32))
    return s, off


def test_block_diagonal_er_matches_single_networks(ctx, orc):
    s, off = batch_sim(ctx, grids=False)
    rp, col, w, d, _ = s.get_network()
    for b, (n_b, p_b) in enumerate(zip(SIZES, P)):
        ref = orc.gen_er(n_b, p_b, 0.5, 11 + b)
        lo, hi = rp[off[b]], rp[off[b + 1]]
        assert np.array_equal(rp[off[b]:off[b + 1] + 1] - lo, ref.row_ptr)
        assert np.array_equal(col[lo:hi] - off[b], ref.col)
        assert np.array_equal(w[lo:hi], ref.weight)
        assert np.all(d[lo:hi] == 1)


def test_batched_pcg_matches_single_solves(ctx, orc):
    sides = [16, 24, 20, 32, 12]
    alpha_unit, beta = 4e-3, 1e-4
    bp = nn.BatchedPCG(ctx, sides, alpha_unit, beta)
    rng = np.random.default_rng(0)
    G = int(bp.offsets[-1])
    b = np.zeros(G, np.float32)
    b[rng.integers(0, G, 500)] += 1.0
    b += 0.01 * rng.random(G).astype(np.float32)
    db, dx = ctx.to_device(b), ctx.to_device(np.zeros(G, np.float32))
    its, bad = bp.solve(db, dx, 1e-6, 5000)
    assert bad == 0
    x = dx.numpy()
    for k, g in enumerate(sides):
        lo, hi = bp.offsets[k], bp.offsets[k + 1]
        al = alpha_unit * g * g
        ref, _, _ = orc.pcg7(b[lo:hi], np.zeros(hi - lo), (g, g, g), al, beta, rtol=1e-12)
        assert np.linalg.norm(x[lo:hi] - ref) <= 1e-5 * np.linalg.norm(ref), k
        single = nn.PCG(ctx, g, g, g, al, beta)
        xs = ctx.to_device(np.zeros(hi - lo, np.float32))
        it1, _ = single.solve(ctx.to_device(b[lo:hi]), xs, 1e-6, 5000)
        assert abs(int(its[k]) - it1) <= 3, (k, its[k], it1)


def test_batched_pcg_block_layouts_and_autotune(ctx, orc):
    """Every block layout of the batched PCG (512 .. 4,096 cells per block)
    solves each instance within 1e-5 of FP64 CG; the autotuner picks one of
    them and leaves the solver correct."""
    sides = [16, 24, 20, 32, 12]
    alpha_unit, beta = 4e-3, 1e-4
    bp = nn.BatchedPCG(ctx, sides, alpha_unit, beta)
    rng = np.random.default_rng(1)
    G = int(bp.offsets[-1])
    b = np.zeros(G, np.float32)
    b[rng.integers(0, G, 500)] += 1.0
    b += 0.01 * rng.random(G).astype(np.float32)
    db = ctx.to_device(b)
    refs = []
    for k, g in enumerate(sides):
        lo, hi = bp.offsets[k], bp.offsets[k + 1]
        refs.append(orc.pcg7(b[lo:hi], np.zeros(hi - lo), (g, g, g), alpha_unit * g * g, beta, rtol=1e-12)[0])

    def check():
        dx = ctx.to_device(np.zeros(G, np.float32))
        its, bad = bp.solve(db, dx, 1e-6, 5000)
        assert bad == 0
        x = dx.numpy()
        for k in range(len(sides)):
            lo, hi = bp.offsets[k], bp.offsets[k + 1]
            assert np.linalg.norm(x[lo:hi] - refs[k]) <= 1e-5 * np.linalg.norm(refs[k]), k
        return its

    its = [check() for cpb in (512, 1024, 2048, 4096) if bp.set_cells_per_block(cpb) is None]
    assert all(np.abs(i.astype(int) - its[2]).max() <= 2 for i in its)
    cpb, ms = bp.autotune(db, ctx.to_device(np.zeros(G, np.float32)), 8)
    assert cpb in (512, 1024, 2048, 4096) and ms > 0
    check()


def test_solver_autotune_keeps_simulation(ctx):
    """The field solver's autotuner (batched block size; single-grid tile
    depth) works on scratch vectors: the neurons stay bit-identical to an
    untuned twin's, the fields agree within the solves' tolerance (pull
    delivery: sums independent of arrival order)."""
    a, _ = batch_sim(ctx, seed=5, delivery=1)
    b, _ = batch_sim(ctx, seed=5, delivery=1)
    a.step(100)
    b.step(100)
    cpb, ms = a.autotune_solver(5)
    assert cpb in (512, 1024, 2048, 4096) and ms > 0
    a.step(200)
    b.step(200)
    for k in ("V", "M", "H", "N"):
        assert np.array_equal(a.get_field(k), b.get_field(k)), k
    ua, ub = a.get_density(), b.get_density()
    assert np.linalg.norm(ua - ub) <= 1e-4 * np.linalg.norm(ub)
    sims = []
    for tune in (True, False):
        c = nn.default_config(2000)
        c.seed, c.grid, c.timescale, c.delivery = 7, 32, 50, nn.NN_DELIVERY_PULL
        s = nn.Simulation(ctx, c)
        spec = nn.default_net_spec(nn.NN_NET_ER)
        s.generate_network(spec)
        s.init_state(-65.0, 5.0, 15.0)
        s.set_field("V", np.random.default_rng(7).uniform(-65, -35, 2000).astype(np.float32))
        s.step(50)
        if tune:
            zc, ms = s.autotune_solver(5)
            assert zc in (4, 6, 8, 12, 16, 24, 32) and ms > 0
        s.step(150)
        sims.append(s)
    for k in ("V", "M", "H", "N"):
        assert np.array_equal(sims[0].get_field(k), sims[1].get_field(k)), k
    ua, ub = sims[0].get_density(), sims[1].get_density()
    assert np.linalg.norm(ub) > 0
    assert np.linalg.norm(ua - ub) <= 1e-4 * np.linalg.norm(ub)


def test_batch_simulation_matches_oracle(ctx, orc):
    s, off = batch_sim(ctx)
    rp, col, w, d, inh = s.get_network()
    state = np.stack([s.get_field(k) for k in ("V", "M", "H", "N", "GE", "GI")])
    o = orc.Sim(orc.CSR(rp, col, w, d), inh, s.get_field("IDRIVE"), 11, 2, state)
    ref = {}
    for t in range(100):
        for j in o.step():
            ref[(t, int(j))] = o.margins[(t, int(j))]
    s.step(100)
    st, ne = s.raster()
    assert len(ref) > 50
    assert_rasters_match(set(zip(st.tolist(), ne.tolist())), ref)
    # one batched solve after 100 steps: each instance's field from its deposits
    u = s.get_density()
    vox = s.get_vox()
    G = sum(g ** 3 for g in GRIDS)
    src = np.zeros(G)
    for (t, j) in ref:
        src[vox[j]] += 1.0
    goff = np.concatenate([[0], np.cumsum(np.array(GRIDS) ** 3)])
    dt_s = 100 * s.config.hp.dt * 1e-3
    iters = s.instance_iterations()
    for b, g in enumerate(GRIDS):
        lo, hi = goff[b], goff[b + 1]
        refu, _, _ = orc.pcg7(src[lo:hi], np.zeros(hi - lo), (g, g, g), dt_s * g * g, 0.0, rtol=1e-12)
        if np.linalg.norm(refu) > 0:
            assert np.linalg.norm(u[lo:hi] - refu) <= 1e-4 * np.linalg.norm(refu), b
            assert iters[b] > 0


def test_per_instance_weight_ceiling(ctx):
    n = sum(SIZES)
    c = nn.default_config(n)
    c.seed, c.grid = 2, 0
    s = nn.Simulation(ctx, c)
    off = np.concatenate([[0], np.cumsum(SIZES)])
    s.set_instances(off)
    wmax = np.array([0.1, 0.2, 0.3, 0.4, 0.5], np.float32)
    s.generate_batch_er(P, w_max=wmax)
    rp, col, w, _, _ = s.get_network()
    for b in range(len(SIZES)):
        wb = w[rp[off[b]]:rp[off[b + 1]]]
        assert wb.max() <= wmax[b] and wb.max() > 0.5 * wmax[b]


def test_autotune_keeps_state_and_results(ctx):
    a, _ = batch_sim(ctx, seed=3, delivery=1, grids=False, raster=0)
    b, _ = batch_sim(ctx, seed=3, delivery=1, grids=False, raster=0)
    a.step(37)
    b.step(37)
    tpb, npt, ms = a.autotune(trial_steps=5)
    assert tpb in (64, 128, 256) and npt in (1, 2, 4) and ms > 0
    assert a.counters() == b.counters()
    a.step(120)
    b.step(120)
    for k in ("V", "M", "H", "N", "GE", "GI"):
        assert np.array_equal(a.get_field(k), b.get_field(k)), k
    assert a.counters() == b.counters()


def test_overlapped_batched_solve_matches_serial(ctx):
    """With no field feedback each period's batched solve runs on its own
    stream while the next period's steps run (its first iterations over all
    blocks, then the blocks of unconverged instances); the fields and the
    per-instance iteration counts equal the in-line solve's bit for bit (pull
    delivery: fixed-point sums independent of arrival order)."""
    out = []
    for overlap in (1, 0):
        s, off = batch_sim(ctx, seed=13, delivery=1, overlap=overlap)
        s.step(250)
        s.step(150)
        out.append((s.get_density(), s.instance_iterations(), s.counters()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]
    assert np.abs(out[0][0]).max() > 0
