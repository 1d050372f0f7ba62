"""Small, self-contained GPU cases for kernel profiling (ncu captures).

    python -m neuronephys_clean_gb300.profile_cases hh1m     # 2 steps, 1M neurons, 128^3 grid
    python -m neuronephys_clean_gb300.profile_cases cg128    # 3 PCG iterations, 128^3, constant D
    python -m neuronephys_clean_gb300.profile_cases cghet    # 3 PCG iterations, 128^3, lognormal D
    python -m neuronephys_clean_gb300.profile_cases conv128  # 3x3x3 convs (16->16, 48->16) + wgrad at 128^3
    python -m neuronephys_clean_gb300.profile_cases mg256    # multigrid FCG solve to 1e-6, 256^3, lognormal D
    python -m neuronephys_clean_gb300.profile_cases lmg256   # the same with the learned 32^3 level (20 training steps)
    python -m neuronephys_clean_gb300.profile_cases pull1m   # one pull gather, 1M neurons, 1e8 synapses, delays 1..20
    python -m neuronephys_clean_gb300.profile_cases burst1m  # 200 steps of the 1M-neuron workload from rest: its first burst
    python -m neuronephys_clean_gb300.profile_cases burst1m_steps  # its first 400 steps timed one by one (no ncu)

Each case holds a few GB at most and launches a handful of kernels, so that
an ncu capture of it ends by itself; every case also runs without ncu.
"""
from __future__ import annotations

import sys

import numpy as np

import neuronephys_clean_gb300 as nn


def hh1m(ctx):
    c = nn.default_config(1_000_000)
    c.seed, c.max_delay, c.grid, c.timescale = 1, 20, 128, 100
    c.par_D, c.par_rtol, c.par_max_iter = 1.0, 1e-6, 8
    s = nn.Simulation(ctx, c)
    sp = nn.default_net_spec(nn.NN_NET_GAUSS)
    sp.k, sp.dmax = 10, 20
    s.generate_network(sp)
    s.init_state(-65.0, 6.0, 12.0)
    s.set_field("V", np.random.default_rng(0).uniform(-70, -30, 1_000_000).astype(np.float32))
    s.step(2)


def _pcg(ctx, D=None):
    n = 128
    dD = None if D is None else ctx.to_device(D.ravel())
    pc = nn.PCG(ctx, n, n, n, 16.384, 0.0, dD)
    b = ctx.to_device(np.random.default_rng(1).random(n ** 3).astype(np.float32))
    x = ctx.to_device(np.zeros(n ** 3, np.float32))
    try:
        pc.solve(b, x, rtol=1e-6, max_iter=3)
    except nn.NNError as e:
        if e.status != nn.NN_ERR_NOT_CONVERGED:
            raise


def cg128(ctx):
    _pcg(ctx)


def cghet(ctx):
    from neuronephys_clean_gb300 import fields
    _pcg(ctx, fields.lognormal_diffusivity((128, 128, 128), 1.0, 8.0, seed=1))


def conv128(ctx):
    shape = (128, 128, 128)
    rng = np.random.default_rng(2)
    for cin, cout in [(16, 16), (48, 16)]:
        a = nn.Activation(ctx, shape, cin)
        a.pack(ctx.to_device(rng.standard_normal((cin,) + shape).astype(np.float32)))
        w = ctx.to_device((rng.standard_normal((27, cin, cout)) * 0.05).astype(np.float32))
        wp = nn.conv3d_pack_weights(ctx, w, cin, cout)
        y = nn.Activation(ctx, shape, cout)
        nn.conv3d_forward(ctx, a, wp, y, relu=True)
        dw = ctx.to_device(np.zeros((27, cin, cout), np.float32))
        nn.conv3d_wgrad(ctx, a, y, dw)


def mg256(ctx):
    from neuronephys_clean_gb300 import fields
    n = 256
    D = ctx.to_device(fields.lognormal_diffusivity((n, n, n), 1.0, 8.0, seed=1).ravel())
    b = ctx.to_device(fields.spike_sources((n, n, n), 20000, 2.0, seed=2))
    pc = nn.PCG(ctx, n, n, n, 1e-3 * n * n, 1e-4, D)
    mg = nn.MultigridPCG(pc)
    x = ctx.to_device(np.zeros(n ** 3, np.float32))
    mg.solve(b, x, rtol=1e-6)


def lmg256(ctx):
    from neuronephys_clean_gb300 import fields
    n = 256
    D = ctx.to_device(fields.lognormal_diffusivity((n, n, n), 1.0, 8.0, seed=1).ravel())
    b = fields.spike_sources((n, n, n), 20000, 2.0, seed=2)
    pc = nn.PCG(ctx, n, n, n, 1e-3 * n * n, 1e-4, D)
    lm = nn.LearnedMultigrid(pc, level=3)
    lm.add_solves([fields.spike_sources((n, n, n), 20000, 2.0, seed=3)])
    lm.train(20)
    x = ctx.to_device(np.zeros(n ** 3, np.float32))
    lm.solve(ctx.to_device(b), x, rtol=1e-6)


def pull1m(ctx):
    n = 1_000_000
    c = nn.default_config(n)
    c.seed, c.max_delay, c.delivery = 1, 20, nn.NN_DELIVERY_PULL
    s = nn.Simulation(ctx, c)
    sp = nn.default_net_spec(nn.NN_NET_GAUSS)
    sp.k, sp.sigma, sp.w_mu, sp.w_sigma, sp.dmax = 100, 0.1, -1.0, 1.0, 20
    s.generate_network(sp)
    s.init_state(-65.0, 0.0, 0.0)
    s.step(21)  # past the longest delay: the gather covers every delay slice
    lst = np.sort(np.random.default_rng(5).choice(n, 1000, replace=False)).astype(np.int32)
    s.deliver_spikes(ctx.to_device(lst), len(lst), nn.NN_DELIVERY_PULL)


def _burst_sim(ctx):
    n = 1_000_000
    c = nn.default_config(n)
    c.seed, c.max_delay = 1, 20
    s = nn.Simulation(ctx, c)
    sp = nn.default_net_spec(nn.NN_NET_GAUSS)
    sp.k, sp.sigma, sp.w_mu, sp.w_sigma, sp.dmax = 100, 0.1, -1.0, 1.0, 20
    sp.inh_fraction, sp.inh_random = 0.2, 1
    s.generate_network(sp)
    s.init_state(-65.0, 6.0, 12.0)
    return s


def burst1m_steps(ctx):
    """The same 400 steps one at a time, each timed with CUDA events, printed
    as step time against spikes per step (JSON)."""
    import json
    s = _burst_sim(ctx)
    ms, spk = [], []
    _, t0 = s.counters()
    for _ in range(400):
        ctx.time_begin()
        s.step(1)
        ms.append(ctx.time_end())
        _, t1 = s.counters()
        spk.append(t1 - t0)
        t0 = t1
    ms, spk = np.array(ms), np.array(spk)
    out = {"quiet_median_ms": float(np.median(ms[spk < 10]))}
    for lo, hi in ((10, 1000), (1000, 5000), (5000, 20000), (20000, 10 ** 9)):
        m = (spk >= lo) & (spk < hi)
        if m.any():
            out[f"spikes_{lo}_{hi}"] = {"steps": int(m.sum()), "mean_ms": float(ms[m].mean()),
                                        "mean_spikes": float(spk[m].mean())}
    print(json.dumps(out))


def burst1m(ctx):
    """The 1M-neuron workload (Gaussian network, 100 synapses per neuron,
    delays 1..20, no field) for 200 steps from rest: its first population
    burst (the neuron updates from step ~120 on carry thousands of spikes per
    step, pushed inside the kernel)."""
    _burst_sim(ctx).step(200)


CASES = {"hh1m": hh1m, "cg128": cg128, "cghet": cghet, "conv128": conv128, "mg256": mg256, "lmg256": lmg256,
         "pull1m": pull1m,
         "burst1m": burst1m, "burst1m_steps": burst1m_steps}


def main(argv: list[str]) -> None:
    names = argv or [c for c in CASES if c != "burst1m_steps"]
    ctx = nn.Context(0)
    for name in names:
        CASES[name](ctx)
        ctx.synchronize()
        print(f"{name} done", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
