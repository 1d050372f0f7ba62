"""The whole-brain step (MouseCortex): local Gaussian-ball network on the
device against the oracle's restatement (bit-exact), and MouseCortex
simulate() -- gray GABA, white GABA, white AMPA couplings then one leapfrog
step -- against the oracle composition of the same primitives (one step
within 5e-5, the leapfrog test's bound; firing counts and coupling inputs
exact)."""
import numpy as np
import pytest

import neuronephys_clean_gb300 as nn

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,stddev", [(3000, 0.1), (20000, 0.045)])
def test_local_gaussian_network(ctx, orc, n, stddev):
    rng = np.random.default_rng(n)
    pos = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    d = [ctx.to_device(np.ascontiguousarray(pos[:, a])) for a in range(3)]
    net = nn.NormalNetwork(*d, stddev=stddev, n_stddevs=2, seed=9)
    lst = net.to_adjacency_list(ctx)
    off, idx = orc.local_gaussian(pos[:, 0], pos[:, 1], pos[:, 2], stddev, 2, 9)
    assert np.array_equal(lst.offset_in_indices.numpy(), off)
    assert np.array_equal(lst.indices.numpy()[:len(idx)], idx)
    # acceptance follows exp(-d^2 / (2 stddev^2)) within the 2-stddev ball
    src = np.repeat(np.arange(n), np.diff(off))
    dist = np.linalg.norm(pos[src] - pos[idx], axis=1)
    assert dist.max() <= 2 * stddev * (1 + 1e-6) and not np.any(src == idx)


def test_mouse_cortex_step_matches_oracle(ctx, orc):
    n, seed = 3000, 5
    nn.UniformRandomNetwork.reset_engine(1)
    mc = nn.MouseCortex(ctx, n, ncouple=60, use_gray=True, stddev=0.1, seed=seed)
    rng = np.random.default_rng(3)
    host = {name: mc.ephys.get(name) for name in nn.SIM_PARAMS}   # Tcount arrays from construction
    host["V"] = rng.normal(-55, 25, n).astype(np.float32)
    host["M"] = rng.uniform(0, 0.2, n).astype(np.float32)
    host["N"] = rng.uniform(0.2, 0.5, n).astype(np.float32)
    host["H"] = rng.uniform(0.3, 0.7, n).astype(np.float32)
    for k in ("EOUTPUT", "IOUTPUT", "LOCAL_OUTPUT"):
        out = rng.uniform(0, 0.1, n).astype(np.float32)
        fire = rng.random(n) < 0.1
        out[fire] = rng.uniform(0.1001, 1.0, fire.sum()).astype(np.float32)
        host[k] = out
    host["APPCUR"] = rng.uniform(0, 2, n).astype(np.float32)
    for k, v in host.items():
        mc.ephys.set(k, v)
    ref = [host[k].astype(np.float32).copy() for k in nn.SIM_PARAMS]
    R = dict(zip(nn.SIM_PARAMS, ref))
    lists = [(mc.loc_list, "LOCAL_IN", "LOCAL_OUTPUT"), (mc.i_list, "IIN", "IOUTPUT"), (mc.e_list, "EIN", "EOUTPUT")]
    last = None
    for lst, kin, kout in lists:
        nf, inputs, _ = orc.coupling_push(lst.indices.numpy(), lst.offset_in_indices.numpy(), R[kout], 0)
        R[kin] += inputs
        last = nf
    n_firing = mc.simulate()
    assert n_firing == last
    orc.hh_leapfrog(ref, 0.4, orc.leapfrog_params(1), orc.normals(seed, n, 0))
    got = {k: mc.ephys.get(k) for k in nn.SIM_PARAMS}
    assert (np.abs(got["V"] - R["V"]) / (np.abs(R["V"]) + 1.0)).max() < 5e-5
    for k in ("M", "N", "H", "LOCAL_Y", "IY", "EY", "EOUTPUT", "IOUTPUT", "LOCAL_OUTPUT"):
        assert np.abs(got[k] - R[k]).max() < 5e-5, k
