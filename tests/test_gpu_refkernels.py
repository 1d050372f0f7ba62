"""The library's reference-semantics kernels against the reference's own CUDA
kernels, compiled from its sources (src/ephys.cu, src/coupling.cu and their
src_wholebrain variants) and run on the same GPU through the driver-API
harness in oracle/.

* Leapfrog_HH (src/ephys.cu:28-96; src_wholebrain/ephys.cu:149-217) vs
  nn_hh_leapfrog_step_z on the same state and the same standard-normal draws
  (injected into the reference's curand states): one step, every variable of
  every neuron within 2 float ulps (the count of bit-identical values is
  reported); 25 steps (10 ms at dt = 0.4 ms) with fresh draws each step,
  every neuron within 1e-5 relative (floors 1 mV / 1e-3).  The oracle's FP64
  restatement (oracle.c) is held to the reference kernel's one step within
  5e-5.
* signal_spikes_kernel, count mode (src/coupling.cu:34-48) vs nn_coupling_run:
  bit-exact (integer-valued float sums), with the firing list of
  CheckFiringOperator (src/coupling.cu:103-109) equal to the library's
  compaction.
* signal_spikes_kernel, output mode (src_wholebrain/coupling.cu:12-33) vs
  nn_coupling_run(NN_SIGNAL_OUTPUT): FP32 atomic sums within 1e-5 relative of
  each other (both add the same terms in different orders).
* signal_spikes_kernel_chunked + merge_kernel (src/coupling.cu:50-101, valid
  for N <= 14,638) vs nn_coupling_run_chunked on the reference's chunk lists.
"""
import numpy as np
import pytest

import neuronephys_clean_gb300 as nn
from neuronephys_clean_gb300 import SIM_PARAMS

pytestmark = pytest.mark.gpu

refkern = pytest.importorskip("oracle.refkern")
if not refkern.RefKernels.available():
    pytest.skip("reference kernel cubins not built (needs the reference checkout where oracle/build.py ran)",
                allow_module_level=True)


@pytest.fixture(scope="module")
def rk(ctx):
    return refkern.RefKernels(0)


def random_state(n, seed):
    """A state spread over the whole range the kernel meets: potentials from
    -80 to +30 mV (rest, threshold region, spike), gates in (0, 1), synaptic
    inputs and counts as the coupling writes them, applied currents."""
    rng = np.random.default_rng(seed)
    st = {k: np.zeros(n, np.float32) for k in SIM_PARAMS}
    st["V"] = rng.uniform(-80.0, 30.0, n).astype(np.float32)
    # a few neurons exactly at the removable singularities of alpha_m / alpha_n
    st["V"][:4] = [-35.0, -50.0, -35.0, -50.0]
    for k in ("M", "N", "H"):
        st[k] = rng.uniform(0.0, 1.0, n).astype(np.float32)
    for k in ("LOCAL_Y", "IY", "EY"):
        st[k] = rng.uniform(0.0, 0.6, n).astype(np.float32)
    for pre in ("LOCAL", "I", "E"):
        cnt = rng.integers(0, 12, n).astype(np.float32)
        st[f"{pre}_COUNT" if pre == "LOCAL" else f"{pre}COUNT"] = cnt
        st[f"{pre}_IN" if pre == "LOCAL" else f"{pre}IN"] = (cnt * rng.uniform(0, 1, n)).astype(np.float32)
    st["APPCUR"] = rng.uniform(0.0, 5.0, n).astype(np.float32)
    return st


class RefTable:
    """The reference's SoA: 17 device arrays and a device table of their
    pointers (thrust::device_vector<Float*> in src/main.cu:254)."""

    def __init__(self, ctx, st):
        self.ctx = ctx
        self.vars = [ctx.to_device(st[k]) for k in SIM_PARAMS]
        self.table = ctx.to_device(np.array([v.value for v in self.vars], np.uint64))

    def get(self, k):
        return self.vars[SIM_PARAMS.index(k)].numpy()


def ours_from(ctx, st, variant):
    e = nn.HHEphys(ctx, len(st["V"]), variant=variant)
    for k, v in st.items():
        e.set(k, v)
    return e


def ulps(a, b):
    ai = a.view(np.int32).astype(np.int64)
    bi = b.view(np.int32).astype(np.int64)
    ai = np.where(ai < 0, -(ai & 0x7fffffff), ai)
    bi = np.where(bi < 0, -(bi & 0x7fffffff), bi)
    return np.abs(ai - bi)


STATE_KEYS = ("V", "M", "N", "H", "LOCAL_Y", "IY", "EY", "LOCAL_OUTPUT", "IOUTPUT", "EOUTPUT")


@pytest.mark.parametrize("variant", [0, 1])
def test_leapfrog_one_step_matches_reference_kernel(ctx, rk, variant):
    n, dt = 20000, 0.4
    st = random_state(n, 11 + variant)
    ref = RefTable(ctx, st)
    ours = ours_from(ctx, st, variant)
    z = np.random.default_rng(3).standard_normal(n).astype(np.float32)
    states = ctx.to_device(refkern.xorwow_states_with_draw(z).view(np.uint8))
    dz = ctx.to_device(z)
    ctx.synchronize()
    rk.leapfrog(ref.table.value, n, dt, states.value, variant=variant)
    ours.simulate_ephys(z=dz)
    ctx.synchronize()
    worst, exact = 0, 0
    for k in STATE_KEYS:
        a, b = ours.get(k), ref.get(k)
        assert np.all(np.isfinite(a)) and np.all(np.isfinite(b[4:])), k
        u = ulps(a[4:], b[4:])
        worst = max(worst, int(u.max()))
        exact += int((u == 0).sum())
    print(f"variant {variant}: max {worst} ulp, {exact} of {len(STATE_KEYS) * (n - 4)} values bit-identical")
    assert worst <= 2
    # the oracle's FP64 restatement of the same step (oracle.c) against the
    # reference kernel: 5e-5 (1 mV floor for V)
    import oracle
    host = [st[k].copy() for k in SIM_PARAMS]
    oracle.hh_leapfrog(host, dt, oracle.leapfrog_params(variant), z.astype(np.float64))
    o = dict(zip(SIM_PARAMS, host))
    b = ref.get("V")[4:].astype(np.float64)
    assert (np.abs(o["V"][4:] - b) / (np.abs(b) + 1.0)).max() < 5e-5
    for k in ("M", "N", "H", "LOCAL_Y", "IY", "EY", "LOCAL_OUTPUT"):
        assert np.abs(o[k][4:] - ref.get(k)[4:]).max() < 5e-5, k
    # the removable singularities: the reference divides 0/0 only where the
    # FP64 argument is exactly 0; the library takes the limit there
    assert np.all(np.isfinite(ours.get("M")[:4])) and np.all(np.isfinite(ours.get("N")[:4]))


def physiological_state(n, seed):
    """Potentials from -75 to -40 mV with gates at their steady state there
    (rate functions of src/ephys.cu:57-63), so that 10 ms of dynamics stay
    physiological: random gates far from the manifold (M = 0.9 at -80 mV)
    drive the model to overflow within a few steps, in the reference kernel,
    in the FP64 oracle and here alike."""
    st = random_state(n, seed)
    rng = np.random.default_rng(seed + 1000)
    V = rng.uniform(-75.0, -40.0, n)
    am = (3.5 + 0.1 * V) / (1 - np.exp(-3.5 - 0.1 * V))
    an = (-0.5 - 0.01 * V) / (np.exp(-5 - 0.1 * V) - 1)
    ah = 0.07 * np.exp(-V / 20 - 3)
    bm = 4 * np.exp(-(V + 60) / 18)
    bn = 0.125 * np.exp(-(V + 60) / 80)
    bh = 1 / (np.exp(-3 - 0.1 * V) + 1)
    st["V"] = V.astype(np.float32)
    st["M"] = (am / (am + bm)).astype(np.float32)
    st["N"] = (an / (an + bn)).astype(np.float32)
    st["H"] = (ah / (ah + bh)).astype(np.float32)
    for k in ("LOCAL_Y", "IY", "EY"):
        st[k] = rng.uniform(0.0, 0.3, n).astype(np.float32)
    return st


@pytest.mark.parametrize("variant", [0, 1])
def test_leapfrog_25_steps_matches_reference_kernel(ctx, rk, variant):
    n, dt, steps = 20000, 0.4, 25
    st = physiological_state(n, 21 + variant)
    ref = RefTable(ctx, st)
    ours = ours_from(ctx, st, variant)
    rng = np.random.default_rng(5)
    dz = ctx.empty((n,), np.float32)
    states = ctx.empty((n * refkern.XORWOW_DTYPE.itemsize,), np.uint8)
    for _ in range(steps):
        z = rng.standard_normal(n).astype(np.float32)
        dz.copy_from(z)
        states.copy_from(refkern.xorwow_states_with_draw(z).view(np.uint8))
        ctx.synchronize()
        rk.leapfrog(ref.table.value, n, dt, states.value, variant=variant)
        ours.simulate_ephys(z=dz)
    ctx.synchronize()
    floors = {"V": 1.0}
    worst = {}
    for k in ("V", "M", "N", "H", "LOCAL_Y", "IY", "EY", "LOCAL_OUTPUT"):
        a, b = ours.get(k).astype(np.float64), ref.get(k).astype(np.float64)
        rel = np.abs(a - b) / (np.abs(b) + floors.get(k, 1e-3))
        worst[k] = float(rel.max())
    identical = all(np.array_equal(ours.get(k), ref.get(k)) for k in STATE_KEYS)
    spiking = int((ours.get("LOCAL_OUTPUT") > 0.1).sum())
    print(f"variant {variant}, {steps} steps: bit-identical {identical}, max relative difference per variable "
          f"{worst}, {spiking} neurons above the firing threshold at the end")
    assert spiking > 0
    assert max(worst.values()) <= 1e-5, worst


def random_csr(n, k_lo, k_hi, seed):
    rng = np.random.default_rng(seed)
    deg = rng.integers(k_lo, k_hi + 1, n)
    off = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
    idx = rng.integers(0, n, int(off[-1])).astype(np.int32)
    return idx, off


def test_signal_spikes_count_mode_bit_exact(ctx, rk):
    n = 50000
    idx, off = random_csr(n, 0, 60, 1)
    outputs = np.random.default_rng(2).uniform(0.0, 0.35, n).astype(np.float32)  # ~71 % above 0.1
    d_idx, d_off, d_out = ctx.to_device(idx), ctx.to_device(off), ctx.to_device(outputs)
    coup = nn.AtomicCoupling(ctx, n)
    ours = ctx.empty((n,), np.float32)
    nf = coup(nn.AdjacencyList(d_idx, d_off), ours, d_out)
    firing = np.nonzero(outputs > 0.1)[0].astype(np.int32)  # CheckFiringOperator + copy_if
    assert nf == len(firing)
    assert np.array_equal(coup.get_firing_neurons()[:nf], firing)
    d_fire = ctx.to_device(firing)
    spikes = ctx.empty((n,), np.float32)
    spikes.zero()
    ctx.synchronize()
    rk.signal_spikes(nf, d_idx.value, d_off.value, d_fire.value, spikes.value, d_out.value)
    ref = spikes.numpy()
    got = ours.numpy()
    assert ref.sum() == float(sum(off[j + 1] - off[j] for j in firing))
    assert np.array_equal(got, ref)
    coup.close()


def test_signal_spikes_output_mode_wholebrain(ctx, rk):
    n = 30000
    idx, off = random_csr(n, 0, 40, 3)
    outputs = np.random.default_rng(4).uniform(0.0, 1.0, n).astype(np.float32)
    d_idx, d_off, d_out = ctx.to_device(idx), ctx.to_device(off), ctx.to_device(outputs)
    coup = nn.AtomicCoupling(ctx, n)
    ours = ctx.empty((n,), np.float32)
    nf = coup(nn.AdjacencyList(d_idx, d_off), ours, d_out, signal_mode=nn.NN_SIGNAL_OUTPUT)
    firing = np.nonzero(outputs > 0.1)[0].astype(np.int32)
    assert nf == len(firing)
    d_fire = ctx.to_device(firing)
    spikes = ctx.empty((n,), np.float32)
    spikes.zero()
    ctx.synchronize()
    rk.signal_spikes(nf, d_idx.value, d_off.value, d_fire.value, spikes.value, d_out.value,
                     variant=refkern.WHOLEBRAIN)
    np.testing.assert_allclose(ours.numpy(), spikes.numpy(), rtol=1e-5, atol=1e-6)
    coup.close()


def test_signal_spikes_chunked_matches_reference_kernel(ctx, rk):
    """The reference's chunked path at its largest valid size, N = NCHUNKS *
    N_PER_CHUNK = 14,638: the library's chunk lists (bit-exact against the
    reference's ToChunkedAdjacencyList by the golden tests) fed to both."""
    n, npc = refkern.NCHUNKS * refkern.N_PER_CHUNK, refkern.N_PER_CHUNK
    idx, off = random_csr(n, 0, 30, 7)
    net = nn.Network()
    net.indices, net.offset_in_indices = idx, off
    tcount = ctx.empty((n,), np.float32)
    ch = net.to_chunked_adjacency_list(ctx, tcount, refkern.NCHUNKS, npc)
    outputs = np.random.default_rng(8).uniform(0.0, 0.5, n).astype(np.float32)
    d_out = ctx.to_device(outputs)
    coup = nn.AtomicCoupling(ctx, n)
    ours = ctx.empty((n,), np.float32)
    nf = coup(ch, ours, d_out)
    firing = np.nonzero(outputs > 0.1)[0].astype(np.int32)
    assert nf == len(firing)
    d_fire = ctx.to_device(firing)
    conn_tab = ctx.to_device(np.array([a.value for a in ch.indices_chunks], np.uint64))
    off_tab = ctx.to_device(np.array([a.value for a in ch.offset_in_indices_chunks], np.uint64))
    copies = ctx.empty((refkern.NBLOCKS * refkern.NCHUNKS * npc,), np.float32)
    spikes = ctx.empty((refkern.NCHUNKS * npc,), np.float32)
    want = np.zeros(n, np.float64)
    for j in firing:
        np.add.at(want, idx[off[j]:off[j + 1]], 1.0)
    got = ours.numpy()
    assert np.array_equal(got, want.astype(np.float32))
    mismatches = []
    for _ in range(3):
        copies.zero()
        spikes.zero()
        ctx.synchronize()
        rk.signal_spikes_chunked(nf, conn_tab.value, off_tab.value, d_fire.value, copies.value, spikes.value,
                                 d_out.value)
        mismatches.append(int((spikes.numpy()[:n] != got).sum()))
    print(f"reference chunked kernel vs library: mismatching targets per run {mismatches}")
    assert min(mismatches) == 0, mismatches
    coup.close()
