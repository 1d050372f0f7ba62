"""A plain C host (tests/cpp/sim_host.c) drives the device-resident
simulation through the C ABI alone: it compiles as strict C11 against
include/neuronephys.h and links against the library (CPU), and on the GPU its
run matches the same run made through the Python mirror."""
import subprocess

import numpy as np
import pytest

import neuronephys_clean_gb300 as nn
from conftest import ROOT

K, DMAX, REGION, EVERY, CAPACITY = 10, 20, 50, 40, 1024


def build_host(tmp_path, lib):
    exe = tmp_path / "sim_host"
    subprocess.run(["gcc", "-std=c11", "-O1", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "sim_host.c"), "-L", str(lib.parent), "-lneuronephys",
                    f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    return exe


def host_network(n: int):
    """The network sim_host.c builds: the same 64-bit LCG, top 31 bits."""
    s = 12345
    mask = (1 << 64) - 1

    def draw():
        nonlocal s
        s = (s * 6364136223846793005 + 1442695040888963407) & mask
        return s >> 33

    col = np.empty(n * K, np.int32)
    w = np.empty(n * K, np.float32)
    d = np.empty(n * K, np.uint8)
    for e in range(n * K):
        col[e] = draw() % n
        w[e] = np.float32(0.5) * np.float32(draw() % 1000 + 1) / np.float32(1000.0)
        d[e] = 1 + draw() % DMAX
    row_ptr = np.arange(n + 1, dtype=np.int64) * K
    inh = (np.arange(n) >= n - n // 5).astype(np.uint8)
    return row_ptr, col, w, d, inh


def test_sim_host_compiles_as_c11(tmp_path, built_lib):
    assert build_host(tmp_path, built_lib).exists()


@pytest.mark.gpu
def test_sim_host_matches_python_mirror(tmp_path, built_lib, ctx):
    n, steps = 2000, 1000
    out = subprocess.run([str(build_host(tmp_path, built_lib)), str(n), str(steps), str(nn.NN_DELIVERY_PULL)],
                         check=True, capture_output=True, text=True).stdout.split()
    c = nn.default_config(n)
    c.max_delay, c.grid, c.delivery = DMAX, 16, nn.NN_DELIVERY_PULL
    sim = nn.Simulation(ctx, c)
    sim.set_network(*host_network(n))
    sim.init_state(-65.0, 6.0, 12.0)
    R = n // REGION
    sim.set_electrodes(np.arange(R * REGION), np.arange(R + 1) * REGION, EVERY, CAPACITY)
    sim.step(steps)
    step, spikes = sim.counters()
    V = sim.get_field("V")
    first, avg, _ = sim.read_electrodes()
    sim.close()
    assert int(out[0]) == n and int(out[1]) == step == steps
    assert spikes > 0 and int(out[2]) == spikes
    # pull delivery sums in a fixed order, so both runs follow the same bits
    assert abs(float(out[3]) - float(V.astype(np.float64).mean())) < 1e-6
    assert int(out[4]) == len(avg) > 0 and int(out[5]) == first
    assert abs(float(out[6]) - float(avg[-1, 0])) < 1e-6
