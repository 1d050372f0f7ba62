"""The C++ adaptor header (include/neuronephys.hpp) compiles against the
library and runs the reference's hh_benchmark loop; on the GPU its result is
identical to the same loop driven through the Python mirror."""
import subprocess

import numpy as np
import pytest

import neuronephys_clean_gb300 as nn
from conftest import ROOT


def build_loop(tmp_path, lib):
    exe = tmp_path / "hh_loop"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "hh_loop.cpp"),
                    "-L", str(lib.parent), "-lneuronephys", f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    return exe


def test_adaptors_compile_and_link(tmp_path, built_lib):
    assert build_loop(tmp_path, built_lib).exists()


@pytest.mark.gpu
def test_adaptor_loop_matches_python_mirror(tmp_path, built_lib, ctx):
    N, steps = 2000, 50
    out = subprocess.run([str(build_loop(tmp_path, built_lib)), str(N), str(steps)], check=True, capture_output=True,
                         text=True).stdout.split()
    # the same loop through the Python classes
    eph = nn.HHEphys(ctx, N)
    k = ((np.arange(N) * 7919) % N).astype(np.float32)
    eph.set("V", np.float32(-80.0) + (np.float32(50.0) * k) / np.float32(N))  # the C++ float expression
    nn.UniformRandomNetwork.reset_engine()
    e_net, i_net = nn.UniformRandomNetwork(8), nn.UniformRandomNetwork(2)
    e_net.generate(N)
    i_net.generate(N)
    ecnt, icnt = eph.vars[nn.SIM_PARAMS.index("ECOUNT")], eph.vars[nn.SIM_PARAMS.index("ICOUNT")]
    e_list = e_net.to_chunked_adjacency_list(ctx, ecnt)
    i_list = i_net.to_chunked_adjacency_list(ctx, icnt)
    ec, ic = nn.AtomicCoupling(ctx, N), nn.AtomicCoupling(ctx, N)
    v = {k: eph.vars[nn.SIM_PARAMS.index(k)] for k in ("EIN", "EOUTPUT", "IIN", "IOUTPUT")}
    total = 0
    for _ in range(steps):
        total += ec(e_list, v["EIN"], v["EOUTPUT"])
        total += ic(i_list, v["IIN"], v["IOUTPUT"])
        eph.simulate_ephys()
    V = eph.get("V")
    assert int(out[2]) == total
    assert abs(float(out[3]) - float(V.astype(np.float64).mean())) < 1e-4
