"""The C-ABI library: loads, exports every declared entry point, struct
layouts agree with the ctypes mirror, and the host-only entry points work
without a GPU (CPU tests)."""
import ctypes as C
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

HEADER = ROOT / "include" / "neuronephys.h"


def declared() -> list[str]:
    txt = HEADER.read_text()
    return sorted(set(re.findall(r"NN_API[^;(]*?\b(nn_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(built_lib)], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    names = declared()
    assert len(names) > 40
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    from neuronephys_clean_gb300 import _lib
    assert sorted(_lib.declared_symbols()) == names
    lib = _lib.load()
    for n in names:
        assert getattr(lib, n) is not None


def test_struct_layouts_match(tmp_path, built_lib):
    from neuronephys_clean_gb300 import _lib
    structs = {"nn_leapfrog_params": _lib.LeapfrogParams, "nn_paracrine_ref_params": _lib.ParacrineRefParams,
               "nn_hh_params": _lib.HHParams, "nn_sim_config": _lib.SimConfig, "nn_net_spec": _lib.NetSpec,
               "nn_solve_stats": _lib.SolveStats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "neuronephys.h"', "int main(void) {"]
    for s, cls in structs.items():
        lines.append(f'printf("{s} %zu\\n", sizeof({s}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{s}.{f} %zu\\n", offsetof({s}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    for s, cls in structs.items():
        assert int(got[s]) == C.sizeof(cls), s
        for f, _ in cls._fields_:
            assert int(got[f"{s}.{f}"]) == getattr(cls, f).offset, f"{s}.{f}"


def test_host_uniform_random_network_matches_reference(built_lib):
    """nn_net_uniform_random is host code: bit-identical to the reference's
    generator (golden vectors from the reference itself)."""
    from neuronephys_clean_gb300 import _lib
    lib = _lib.load()
    g = np.load(GOLDEN / "ref_netgen_A.npz")
    eng = C.c_uint32(1)
    for k, key in [(8, "e"), (2, "i")]:
        ind = np.zeros(1000 * k, np.int32)
        off = np.zeros(1001, np.int32)
        assert lib.nn_net_uniform_random(1000, k, C.byref(eng), ind.ctypes.data, off.ctypes.data) == 0
        assert np.array_equal(ind, g[f"{key}_indices"]) and np.array_equal(off, g[f"{key}_offsets"])
    # ncouple > n would never terminate in the reference; it is rejected here
    assert lib.nn_net_uniform_random(3, 4, C.byref(eng), ind.ctypes.data, off.ctypes.data) == 1


def test_status_strings_and_defaults(built_lib):
    import neuronephys_clean_gb300 as nn
    lib = nn.lib()
    assert lib.nn_status_string(0) == b"ok"
    assert lib.nn_status_string(4) == b"solver did not converge"
    assert lib.nn_version() >= 100
    c = nn.default_config(1000)
    assert c.n == 1000 and c.max_delay == 1 and abs(c.hp.gNa - 120) < 1e-6 and abs(c.hp.EL + 54.4) < 1e-5
    assert abs(c.hp.dt - 0.01) < 1e-9 and c.par_rtol == pytest.approx(1e-6)
    p = nn.LeapfrogParams()
    lib.nn_leapfrog_params_reference(C.byref(p), 0)
    assert (p.gna, p.ena, p.ek, p.el, p.noise_mean, p.noise_intensity) == (120, 55, -72, -50, 3.0, 1.5)


def test_context_without_device_fails_cleanly(built_lib):
    import neuronephys_clean_gb300 as nn
    lib = nn.lib()
    h = C.c_void_p()
    st = lib.nn_ctx_create(0, C.byref(h))
    if st == 0:  # a GPU is present
        lib.nn_ctx_destroy(h)
    else:
        assert st == 8  # NN_ERR_NO_DEVICE, not a crash
    assert lib.nn_ctx_create(-1, C.byref(h)) in (1, 8)
