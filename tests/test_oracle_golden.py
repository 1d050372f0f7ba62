"""The oracle's restatement of the reference network factory against golden
vectors produced by the reference's own host code (tests/golden/make_golden.py)."""
import ctypes as C
import hashlib
import json

import numpy as np

from conftest import GOLDEN


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_uniform_random_network_and_tcount_bit_exact(orc):
    g = np.load(GOLDEN / "ref_netgen_A.npz")
    eng = C.c_uint32(1)  # the reference's default-constructed UnseededRandomEngine
    e_ind, e_off = orc.uniform_random_network(1000, 8, eng)
    i_ind, i_off = orc.uniform_random_network(1000, 2, eng)
    assert np.array_equal(e_ind, g["e_indices"]) and np.array_equal(e_off, g["e_offsets"])
    assert np.array_equal(i_ind, g["i_indices"]) and np.array_equal(i_off, g["i_offsets"])
    assert np.array_equal(orc.tcount(e_ind, 1000), g["e_tcount"])
    assert np.array_equal(orc.tcount(i_ind, 1000), g["i_tcount"])


def test_chunked_adjacency_list_bit_exact(orc):
    b = json.loads((GOLDEN / "ref_netgen_B.json").read_text())
    eng = C.c_uint32(1)
    orc.uniform_random_network(1000, 8, eng)
    orc.uniform_random_network(1000, 2, eng)
    n = 2 * 7319
    ind, off = orc.uniform_random_network(n, 3, eng)
    assert _sha(ind) == b["B_indices.i32"]["sha256"]
    assert _sha(off) == b["B_offsets.i32"]["sha256"]
    assert _sha(orc.tcount(ind, n)) == b["B_tcount.f32"]["sha256"]
    ci, co = orc.chunked(ind, off, n, 2, 7319)
    for c in range(2):
        assert _sha(ci[c]) == b[f"B_chunk{c}_indices.i32"]["sha256"]
        assert _sha(co[c]) == b[f"B_chunk{c}_offsets.i32"]["sha256"]


def test_minstd_and_uniform_int_known_answers(orc):
    # minstd_rand0 from seed 1: 16807, 282475249, 1622650073 (C++ standard's 10000th value is 1043618065)
    s = C.c_uint32(1)
    assert [orc.lib().orc_minstd_next(C.byref(s)) for _ in range(3)] == [16807, 282475249, 1622650073]
    s = C.c_uint32(1)
    for _ in range(10000):
        orc.lib().orc_minstd_next(C.byref(s))
    assert s.value == 1043618065


def test_block_oracle_structure(orc):
    """The oracle's region-block generator: fixed out-degree, no self-loops,
    delays in range, region sizes summing to n."""
    n, k, R = 3000, 20, 25
    c = orc.gen_block(n, k, R, 1.0, 1.0, 40, -1.0, 1.0, 3)
    src = np.repeat(np.arange(n), k)
    assert np.array_equal(c.row_ptr, np.arange(n + 1) * k)
    assert c.col.min() >= 0 and c.col.max() < n and not np.any(c.col == src)
    assert c.delay.min() >= 1 and c.delay.max() <= 40
    assert np.all(c.weight > 0)
