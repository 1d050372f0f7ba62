"""On-disk connectivity / positions container: host-side round trip (CPU)
and the reference's sub-sampling restated in the oracle."""
import numpy as np

import neuronephys_clean_gb300 as nn
from oracle import probes as P


def _random_csr(rng, n, k):
    deg = rng.integers(0, 2 * k, n)
    rp = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
    return rp, rng.integers(0, n, rp[-1]).astype(np.int32)


def test_network_file_round_trip(built_lib, tmp_path):
    rng = np.random.default_rng(0)
    rp, col = _random_csr(rng, 500, 20)
    f = tmp_path / "net.nncsr"
    nn.write_network_file(f, rp, col)
    rp2, col2 = nn.read_network_file(f)
    assert np.array_equal(rp, rp2) and np.array_equal(col, col2)


def test_oracle_subsample_semantics():
    # 12 rows, N = 4 -> sparsity 3: rows 0, 3, 6, 9; targets divisible by 3, divided by 3
    rp = np.array([0, 3, 3, 3, 6, 6, 6, 8, 8, 8, 10, 10, 10, 10], np.int32)
    col = np.array([0, 1, 3, 6, 7, 9, 2, 3, 11, 0], np.int32)
    off, idx = P.file_network_subsample(rp[:13], col, 4)
    assert off.tolist() == [0, 2, 4, 5, 6]
    assert idx.tolist() == [0, 1, 2, 3, 1, 0]


def test_oracle_positions_span_unit_box():
    rng = np.random.default_rng(1)
    x, y, z = (rng.uniform(-3, 7, 1000).astype(np.float32) for _ in range(3))
    p = P.file_morphology_positions(x, y, z, 100)
    assert p.shape == (100, 3) and p.min() >= -1.0 and p.max() <= 1.0
