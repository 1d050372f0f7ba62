"""Device sub-sampling of on-disk connectivity and positions against the
oracle's restatement of FileNetwork / FileMorphology: bit-exact."""
import numpy as np
import pytest

import neuronephys_clean_gb300 as nn
from oracle import probes as P

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,N", [(3000, 3000), (3000, 1000), (10007, 997)])
def test_file_network_subsample(ctx, tmp_path, n, N):
    rng = np.random.default_rng(n + N)
    deg = rng.integers(0, 80, n)
    rp = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
    col = rng.integers(0, n, rp[-1]).astype(np.int32)
    f = tmp_path / "net.nncsr"
    nn.write_network_file(f, rp, col)
    net = nn.FileNetwork(f)
    assert net.generate(ctx, N)
    off, idx = P.file_network_subsample(rp, col, N)
    assert np.array_equal(net.row_ptr, off)
    assert np.array_equal(net.col, idx)
    assert not nn.FileNetwork(f).generate(ctx, n + 1)
    assert not nn.FileNetwork(tmp_path / "missing.nncsr").generate(ctx, N)


def test_file_morphology(ctx, tmp_path):
    rng = np.random.default_rng(3)
    n, N = 50001, 777
    x, y, z = (rng.uniform(-5, 11, n).astype(np.float32) for _ in range(3))
    f = tmp_path / "pos.nnpos"
    nn.write_positions_file(f, x, y, z)
    m = nn.FileMorphology(f)
    assert m.generate(ctx, N)
    assert np.array_equal(m.positions, P.file_morphology_positions(x, y, z, N))
