"""The multigrid oracle (oracle/multigrid.py) on the CPU: its fine operator is
the PCG oracle's 7-point operator, its coarse operators reduce to the operator
discretised on the coarse grid for a constant field, the transfers do what
they state, and multigrid-preconditioned flexible CG solves to the FP64 CG
solution in a handful of iterations."""
import numpy as np
import pytest

from oracle import multigrid as mgo


def lognormal_field(shape, rng, sigma=1.0):
    from scipy.ndimage import gaussian_filter
    g = gaussian_filter(rng.standard_normal(shape), 8.0 / np.sqrt(2), mode="wrap")
    g /= g.std()
    return np.exp(sigma * g).astype(np.float32)


@pytest.mark.parametrize("hetero", [False, True])
def test_fine_operator_is_the_pcg_operator(orc, hetero):
    shape = (6, 10, 12)
    rng = np.random.default_rng(0)
    D = lognormal_field(shape, rng) if hetero else None
    x = rng.standard_normal(shape)
    L = mgo.fine_level(shape, 3.0, 0.2, D)
    np.testing.assert_allclose(L.A(x).ravel(), orc.apply7(x.ravel(), shape, 3.0, 0.2, D), rtol=1e-12, atol=1e-12)


def test_constant_field_coarse_operator_is_the_coarse_discretisation():
    shape, alpha, beta = (8, 8, 16), 4.0, 0.1
    c = mgo.fine_level(shape, alpha, beta).coarsen()
    assert c.mass == pytest.approx(8 * (1 + beta))
    assert np.allclose(c.wx[:, :, :-1], 2 * alpha) and np.all(c.wx[:, :, -1] == 0)
    assert np.allclose(c.wy[:, :-1, :], 2 * alpha) and np.all(c.wy[:, -1, :] == 0)
    assert np.allclose(c.wz[:-1], 2 * alpha) and np.all(c.wz[-1] == 0)
    # a corner cell has three boundary faces of conductance 2 alpha each
    assert c.wb[0, 0, 0] == pytest.approx(6 * alpha)
    assert c.wb[1, 1, 1] == 0.0


def test_transfers():
    rng = np.random.default_rng(1)
    e = rng.standard_normal((4, 6, 8))
    assert mgo.restrict(np.ones((8, 12, 16))).sum() == 8 * 12 * 16
    np.testing.assert_allclose(mgo.restrict(mgo.prolong(np.ones((4, 6, 8))))[1:-1, 1:-1, 1:-1], 8.0)
    # trilinear interpolation is exact for linear functions away from the boundary
    zc, yc, xc = np.meshgrid(*(np.arange(n) * 2 + 0.5 for n in (4, 6, 8)), indexing="ij")
    lin = 0.3 * xc - 0.7 * yc + 1.1 * zc + 2.0
    zf, yf, xf = np.meshgrid(*(np.arange(n) for n in (8, 12, 16)), indexing="ij")
    np.testing.assert_allclose(mgo.prolong(lin)[2:-2, 2:-2, 2:-2],
                               (0.3 * xf - 0.7 * yf + 1.1 * zf + 2.0)[2:-2, 2:-2, 2:-2], atol=1e-12)
    assert e.shape == (4, 6, 8)


@pytest.mark.parametrize("hetero", [False, True])
def test_fcg_converges_to_the_cg_solution(orc, hetero):
    shape, alpha, beta = (32, 32, 32), 65.5, 1e-4
    rng = np.random.default_rng(2)
    D = lognormal_field(shape, rng) if hetero else None
    b = np.zeros(shape)
    b.ravel()[rng.integers(0, b.size, 200)] += 1.0
    lv = mgo.hierarchy(shape, alpha, beta, D)
    assert [L.diag.shape for L in lv] == [(32, 32, 32), (16, 16, 16)]
    x, it, rel = mgo.fcg(lv, b, rtol=1e-6)
    assert rel <= 1e-6
    _, it_cg, _ = orc.pcg7(b.ravel(), np.zeros(b.size), shape, alpha, beta, D, rtol=1e-6)
    ref, _, _ = orc.pcg7(b.ravel(), np.zeros(b.size), shape, alpha, beta, D, rtol=1e-12)
    assert np.linalg.norm(x.ravel() - ref) <= 1e-5 * np.linalg.norm(ref)
    assert it <= 20 and it * 3 < it_cg


def test_hierarchy_depth_rules():
    assert len(mgo.hierarchy((256, 256, 256), 1.0, 0.0)) == 5         # down to 16^3
    assert len(mgo.hierarchy((24, 28, 32), 1.0, 0.0, levels=3)) == 3   # 12x14x16, 6x7x8
    assert len(mgo.hierarchy((24, 28, 32), 1.0, 0.0, levels=5)) == 3   # 7 is odd: stops
