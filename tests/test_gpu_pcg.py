"""7-point Jacobi-PCG on the GPU against the FP64 oracle.

Tolerances: the solver's own FP64-reduced relative residual <= rtol = 1e-6;
the solution within 1e-5 (relative 2-norm) of an FP64 CG solution solved to
1e-12; the true residual of the FP32-stored solution, evaluated in FP64,
<= 1e-5 (FP32 storage floor)."""
import numpy as np
import pytest

import neuronephys_clean_gb300 as nn

pytestmark = pytest.mark.gpu


def lognormal_field(shape, rng, sigma=1.0):
    from scipy.ndimage import gaussian_filter
    g = gaussian_filter(rng.standard_normal(shape), 8.0 / np.sqrt(2), mode="wrap")
    g /= g.std()
    return np.exp(sigma * g).astype(np.float32)


@pytest.mark.parametrize("hetero", [False, True])
def test_apply_matches_oracle(ctx, orc, hetero):
    shape = (20, 24, 32)
    rng = np.random.default_rng(0)
    D = lognormal_field(shape, rng) if hetero else None
    x = rng.standard_normal(np.prod(shape)).astype(np.float32)
    pc = nn.PCG(ctx, shape[2], shape[1], shape[0], 2.5, 0.1, ctx.to_device(D.ravel()) if hetero else None)
    dx, dy = ctx.to_device(x), ctx.empty((x.size,), np.float32)
    pc.apply(dx, dy)
    ref = orc.apply7(x, shape, 2.5, 0.1, D)
    np.testing.assert_allclose(dy.numpy(), ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())


@pytest.mark.parametrize("hetero,shape,alpha", [(False, (32, 32, 32), 16.0), (True, (24, 28, 32), 8.0)])
def test_solve_matches_oracle(ctx, orc, hetero, shape, alpha):
    rng = np.random.default_rng(1)
    D = lognormal_field(shape, rng) if hetero else None
    G = int(np.prod(shape))
    b = np.zeros(G, np.float32)
    b[rng.integers(0, G, 300)] += 1.0      # spike-like point sources
    b += 0.01 * rng.random(G).astype(np.float32)
    pc = nn.PCG(ctx, shape[2], shape[1], shape[0], alpha, 0.1, ctx.to_device(D.ravel()) if hetero else None)
    db, dx = ctx.to_device(b), ctx.to_device(np.zeros(G, np.float32))
    it, rel = pc.solve(db, dx, rtol=1e-6, max_iter=5000)
    assert rel <= 1e-6 and it > 0
    x = dx.numpy().astype(np.float64)
    ref, rit, _ = orc.pcg7(b, np.zeros(G), shape, alpha, 0.1, D, rtol=1e-12)
    assert np.linalg.norm(x - ref) <= 1e-5 * np.linalg.norm(ref)
    true_res = np.linalg.norm(b - orc.apply7(x, shape, alpha, 0.1, D)) / np.linalg.norm(b)
    assert true_res <= 1e-5
    _, it64, _ = orc.pcg7(b, np.zeros(G), shape, alpha, 0.1, D, rtol=1e-6)
    assert abs(it - it64) <= max(3, 0.05 * it64)


def test_not_converged_status(ctx):
    pc = nn.PCG(ctx, 32, 32, 32, 50.0, 0.0)
    b = ctx.to_device(np.random.default_rng(2).random(32 ** 3).astype(np.float32))
    x = ctx.to_device(np.zeros(32 ** 3, np.float32))
    with pytest.raises(nn.NNError) as e:
        pc.solve(b, x, rtol=1e-6, max_iter=3)
    assert e.value.status == 4


@pytest.mark.parametrize("hetero", [False, True])
@pytest.mark.parametrize("shape", [(18, 20, 36), (33, 40, 64), (26, 28, 30)])
def test_single_kernel_and_two_kernel_paths_agree(ctx, orc, shape, hetero, monkeypatch):
    """The TMA single-kernel iteration (nx % 4 == 0; partial tiles and
    z-chunks here; constant and lognormal D) and the two-kernel path solve to
    the same answer."""
    nz, ny, nx = shape
    G = nx * ny * nz
    rng = np.random.default_rng(4)
    D = lognormal_field(shape, rng) if hetero else None
    dD = ctx.to_device(D.ravel()) if hetero else None
    b = rng.random(G).astype(np.float32)
    b[rng.integers(0, G, 40)] += 3.0
    alpha, beta = 5.0, 0.05
    fast = nn.PCG(ctx, nx, ny, nz, alpha, beta, dD)
    monkeypatch.setenv("NN_PCG_TWO_KERNEL", "1")
    two = nn.PCG(ctx, nx, ny, nz, alpha, beta, dD)
    ref, _, _ = orc.pcg7(b, np.zeros(G), shape, alpha, beta, D, rtol=1e-12)
    its = []
    for pc in (fast, two):
        db, dx = ctx.to_device(b), ctx.to_device(np.zeros(G, np.float32))
        it, rel = pc.solve(db, dx, rtol=1e-6, max_iter=2000)
        assert rel <= 1e-6
        x = dx.numpy().astype(np.float64)
        assert np.linalg.norm(x - ref) <= 1e-5 * np.linalg.norm(ref)
        its.append(it)
    assert abs(its[0] - its[1]) <= 2

