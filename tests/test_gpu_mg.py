"""Geometric multigrid V-cycle and multigrid-preconditioned flexible CG on the
GPU against the FP64 numpy oracle (oracle/multigrid.py).  Shapes cover the
four-cells-per-thread fine-level kernels (x side a multiple of 4, with one or
two coarse cells per restriction thread) and the one-cell form (x = 30).

Tolerances: one V-cycle (FP32 arithmetic through up to five levels) within
1e-4 of the oracle's, relative to its largest magnitude; solves reach the
FP64-reduced relative residual 1e-6 and lie within 1e-5 (relative 2-norm) of
an FP64 CG solution solved to 1e-12; iteration counts within one of the
oracle's flexible CG."""
import numpy as np
import pytest

import neuronephys_clean_gb300 as nn
from oracle import multigrid as mgo

pytestmark = pytest.mark.gpu


def lognormal_field(shape, rng, sigma=1.0):
    from scipy.ndimage import gaussian_filter
    g = gaussian_filter(rng.standard_normal(shape), 8.0 / np.sqrt(2), mode="wrap")
    g /= g.std()
    return np.exp(sigma * g).astype(np.float32)


def sources(shape, rng, k=300):
    G = int(np.prod(shape))
    b = np.zeros(G, np.float32)
    b[rng.integers(0, G, k)] += 1.0
    b += 0.01 * rng.random(G).astype(np.float32)
    return b


@pytest.mark.parametrize("hetero,shape,levels", [(False, (16, 24, 32), 0), (True, (16, 24, 32), 0),
                                                 (True, (24, 28, 32), 3), (True, (32, 32, 32), 2),
                                                 (True, (16, 20, 30), 0), (False, (12, 16, 36), 3)])
def test_vcycle_matches_oracle(ctx, hetero, shape, levels):
    rng = np.random.default_rng(0)
    D = lognormal_field(shape, rng) if hetero else None
    alpha, beta = 65.5, 1e-4
    pc = nn.PCG(ctx, shape[2], shape[1], shape[0], alpha, beta, ctx.to_device(D.ravel()) if hetero else None)
    mg = nn.MultigridPCG(pc, levels)
    lv = mgo.hierarchy(shape, alpha, beta, D, levels=levels)
    assert mg.levels == len(lv)
    r = rng.standard_normal(int(np.prod(shape))).astype(np.float32)
    dz = ctx.empty((r.size,), np.float32)
    mg.apply(ctx.to_device(r), dz)
    ref = mgo.vcycle(lv, r.reshape(shape).astype(np.float64)).ravel()
    np.testing.assert_allclose(dz.numpy(), ref, rtol=0, atol=1e-4 * np.abs(ref).max())


@pytest.mark.parametrize("hetero,shape,alpha", [(False, (32, 32, 32), 16.0), (True, (24, 28, 32), 8.0),
                                                (True, (64, 64, 64), 65.5), (True, (16, 20, 30), 20.0)])
def test_solve_matches_oracle(ctx, orc, hetero, shape, alpha):
    rng = np.random.default_rng(1)
    D = lognormal_field(shape, rng) if hetero else None
    beta = 0.1 if alpha < 60 else 1e-4
    b = sources(shape, rng)
    G = b.size
    pc = nn.PCG(ctx, shape[2], shape[1], shape[0], alpha, beta, ctx.to_device(D.ravel()) if hetero else None)
    mg = nn.MultigridPCG(pc)
    db, dx = ctx.to_device(b), ctx.to_device(np.zeros(G, np.float32))
    it, rel = mg.solve(db, dx, rtol=1e-6)
    assert rel <= 1e-6 and it > 0
    x = dx.numpy().astype(np.float64)
    ref, _, _ = orc.pcg7(b, np.zeros(G), shape, alpha, beta, D, rtol=1e-12)
    assert np.linalg.norm(x - ref) <= 1e-5 * np.linalg.norm(ref)
    true_res = np.linalg.norm(b - orc.apply7(x, shape, alpha, beta, D)) / np.linalg.norm(b)
    assert true_res <= 1e-5
    _, it_o, _ = mgo.fcg(mgo.hierarchy(shape, alpha, beta, D), b.reshape(shape), rtol=1e-6)
    assert abs(it - it_o) <= 1
    # far fewer iterations than Jacobi-PCG on the same system
    it_j, _ = pc.solve(db, ctx.to_device(np.zeros(G, np.float32)), rtol=1e-6, max_iter=20000)
    assert it * 3 < it_j


def test_solve_is_deterministic_and_reuses_nothing_stale(ctx):
    """Two solves into different solution arrays (the iteration graph is
    recaptured) and one more into the first array give bit-identical answers;
    a nonzero initial guess is honoured."""
    shape = (32, 32, 64)
    rng = np.random.default_rng(3)
    D = lognormal_field(shape, rng)
    b = sources(shape, rng)
    pc = nn.PCG(ctx, shape[2], shape[1], shape[0], 20.0, 0.01, ctx.to_device(D.ravel()))
    mg = nn.MultigridPCG(pc)
    db = ctx.to_device(b)
    outs = []
    x1, x2 = ctx.empty((b.size,), np.float32), ctx.empty((b.size,), np.float32)
    for x in (x1, x2, x1):
        x.zero()
        it, rel = mg.solve(db, x, rtol=1e-6)
        outs.append((x.numpy(), it))
    assert outs[0][1] == outs[1][1] == outs[2][1]
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][0], outs[2][0])
    # restart from the converged answer: zero or one iteration
    it, rel = mg.solve(db, x1, rtol=1e-6)
    assert it <= 1 and rel <= 1e-6


def test_not_converged_and_bad_depth(ctx):
    pc = nn.PCG(ctx, 32, 32, 32, 50.0, 0.0)
    with pytest.raises(nn.NNError):
        nn.MultigridPCG(pc, 7)       # 32 -> 16 -> 8 -> 4 -> 2: at most 5 levels
    mg = nn.MultigridPCG(pc)
    b = ctx.to_device(np.random.default_rng(2).random(32 ** 3).astype(np.float32))
    x = ctx.to_device(np.zeros(32 ** 3, np.float32))
    with pytest.raises(nn.NNError) as e:
        mg.solve(b, x, rtol=1e-12, max_iter=2)
    assert e.value.status == nn.NN_ERR_NOT_CONVERGED
    # zero right-hand side: converged at once
    z = ctx.to_device(np.zeros(32 ** 3, np.float32))
    x.zero()
    it, rel = mg.solve(z, x, rtol=1e-6)
    assert it == 0
