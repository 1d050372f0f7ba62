"""Multigrid with a learned coarse-level solver (nn_lmg_*).

Checks: solves reach the FP64-reduced relative residual 1e-6 and lie within
1e-5 (relative 2-norm) of an FP64 CG solution; with the network switched off
the object is the classical hierarchy (same iteration count as MultigridPCG);
training on pairs from the classical solver lowers the loss, and the trained
network solves in fewer iterations than an untrained one."""
import numpy as np
import pytest

import neuronephys_clean_gb300 as nn

pytestmark = pytest.mark.gpu


def lognormal_field(shape, rng, sigma=1.0):
    from scipy.ndimage import gaussian_filter
    g = gaussian_filter(rng.standard_normal(shape), 8.0 / np.sqrt(2), mode="wrap")
    g /= g.std()
    return np.exp(sigma * g).astype(np.float32)


def sources(shape, rng, k=400):
    G = int(np.prod(shape))
    b = np.zeros(G, np.float32)
    b[rng.integers(0, G, k)] += 1.0
    return b


def test_learned_coarse_solver(ctx, orc):
    shape, alpha, beta = (64, 64, 64), 65.5, 1e-4
    rng = np.random.default_rng(11)
    D = lognormal_field(shape, rng)
    G = int(np.prod(shape))
    pc = nn.PCG(ctx, shape[2], shape[1], shape[0], alpha, beta, ctx.to_device(D.ravel()))
    lm = nn.LearnedMultigrid(pc, level=2, seed=3)          # 16^3 level
    b = sources(shape, rng)
    db, dx = ctx.to_device(b), ctx.empty((G,), np.float32)
    # classical hierarchy on the same object = MultigridPCG
    lm.use_network(False)
    dx.zero()
    it_classic, rel = lm.solve(db, dx)
    mg = nn.MultigridPCG(pc)
    dx2 = ctx.to_device(np.zeros(G, np.float32))
    it_mg, _ = mg.solve(db, dx2)
    assert it_classic == it_mg and rel <= 1e-6
    # untrained network (its coarse correction is noise: the solve may not
    # converge within the limit, which counts as the limit)
    lm.use_network(True)
    dx.zero()
    try:
        it_untrained, _ = lm.solve(db, dx, max_iter=300)
    except nn.NNError as e:
        assert e.status == nn.NN_ERR_NOT_CONVERGED
        it_untrained = 300
    # training pairs from classical solves of other right-hand sides
    n = lm.add_solves([sources(shape, np.random.default_rng(100 + j)) for j in range(4)])
    assert n >= 20 and lm.pairs == n
    first = lm.train(20, 1e-3)
    last = lm.train(300, 1e-3)
    assert last < first
    dx.zero()
    it_trained, rel = lm.solve(db, dx)
    assert rel <= 1e-6
    assert it_trained < it_untrained
    x = dx.numpy().astype(np.float64)
    ref, _, _ = orc.pcg7(b, np.zeros(G), shape, alpha, beta, D, rtol=1e-12)
    assert np.linalg.norm(x - ref) <= 1e-5 * np.linalg.norm(ref)
    # Jacobi sweeps after the network's correction, chosen by time: the
    # solve keeps its tolerance and its FP64 agreement
    sw, ms = lm.autotune_post_sweeps([ctx.to_device(sources(shape, np.random.default_rng(100 + j))) for j in range(2)])
    assert sw in (2, 4, 8, 12, 16, 20, 24) and ms > 0
    dx.zero()
    it_tuned, rel = lm.solve(db, dx)
    assert rel <= 1e-6 and it_tuned <= it_trained + 1
    x = dx.numpy().astype(np.float64)
    assert np.linalg.norm(x - ref) <= 1e-5 * np.linalg.norm(ref)
