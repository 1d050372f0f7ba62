"""The learned preconditioner's U-Net on the GPU against the FP64 numpy
oracle (oracle/unet.py), and what training buys inside flexible CG.

Gradient check: same parameters and inputs on both sides; the oracle rounds
weights and stored activations/gradients to BF16 exactly where the GPU
stores BF16, so the remaining differences come from FP32 accumulation order
flipping individual BF16 roundings.  Bounds: loss within 1e-3 relative,
network output within 1e-2 of its scale, every layer's weight gradient within
6e-2 relative (L2) and the whole gradient at cosine >= 0.999."""
import numpy as np
import pytest

import neuronephys_clean_gb300 as nn
from oracle import unet as U

pytestmark = pytest.mark.gpu


def he_params(rng):
    return np.concatenate([np.concatenate([
        rng.standard_normal(27 * ci * co) * np.sqrt(2 / (27 * ci)) * (0.1 if name == "out" else 1.0),
        rng.standard_normal(co) * 0.05]) for name, ci, co in U.LAYERS]).astype(np.float32)


def test_gradients_match_oracle(ctx):
    n = 32                      # fine grid; the network runs on 16^3, 8^3, 4^3
    pc = nn.PCG(ctx, n, n, n, 5.0, 0.01)
    lp = nn.LearnedPreconditioner(pc, seed=1)
    rng = np.random.default_rng(0)
    p = he_params(rng)
    lp.set_params(p)
    assert np.array_equal(lp.get_params(), p)
    m = n // 2
    rc = rng.standard_normal((m, m, m)).astype(np.float32)
    t = rng.standard_normal((m, m, m)).astype(np.float32)
    loss, g, y = lp.net_gradient(ctx.to_device(rc.ravel()), ctx.to_device(t.ravel()))
    rloss, rg, ry = U.unet_loss_and_grad(p.astype(np.float64), rc, t, None, rounding=True)
    assert abs(loss - rloss) <= 1e-3 * abs(rloss)
    assert np.abs(y.reshape(m, m, m) - ry).max() <= 1e-2 * np.abs(ry).max()
    offs = np.cumsum([0] + [27 * ci * co + co for _, ci, co in U.LAYERS])
    for l, (name, _, _) in enumerate(U.LAYERS):
        a, b = g[offs[l]:offs[l + 1]], rg[offs[l]:offs[l + 1]]
        assert np.linalg.norm(a - b) <= 6e-2 * np.linalg.norm(b), name
    assert np.dot(g, rg) / (np.linalg.norm(g) * np.linalg.norm(rg)) >= 0.999
    lp.close()
    pc.close()


def test_training_reduces_flexible_cg_iterations(ctx, orc):
    """Pairs from the solver's own iterates train the network; flexible CG
    with the trained coarse correction needs fewer iterations than the same
    preconditioner without the network and than plain Jacobi-PCG, and reaches
    the same 1e-6 relative residual with a solution as close to the FP64
    oracle's as the plain solver's (within 2x its error, or 1e-5)."""
    from neuronephys_clean_gb300 import fields
    n = 32
    shape = (n, n, n)
    G = n ** 3
    D = fields.lognormal_diffusivity(shape, 1.0, 4.0, seed=3)
    alpha, beta = 65.536, 1e-4
    dD = ctx.to_device(D.ravel())
    pc = nn.PCG(ctx, n, n, n, alpha, beta, dD)
    lp = nn.LearnedPreconditioner(pc, seed=2)
    tmp = ctx.empty((G,), np.float32)
    for j in range(8):
        b = fields.spike_sources(shape, neurons=200, rate=2.0, seed=100 + j)
        db = ctx.to_device(b)
        xs = ctx.to_device(np.zeros(G, np.float32))
        pc.solve(db, xs, 1e-7, 20000)
        xstar = xs.numpy()
        for k in [0, 1, 2, 4, 8, 16, 32, 64]:
            xk = ctx.to_device(np.zeros(G, np.float32))
            if k:
                with pytest.raises(nn.NNError):
                    pc.solve(db, xk, 1e-30, k)
            pc.apply(xk, tmp)
            lp.add_pair(ctx.to_device(b - tmp.numpy()), ctx.to_device(xstar - xk.numpy()))
    bt = fields.spike_sources(shape, neurons=200, rate=2.0, seed=999)
    dbt = ctx.to_device(bt)

    def fcg(net):
        lp.use_network(net)
        x = ctx.to_device(np.zeros(G, np.float32))
        it, rel = lp.solve(dbt, x, 1e-6, 2000)
        assert rel <= 1e-6
        return it, x.numpy()

    x0 = ctx.to_device(np.zeros(G, np.float32))
    it_plain, _ = pc.solve(dbt, x0, 1e-6, 20000)
    x_plain = x0.numpy()
    it_smooth, _ = fcg(False)
    lp.train(600, 1e-3)
    it_learned, x = fcg(True)
    ref, _, _ = orc.pcg7(bt, np.zeros(G), shape, alpha, beta, D, rtol=1e-12)
    err_plain = np.linalg.norm(x_plain - ref) / np.linalg.norm(ref)
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) <= max(1e-5, 2 * err_plain)
    assert it_learned <= 0.9 * it_smooth, (it_learned, it_smooth, it_plain)
    assert it_learned < it_plain, (it_learned, it_smooth, it_plain)
    lp.close()
    pc.close()
