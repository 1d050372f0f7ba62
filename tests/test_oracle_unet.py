"""The numpy oracle of the preconditioner layers is self-consistent (CPU)."""
import numpy as np

from oracle import unet as U


def test_conv_adjoint_and_gradients():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((16, 4, 5, 6))
    w = rng.standard_normal((27, 16, 32))
    gy = rng.standard_normal((32, 4, 5, 6))
    lhs = np.sum(U.conv3d(x, w) * gy)
    assert np.isclose(lhs, np.sum(x * U.conv3d_input_grad(gy, w)), rtol=1e-12)
    dw, db = U.conv3d_weight_grad(x, gy)
    eps = 1e-6
    for (t, i, j) in [(0, 0, 0), (13, 5, 7), (26, 15, 31)]:
        w2 = w.copy()
        w2[t, i, j] += eps
        fd = (np.sum(U.conv3d(x, w2) * gy) - lhs) / eps
        assert np.isclose(fd, dw[t, i, j], rtol=1e-5, atol=1e-6)
    b = rng.standard_normal(32)
    assert np.isclose(np.sum(U.conv3d(x, w, b) * gy) - lhs, np.dot(b, db), rtol=1e-12)


def test_pool_upsample_adjoint():
    rng = np.random.default_rng(1)
    x = rng.standard_normal((8, 4, 6, 8))
    y = rng.standard_normal((8, 2, 3, 4))
    assert np.isclose(np.sum(U.avgpool2(x) * y), np.sum(x * U.upsample2(y)) / 8.0)


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.0e-3], np.float32)
    r = U.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5
    assert abs(r[4] - 3.0e-3) <= 3.0e-3 * 2 ** -8


def test_unet_backprop_matches_finite_differences():
    rng = np.random.default_rng(2)
    p = np.concatenate([np.concatenate([rng.standard_normal(27 * ci * co) * np.sqrt(2 / (27 * ci)),
                                        rng.standard_normal(co) * 0.1]) for _, ci, co in U.LAYERS])
    rc, t, ld = (rng.standard_normal((8, 8, 8)) for _ in range(3))
    loss, g, _ = U.unet_loss_and_grad(p, rc, t, ld, rounding=False)
    offs = np.cumsum([0] + [27 * ci * co + co for _, ci, co in U.LAYERS])
    for l in range(len(U.LAYERS)):
        for idx in (offs[l] + 3, offs[l + 1] - 2):   # a weight and a bias of every layer
            p2 = p.copy()
            p2[idx] += 1e-6
            fd = (U.unet_loss_and_grad(p2, rc, t, ld, rounding=False)[0] - loss) / 1e-6
            assert np.isclose(fd, g[idx], rtol=1e-4, atol=1e-6 * max(1.0, abs(loss))), (l, idx, fd, g[idx])
