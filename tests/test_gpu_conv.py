"""3x3x3 BF16 tensor-core convolutions against the FP64 numpy oracle.

Inputs and weights are BF16-representable, so the only differences are the
FP32 accumulation order and the final rounding of the output to BF16:
outputs within one BF16 ulp (2^-7 relative) plus 1e-6 of the output scale;
FP32 outputs (dense channel 0, weight and bias gradients) within 1e-5 of
the scale."""
import numpy as np
import pytest

import neuronephys_clean_gb300 as nn
from oracle import unet as U

pytestmark = pytest.mark.gpu

FWD = [(16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (96, 32), (48, 16)]
SHAPE = (5, 7, 12)   # tiles span several rows and planes; pads inside tiles


def rand_act(rng, c, shape):
    return U.bf16(rng.standard_normal((c,) + shape).astype(np.float32))


def rand_w(rng, cin, cout):
    return U.bf16((rng.standard_normal((27, cin, cout)) / np.sqrt(27 * cin)).astype(np.float32))


def to_act(ctx, dense):
    a = nn.Activation(ctx, dense.shape[1:], dense.shape[0])
    a.pack(ctx.to_device(np.ascontiguousarray(dense, np.float32)))
    return a


def assert_bf16_close(got, ref):
    scale = np.abs(ref).max() + 1e-30
    np.testing.assert_array_less(np.abs(got - ref), 2.0 ** -7 * np.abs(ref) + 1e-6 * scale)


@pytest.mark.parametrize("cin,cout", FWD)
def test_forward_matches_oracle(ctx, cin, cout):
    rng = np.random.default_rng(cin * 100 + cout)
    x, w = rand_act(rng, cin, SHAPE), rand_w(rng, cin, cout)
    b = rng.standard_normal(cout).astype(np.float32) * 0.1
    ax = to_act(ctx, x)
    wp = nn.conv3d_pack_weights(ctx, ctx.to_device(w), cin, cout)
    for relu in (False, True):
        ay = nn.Activation(ctx, SHAPE, cout)
        nn.conv3d_forward(ctx, ax, wp, ay, bias=ctx.to_device(b), relu=relu)
        ref = U.conv3d(x, w, b)
        if relu:
            ref = np.maximum(ref, 0.0)
        assert_bf16_close(ay.unpack(), ref)


@pytest.mark.parametrize("cin,cout", FWD)
def test_input_gradient_matches_oracle(ctx, cin, cout):
    """The adjoint-packed weights run through the same kernel give the input
    gradient (cout -> cin channels)."""
    rng = np.random.default_rng(7 + cin + cout)
    gy, w = rand_act(rng, cout, SHAPE), rand_w(rng, cin, cout)
    wp = nn.conv3d_pack_weights(ctx, ctx.to_device(w), cin, cout, adjoint=True)
    agx = nn.Activation(ctx, SHAPE, cin)
    nn.conv3d_forward(ctx, to_act(ctx, gy), wp, agx)
    assert_bf16_close(agx.unpack(), U.conv3d_input_grad(gy, w))


def test_mask_and_dense_output(ctx):
    rng = np.random.default_rng(3)
    x, w = rand_act(rng, 16, SHAPE), rand_w(rng, 16, 16)
    m = rand_act(rng, 16, SHAPE)
    wp = nn.conv3d_pack_weights(ctx, ctx.to_device(w), 16, 16)
    ay = nn.Activation(ctx, SHAPE, 16)
    y32 = ctx.empty(SHAPE, np.float32)
    nn.conv3d_forward(ctx, to_act(ctx, x), wp, ay, mask=to_act(ctx, m), y32=y32)
    ref = U.conv3d(x, w) * (m > 0)
    assert_bf16_close(ay.unpack(), ref)
    np.testing.assert_allclose(y32.numpy(), U.bf16(ref[0]), rtol=2.0 ** -7, atol=1e-6 * np.abs(ref).max())


WGRAD = FWD + [(32, 16), (64, 32), (32, 96), (16, 48)]


@pytest.mark.parametrize("cin,cout", WGRAD)
def test_weight_gradient_matches_oracle(ctx, cin, cout):
    rng = np.random.default_rng(11 + cin * cout)
    x, gy = rand_act(rng, cin, SHAPE), rand_act(rng, cout, SHAPE)
    dw = ctx.to_device(np.zeros((27, cin, cout), np.float32))
    db = ctx.to_device(np.zeros(cout, np.float32))
    nn.conv3d_wgrad(ctx, to_act(ctx, x), to_act(ctx, gy), dw, db)
    rdw, rdb = U.conv3d_weight_grad(x, gy)
    np.testing.assert_allclose(dw.numpy(), rdw, rtol=1e-5, atol=1e-5 * np.abs(rdw).max())
    np.testing.assert_allclose(db.numpy(), rdb, rtol=1e-5, atol=1e-5 * np.abs(rdb).max())


def test_large_grid_many_tiles(ctx):
    shape = (40, 48, 64)
    rng = np.random.default_rng(5)
    x, w = rand_act(rng, 16, shape), rand_w(rng, 16, 32)
    wp = nn.conv3d_pack_weights(ctx, ctx.to_device(w), 16, 32)
    ay = nn.Activation(ctx, shape, 32)
    nn.conv3d_forward(ctx, to_act(ctx, x), wp, ay, relu=True)
    assert_bf16_close(ay.unpack(), np.maximum(U.conv3d(x, w), 0.0))


@pytest.mark.parametrize("cin,cout", [(16, 16), (32, 96), (96, 32)])
def test_weight_gradient_many_tiles(ctx, cin, cout):
    """The tensor-core weight gradient over a grid of many tiles per CTA
    (persistent CTAs accumulating in tensor memory across tiles)."""
    shape = (18, 24, 30)
    rng = np.random.default_rng(3 + cin + cout)
    x, gy = rand_act(rng, cin, shape), rand_act(rng, cout, shape)
    dw = ctx.to_device(np.zeros((27, cin, cout), np.float32))
    nn.conv3d_wgrad(ctx, to_act(ctx, x), to_act(ctx, gy), dw, None)
    rdw, _ = U.conv3d_weight_grad(x, gy)
    np.testing.assert_allclose(dw.numpy(), rdw, rtol=1e-5, atol=1e-5 * np.abs(rdw).max())
