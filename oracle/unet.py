"""FP64 numpy oracle of the learned preconditioner's layers.  TEST
INFRASTRUCTURE ONLY (imported by tests/ as the checker).

The preconditioner has no counterpart in the reference; these restate the
textbook operations the GPU kernels implement:
* conv3d: 3x3x3 cross-correlation with zero padding ("same"), weights
  w[27][cin][cout], tap = (dz+1)*9 + (dy+1)*3 + (dx+1), plus bias;
* its adjoint with respect to the input, and the weight / bias gradients;
* 2x average pooling and nearest upsampling (each other's adjoint up to 1/8);
* the 3-level U-Net forward/backward built from them.
Tensors are (C, nz, ny, nx).
"""
from __future__ import annotations

import numpy as np

TAPS = [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def _shift(x, dz, dy, dx):
    """s[..., z, y, x] = x[..., z+dz, y+dy, x+dx] with zeros outside."""
    C, nz, ny, nx = x.shape
    p = np.zeros((C, nz + 2, ny + 2, nx + 2), x.dtype)
    p[:, 1:-1, 1:-1, 1:-1] = x
    return p[:, 1 + dz:1 + dz + nz, 1 + dy:1 + dy + ny, 1 + dx:1 + dx + nx]


def conv3d(x, w, b=None):
    x = np.asarray(x, np.float64)
    w = np.asarray(w, np.float64)
    cin, cout = w.shape[1], w.shape[2]
    y = np.zeros((cout,) + x.shape[1:])
    for t, (dz, dy, dx) in enumerate(TAPS):
        s = _shift(x, dz, dy, dx).reshape(cin, -1)
        y += (w[t].T @ s).reshape(y.shape)
    if b is not None:
        y += np.asarray(b, np.float64)[:, None, None, None]
    return y


def conv3d_input_grad(gy, w):
    """Adjoint of conv3d in x: sum over taps of w[t] gy shifted by -tap."""
    gy = np.asarray(gy, np.float64)
    w = np.asarray(w, np.float64)
    cin = w.shape[1]
    gx = np.zeros((cin,) + gy.shape[1:])
    for t, (dz, dy, dx) in enumerate(TAPS):
        s = _shift(gy, -dz, -dy, -dx).reshape(gy.shape[0], -1)
        gx += (w[t] @ s).reshape(gx.shape)
    return gx


def conv3d_weight_grad(x, gy):
    x = np.asarray(x, np.float64)
    gy = np.asarray(gy, np.float64)
    cin, cout = x.shape[0], gy.shape[0]
    dw = np.zeros((27, cin, cout))
    g2 = gy.reshape(cout, -1)
    for t, (dz, dy, dx) in enumerate(TAPS):
        s = _shift(x, dz, dy, dx).reshape(cin, -1)
        dw[t] = s @ g2.T
    return dw, g2.sum(axis=1)


def avgpool2(x):
    C, nz, ny, nx = x.shape
    return x.reshape(C, nz // 2, 2, ny // 2, 2, nx // 2, 2).mean(axis=(2, 4, 6))


def upsample2(x):
    return x.repeat(2, axis=1).repeat(2, axis=2).repeat(2, axis=3)


def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


# --------------------------------------------------------------- U-Net --

LAYERS = [("e0a", 16, 16), ("e0b", 16, 16), ("e1a", 16, 32), ("e1b", 32, 32), ("b2a", 32, 64), ("b2b", 64, 64),
          ("d1a", 96, 32), ("d1b", 32, 32), ("d0a", 48, 16), ("d0b", 16, 16), ("out", 16, 16)]


def unflatten(params):
    out, off = {}, 0
    for name, ci, co in LAYERS:
        w = params[off:off + 27 * ci * co].reshape(27, ci, co)
        off += 27 * ci * co
        b = params[off:off + co]
        off += co
        out[name] = (w, b)
    assert off == params.size
    return out


def flatten(grads):
    return np.concatenate([np.concatenate([grads[n][0].ravel(), grads[n][1].ravel()]) for n, _, _ in LAYERS])


def unet_loss_and_grad(params, rc, target, logd=None, rounding=True):
    """Forward + backward of the preconditioner's U-Net in FP64, rounding
    stored tensors to BF16 where the GPU stores BF16 (rounding=True).
    rc, target, logd: (nz, ny, nx).  Returns (loss, flat gradient, y)."""
    R = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    P = unflatten(np.asarray(params, np.float64))
    W = {n: ((R(P[n][0].astype(np.float32)).astype(np.float64) if rounding else P[n][0]), P[n][1])
         for n, _, _ in LAYERS}
    rc = np.asarray(rc, np.float64)
    s = np.sqrt(np.mean(rc.astype(np.float64) ** 2))
    x0 = np.zeros((16,) + rc.shape)
    x0[0] = rc / s if s > 0 else 0.0
    if logd is not None:
        x0[1] = logd
    if rounding:
        x0 = R(x0.astype(np.float32)).astype(np.float64)

    def fwd(n, x, relu=True):
        y = conv3d(x, W[n][0], W[n][1])
        return np.maximum(y, 0.0) if relu else y

    def st(a):
        return R(a.astype(np.float32)).astype(np.float64) if rounding else a

    e0a = st(fwd("e0a", x0))
    sk0 = st(fwd("e0b", e0a))
    p1 = st(avgpool2(sk0))
    e1a = st(fwd("e1a", p1))
    sk1 = st(fwd("e1b", e1a))
    p2 = st(avgpool2(sk1))
    b2a = st(fwd("b2a", p2))
    b2b = st(fwd("b2b", b2a))
    cat1 = np.concatenate([upsample2(b2b), sk1])
    d1a = st(fwd("d1a", cat1))
    d1b = st(fwd("d1b", d1a))
    cat0 = np.concatenate([upsample2(d1b), sk0])
    d0a = st(fwd("d0a", cat0))
    d0b = st(fwd("d0b", d0a))
    yfull = fwd("out", d0b, relu=False)
    y = yfull[0].astype(np.float32).astype(np.float64) if rounding else yfull[0]
    t = np.asarray(target, np.float64) / s
    diff = y - t
    loss = 0.5 * np.sum(diff ** 2)
    g = {}
    gout = np.zeros_like(yfull)
    gout[0] = diff
    gout = st(gout)

    def back(n, x, gy, mask):
        g[n] = conv3d_weight_grad(x, gy)
        gx = conv3d_input_grad(gy, W[n][0])
        if mask is not None:
            gx = gx * (mask > 0)
        return st(gx)

    gd0b = back("out", d0b, gout, d0b)
    gd0a = back("d0b", d0a, gd0b, d0a)
    gcat0 = back("d0a", cat0, gd0a, cat0)
    c_up0 = d1b.shape[0]
    gd1b = st(gcat0[:c_up0].reshape(c_up0, d1b.shape[1], 2, d1b.shape[2], 2, d1b.shape[3], 2).sum(axis=(2, 4, 6)))
    gd1a = back("d1b", d1a, gd1b, d1a)
    gcat1 = back("d1a", cat1, gd1a, cat1)
    c_up1 = b2b.shape[0]
    gb2b = st(gcat1[:c_up1].reshape(c_up1, b2b.shape[1], 2, b2b.shape[2], 2, b2b.shape[3], 2).sum(axis=(2, 4, 6)))
    gb2a = back("b2b", b2a, gb2b, b2a)
    gp2 = back("b2a", p2, gb2a, None)
    gsk1 = st((gcat1[c_up1:] + upsample2(gp2) / 8.0) * (sk1 > 0))
    ge1a = back("e1b", e1a, gsk1, e1a)
    gp1 = back("e1a", p1, ge1a, None)
    gsk0 = st((gcat0[c_up0:] + upsample2(gp1) / 8.0) * (sk0 > 0))
    ge0a = back("e0b", e0a, gsk0, e0a)
    g["e0a"] = conv3d_weight_grad(x0, ge0a)
    return loss, flatten(g), y
