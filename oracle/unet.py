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
