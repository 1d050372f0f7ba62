"""FP64 numpy oracle of the geometric multigrid preconditioner and its flexible
CG.  TEST INFRASTRUCTURE ONLY (imported by tests/ as the checker).

No counterpart in the reference (its paracrine solver is unpreconditioned CG,
src/paracrine.cu:63-134).  This restates, in plain numpy on (nz, ny, nx) arrays:
* the fine operator (A v)_c = (1 + beta) v_c + alpha sum_f cf (v_c - v_nb),
  cf = harmonic mean of the cell field across an interior face, the cell's
  own value on a boundary face (v = 0 outside), cf = 1 without a field
  (the same operator as oracle.pcg7);
* the coarse operators: mass = sum of the eight children; face conductance =
  half the sum of the four fine conductances across the coarse face;
  boundary conductance = half the children's boundary sum;
* restriction = sum of the eight children; prolongation = cell-centred
  trilinear interpolation (3/4, 1/4 per axis, zero outside);
* the V-cycle (damped Jacobi, omega 0.8; nu sweeps from a zero guess before
  and after the coarse correction; coarse_sweeps on the coarsest level);
* flexible CG (Notay 2000): beta_k = -(z_k, q_{k-1}) / (p_{k-1}, q_{k-1}).
"""
from __future__ import annotations

import numpy as np


class Level:
    """7-point operator: diag v_c - sum over interior faces w v_nb.  wx[z, y, x]
    couples (x, x+1) (0 in the last column); wb = boundary conductance."""

    def __init__(self, mass: float, wx, wy, wz, wb):
        self.mass, self.wx, self.wy, self.wz, self.wb = mass, wx, wy, wz, wb
        d = mass + wb + wx + wy + wz
        d[:, :, 1:] += wx[:, :, :-1]
        d[:, 1:, :] += wy[:, :-1, :]
        d[1:] += wz[:-1]
        self.diag = d

    def A(self, v):
        out = self.diag * v
        out[:, :, :-1] -= self.wx[:, :, :-1] * v[:, :, 1:]
        out[:, :, 1:] -= self.wx[:, :, :-1] * v[:, :, :-1]
        out[:, :-1, :] -= self.wy[:, :-1, :] * v[:, 1:, :]
        out[:, 1:, :] -= self.wy[:, :-1, :] * v[:, :-1, :]
        out[:-1] -= self.wz[:-1] * v[1:]
        out[1:] -= self.wz[:-1] * v[:-1]
        return out

    def coarsen(self) -> "Level":
        nz, ny, nx = self.diag.shape
        cz, cy, cx = nz // 2, ny // 2, nx // 2
        fx = self.wx[:, :, 1::2].reshape(cz, 2, cy, 2, cx).sum(axis=(1, 3))
        fy = self.wy[:, 1::2, :].reshape(cz, 2, cy, cx, 2).sum(axis=(1, 4))
        fz = self.wz[1::2].reshape(cz, cy, 2, cx, 2).sum(axis=(2, 4))
        wx, wy, wz = 0.5 * fx, 0.5 * fy, 0.5 * fz
        wx[:, :, -1] = 0.0
        wy[:, -1, :] = 0.0
        wz[-1] = 0.0
        wb = 0.5 * restrict(self.wb)
        return Level(8.0 * self.mass, wx, wy, wz, wb)


def fine_level(shape, alpha: float, beta: float, D=None) -> Level:
    nz, ny, nx = shape
    Dd = np.ones(shape) if D is None else np.asarray(D, np.float64).reshape(shape)
    hm = (lambda a, b: 2 * a * b / (a + b)) if D is not None else (lambda a, b: np.ones_like(a))
    wx = np.zeros(shape)
    wy = np.zeros(shape)
    wz = np.zeros(shape)
    wx[:, :, :-1] = alpha * hm(Dd[:, :, :-1], Dd[:, :, 1:])
    wy[:, :-1, :] = alpha * hm(Dd[:, :-1, :], Dd[:, 1:, :])
    wz[:-1] = alpha * hm(Dd[:-1], Dd[1:])
    nb = np.zeros(shape)
    nb[:, :, 0] += 1
    nb[:, :, -1] += 1
    nb[:, 0, :] += 1
    nb[:, -1, :] += 1
    nb[0] += 1
    nb[-1] += 1
    return Level(1.0 + beta, wx, wy, wz, alpha * nb * Dd)


def restrict(r):
    nz, ny, nx = r.shape
    return r.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2).sum(axis=(1, 3, 5))


def prolong(e):
    out = e
    for ax in range(3):
        n = out.shape[ax]
        pad = [(0, 0)] * 3
        pad[ax] = (1, 1)
        ep = np.pad(out, pad)

        def sl(a, b):
            return tuple(slice(a, b) if i == ax else slice(None) for i in range(3))

        c, lo, hi = ep[sl(1, n + 1)], ep[sl(0, n)], ep[sl(2, n + 2)]
        shp = list(out.shape)
        shp[ax] = 2 * n
        res = np.empty(shp)
        res[tuple(slice(0, None, 2) if i == ax else slice(None) for i in range(3))] = 0.75 * c + 0.25 * lo
        res[tuple(slice(1, None, 2) if i == ax else slice(None) for i in range(3))] = 0.75 * c + 0.25 * hi
        out = res
    return out


def hierarchy(shape, alpha, beta, D=None, levels: int = 0, coarse_cells: int = 4096):
    """Levels as nn_mg_create builds them (levels = 0: coarsen while the
    coarsest level has more than coarse_cells cells)."""
    lv = [fine_level(shape, alpha, beta, D)]
    while True:
        nz, ny, nx = lv[-1].diag.shape
        if levels:
            if len(lv) >= levels:
                break
        elif nz * ny * nx <= coarse_cells:
            break
        if nx % 2 or ny % 2 or nz % 2 or min(nx, ny, nz) < 4:
            break
        lv.append(lv[-1].coarsen())
    return lv


def vcycle(lv, b, l: int = 0, omega: float = 0.8, nu: int = 2, coarse_sweeps: int = 8):
    L = lv[l]
    inv = 1.0 / L.diag
    sweeps = coarse_sweeps if l == len(lv) - 1 else nu
    x = omega * inv * b
    for _ in range(sweeps - 1):
        x = x + omega * inv * (b - L.A(x))
    if l == len(lv) - 1:
        return x
    x = x + prolong(vcycle(lv, restrict(b - L.A(x)), l + 1, omega, nu, coarse_sweeps))
    for _ in range(nu):
        x = x + omega * inv * (b - L.A(x))
    return x


def fcg(lv, b, x0=None, rtol: float = 1e-6, max_iter: int = 500):
    """Flexible CG with one V-cycle per iteration; returns (x, iterations, relres)."""
    A = lv[0].A
    b = np.asarray(b, np.float64).reshape(lv[0].diag.shape)
    x = np.zeros_like(b) if x0 is None else np.asarray(x0, np.float64).reshape(b.shape).copy()
    r = b - A(x)
    bb = float((b * b).sum())
    rr = float((r * r).sum())
    it = 0
    if rr <= rtol * rtol * bb:
        return x, 0, np.sqrt(rr / bb) if bb > 0 else 0.0
    z = vcycle(lv, r)
    p = z.copy()
    rz = float((r * z).sum())
    while it < max_iter:
        q = A(p)
        pq = float((p * q).sum())
        a = rz / pq
        x += a * p
        r -= a * q
        it += 1
        rr = float((r * r).sum())
        if rr <= rtol * rtol * bb:
            break
        z = vcycle(lv, r)
        rz = float((r * z).sum())
        p = z - float((z * q).sum()) / pq * p
    return x, it, np.sqrt(rr / bb)
