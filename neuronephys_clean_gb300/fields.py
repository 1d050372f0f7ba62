"""Seeded synthetic inputs for the paracrine solver.

* ``lognormal_diffusivity``: D = exp(sigma * g) on an (nz, ny, nx) cell grid,
  g a unit-variance Gaussian random field with Gaussian correlation
  exp(-r^2 / (2 l^2)) (l in cells), made by filtering white noise in Fourier
  space (periodic) with the Gaussian of standard deviation l / sqrt(2).
* ``spike_sources``: a right-hand side of the kind the paracrine step builds,
  unit deposits at the voxels of spiking neurons (Poisson counts at uniformly
  placed neurons) on top of a smooth previous field.
* ``be_coefficients``: alpha and beta of the backward-Euler operator
  A = (1 + dt k) I + (dt D0 / h^2) L_D on the unit cube with n cells a side.
"""
from __future__ import annotations

import numpy as np


def lognormal_diffusivity(shape, sigma: float = 1.0, corr_cells: float = 8.0, seed: int = 0) -> np.ndarray:
    nz, ny, nx = shape
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(shape)
    s = corr_cells / np.sqrt(2.0)
    fz = np.fft.fftfreq(nz)[:, None, None]
    fy = np.fft.fftfreq(ny)[None, :, None]
    fx = np.fft.rfftfreq(nx)[None, None, :]
    filt = np.exp(-2.0 * (np.pi * s) ** 2 * (fz ** 2 + fy ** 2 + fx ** 2))
    g = np.fft.irfftn(np.fft.rfftn(w) * filt, s=shape, axes=(0, 1, 2))
    g -= g.mean()
    g /= g.std()
    return np.exp(sigma * g).astype(np.float32)


def spike_sources(shape, neurons: int = 1000, rate: float = 2.0, seed: int = 0,
                  background: float = 1e-3) -> np.ndarray:
    nz, ny, nx = shape
    rng = np.random.default_rng(seed)
    b = np.full(nz * ny * nx, background, np.float32)
    vox = rng.integers(0, nz * ny * nx, neurons)
    np.add.at(b, vox, rng.poisson(rate, neurons).astype(np.float32))
    return b


def be_coefficients(n: int, dt_s: float, D0: float = 1.0, uptake: float = 0.0) -> tuple[float, float]:
    return dt_s * D0 * n * n, dt_s * uptake
