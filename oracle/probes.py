"""Numpy restatements of the step's consumers.  TEST INFRASTRUCTURE ONLY.

* electrodes_measure: src_wholebrain/electrode_net.cu:3-31 (per region: FP32
  running sum of V over its index list / count; sum of is_firing);
* SynchronyOracle: src_wholebrain/electrode_net.cu:56-124 (running FP64
  sums of V_i^2, V_i; sub-population means; chi_sub);
* hebbian_update: src_wholebrain/hebbian.cu:3-51 (set timers of firing rows,
  then the rule over every synapse with a running timer), FP32 weights.
"""
from __future__ import annotations

import numpy as np


def electrodes_measure(idx, off, V, is_firing=None):
    R = len(off) - 1
    avg = np.zeros(R, np.float32)
    fir = np.zeros(R, np.int64)
    for r in range(R):
        s = np.float32(0.0)
        for i in idx[off[r]:off[r + 1]]:
            s = np.float32(s + np.float32(V[i]))
        avg[r] = np.float32(s / np.float32(off[r + 1] - off[r]))
        if is_firing is not None:
            fir[r] = int(np.sum(is_firing[idx[off[r]:off[r + 1]]]))
    return avg, fir


class SynchronyOracle:
    def __init__(self, region_inds, sub_counts):
        self.idx = np.asarray(region_inds)
        self.sub = list(sub_counts)
        self.vi2 = np.zeros(len(self.idx))
        self.vi = np.zeros(len(self.idx))
        self.avg = np.zeros(len(self.sub))
        self.avg2 = np.zeros(len(self.sub))
        self.T = 0

    def measure(self, V):
        v = np.asarray(V, np.float32)[self.idx]
        self.vi2 += (v * v).astype(np.float64)
        self.vi += v.astype(np.float64)
        for q, ns in enumerate(self.sub):
            a = float(np.sum(v[:ns].astype(np.float64))) / ns
            self.avg[q] += a
            self.avg2[q] += a * a
        self.T += 1

    def chi(self):
        vi2, vi = self.vi2 / self.T, self.vi / self.T
        out = []
        for q, ns in enumerate(self.sub):
            denom = np.sum(vi2[:ns] - vi[:ns] ** 2)
            var = (self.avg2[q] - self.avg[q] ** 2 / self.T) / self.T
            out.append(ns * var / denom)
        return np.array(out)


def hebbian_update(col, off, w, timers, is_firing, firing_inds, window, inc):
    """In place on w (float32) and timers (int)."""
    for pre in firing_inds:
        timers[off[pre]:off[pre + 1]] = window
    act = timers > 0
    timers[act] -= 1
    alpha = np.exp(-np.abs(w - np.float32(1.0))).astype(np.float32)
    dep = act & (timers == 0)
    pot = act & ~dep & (np.asarray(is_firing)[col] != 0)
    w[dep] = (w[dep] - np.float32(inc) * alpha[dep]).astype(np.float32)
    w[pot] = (w[pot] + np.float32(inc) * alpha[pot]).astype(np.float32)
    timers[pot] = 0


def file_network_subsample(row_ptr, col, N):
    """FileNetwork::GenerateFromHDF's loop (src/network_factory.cu:194-210)."""
    numpnts = len(row_ptr) - 1
    sparsity = numpnts // N
    indices, offsets = [], [0]
    for i in range(N):
        r = i * sparsity
        for e in range(row_ptr[r], row_ptr[r + 1]):
            if col[e] % sparsity == 0:
                indices.append(col[e] // sparsity)
        offsets.append(len(indices))
    return np.array(offsets, np.int64), np.array(indices, np.int32)


def file_morphology_positions(x, y, z, N):
    """FileMorphology::GenerateFromHDF (src/morphology.cpp:297-329), FP32 ops in order."""
    axes = [np.asarray(v, np.float32) for v in (x, y, z)]
    n = len(axes[0])
    stride = n // N
    out = np.zeros((N, 3), np.float32)
    for a in range(3):
        lo, hi = axes[a].min(), axes[a].max()
        scale = np.float32(2.0) / np.float32(hi - lo)
        t = (axes[a][stride * np.arange(N)] + np.float32(-lo)).astype(np.float32)
        out[:, a] = ((t * scale).astype(np.float32) + np.float32(-1.0)).astype(np.float32)
    return out
