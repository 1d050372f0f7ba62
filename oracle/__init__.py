"""ctypes access to the CPU oracle (oracle.c).  TEST INFRASTRUCTURE ONLY.

Imported by tests/, by __graft_entry__.smoke() as the checker and by
bench.py's CPU-baseline leg; never by the product package.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .build import build_oracle

P = C.POINTER
_lib = None


class OrcLeapfrogParams(C.Structure):
    _fields_ = [(n, C.c_float) for n in (
        "gna", "ena", "gk", "ek", "gl", "el", "Tmax", "Vt", "Kp", "Ar", "Ad",
        "g_local", "e_local", "g_gaba", "e_gaba", "g_exc", "e_exc", "noise_mean", "noise_intensity")]


class OrcHHParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "C", "gNa", "gK", "gL", "ENa", "EK", "EL", "E_exc", "E_inh", "tau_exc", "tau_inh",
        "v_thresh", "noise_sigma", "dt", "g_par", "E_par")]


class OrcCSR(C.Structure):
    _fields_ = [("n", C.c_int), ("nnz", C.c_int64), ("row_ptr", C.c_void_p), ("col", C.c_void_p),
                ("weight", C.c_void_p), ("delay", C.c_void_p)]


class OrcSim(C.Structure):
    _fields_ = [("hp", OrcHHParams), ("n", C.c_int), ("D", C.c_int), ("net", P(OrcCSR)),
                ("is_inh", C.c_void_p), ("i_drive", C.c_void_p), ("gna_scale", C.c_void_p),
                ("u_par", C.c_void_p), ("seed", C.c_uint64), ("y", C.c_void_p), ("ring", C.c_void_p),
                ("vox", C.c_void_p), ("src", C.c_void_p), ("margin", C.c_void_p)]


V = C.c_void_p
_SIGS = {
    "orc_philox4x32_10": (None, [V, V, V]),
    "orc_philox2x32_10": (None, [V, C.c_uint32, V]),
    "orc_normal_ctr": (C.c_double, [C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint32]),
    "orc_minstd_next": (C.c_uint32, [P(C.c_uint32)]),
    "orc_uniform_int": (C.c_int, [P(C.c_uint32), C.c_int, C.c_int]),
    "orc_uniform_random_network": (None, [C.c_int, C.c_int, P(C.c_uint32), V, V]),
    "orc_tcount": (None, [V, C.c_int64, C.c_int, V]),
    "orc_chunked": (None, [V, V, C.c_int, C.c_int, C.c_int, P(C.c_void_p), P(C.c_void_p), V]),
    "orc_leapfrog_params_src": (None, [P(OrcLeapfrogParams)]),
    "orc_leapfrog_params_wholebrain": (None, [P(OrcLeapfrogParams)]),
    "orc_hh_leapfrog": (None, [P(C.c_void_p), C.c_int, C.c_float, P(OrcLeapfrogParams), V]),
    "orc_coupling_push": (C.c_int, [C.c_int, V, V, V, V, C.c_int, V]),
    "orc_trilinear_setup": (None, [C.c_int, V, V, V, C.c_int, C.c_int, C.c_int, C.c_float, V, V]),
    "orc_scatter": (None, [C.c_int, V, V, V, V]),
    "orc_interp": (None, [C.c_int, V, V, V, V]),
    "orc_conv27": (None, [V, V, C.c_int, C.c_int, C.c_int, V]),
    "orc_paracrine_cn_solve": (C.c_int, [V, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                         C.c_double, C.c_double, C.c_int, C.c_int, P(C.c_double)]),
    "orc_hh_params_standard": (None, [P(OrcHHParams)]),
    "orc_hh_steady_state": (None, [C.c_double, P(C.c_double), P(C.c_double), P(C.c_double)]),
    "orc_hh_rk4": (None, [P(OrcHHParams), C.c_double, C.c_double, C.c_double, V]),
    "orc_csr_to_csc": (None, [P(OrcCSR), V, V, V, V, V]),
    "orc_gen_er": (None, [C.c_int, C.c_double, C.c_float, C.c_uint64, P(OrcCSR)]),
    "orc_gauss_table": (None, [C.c_double, V]),
    "orc_local_gaussian": (C.c_int64, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_int, C.c_uint64,
                                       C.c_void_p, C.c_void_p, C.c_int64]),
    "orc_gen_block": (None, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double,
                             C.c_uint64, C.c_void_p]),
    "orc_gen_gauss": (None, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_uint64,
                             P(OrcCSR)]),
    "orc_lattice_positions": (None, [C.c_int, C.c_uint64, V, V, V]),
    "orc_init_drive": (None, [C.c_int, C.c_uint64, C.c_float, C.c_float, V]),
    "orc_inh_flags": (None, [C.c_int, C.c_double, C.c_int, C.c_uint64, V]),
    "orc_sim_step": (C.c_int, [P(OrcSim), C.c_uint64, V]),
    "orc_apply7": (None, [V, V, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, V]),
    "orc_pcg7": (C.c_int, [V, V, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, V, C.c_double, C.c_int,
                           P(C.c_double)]),
    "orc_num_threads": (C.c_int, []),
}


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        l = C.CDLL(str(build_oracle()))
        for name, (res, args) in _SIGS.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def ptr(a: np.ndarray | None) -> C.c_void_p | None:
    """Pointer to a contiguous array; the returned object keeps the array alive
    (so temporaries passed as ptr(np.ascontiguousarray(...)) stay valid)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


# ------------------------------------------------------------ helpers ------

def philox(ctr, key) -> np.ndarray:
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(ptr(c), ptr(k), ptr(out))
    return out


def philox2(ctr, key: int) -> np.ndarray:
    c = np.asarray(ctr, np.uint32)
    out = np.zeros(2, np.uint32)
    lib().orc_philox2x32_10(ptr(c), key, ptr(out))
    return out


def uniform_random_network(n: int, ncouple: int, engine: C.c_uint32):
    ind = np.zeros(n * ncouple, np.int32)
    off = np.zeros(n + 1, np.int32)
    lib().orc_uniform_random_network(n, ncouple, C.byref(engine), ptr(ind), ptr(off))
    return ind, off


def tcount(indices: np.ndarray, n: int) -> np.ndarray:
    out = np.zeros(n, np.float32)
    lib().orc_tcount(ptr(np.ascontiguousarray(indices, np.int32)), len(indices), n, ptr(out))
    return out


def chunked(indices, offsets, n, nchunks, n_per_chunk):
    indices = np.ascontiguousarray(indices, np.int32)
    offsets = np.ascontiguousarray(offsets, np.int32)
    ci = [np.zeros(max(len(indices), 1), np.int32) for _ in range(nchunks)]
    co = [np.zeros(n + 1, np.int32) for _ in range(nchunks)]
    cnt = np.zeros(nchunks, np.int64)
    lib().orc_chunked(ptr(indices), ptr(offsets), n, nchunks, n_per_chunk,
                      (C.c_void_p * nchunks)(*[a.ctypes.data for a in ci]),
                      (C.c_void_p * nchunks)(*[a.ctypes.data for a in co]), ptr(cnt))
    return [ci[c][:cnt[c]] for c in range(nchunks)], co


def leapfrog_params(variant: int = 0) -> OrcLeapfrogParams:
    p = OrcLeapfrogParams()
    (lib().orc_leapfrog_params_src if variant == 0 else lib().orc_leapfrog_params_wholebrain)(C.byref(p))
    return p


def hh_leapfrog(vars17: list[np.ndarray], dt: float, params: OrcLeapfrogParams, z: np.ndarray) -> None:
    n = len(vars17[0])
    table = (C.c_void_p * 17)(*[v.ctypes.data for v in vars17])
    lib().orc_hh_leapfrog(table, n, dt, C.byref(params), ptr(np.ascontiguousarray(z, np.float64)))


def normal_ctr(seed: int, i: int, step: int, purpose: int = 1) -> float:
    return lib().orc_normal_ctr(seed, i, step, purpose)


def normals(seed: int, n: int, step: int, purpose: int = 1) -> np.ndarray:
    return np.array([lib().orc_normal_ctr(seed, i, step, purpose) for i in range(n)], np.float64)


def coupling_push(indices, offsets, outputs, signal_mode=0):
    n = len(outputs)
    inputs = np.zeros(n, np.float32)
    firing = np.zeros(n, np.int32)
    nf = lib().orc_coupling_push(n, ptr(np.ascontiguousarray(indices, np.int32)),
                                 ptr(np.ascontiguousarray(offsets, np.int32)),
                                 ptr(np.ascontiguousarray(outputs, np.float32)), ptr(inputs), signal_mode, ptr(firing))
    return nf, inputs, firing[:nf]


def trilinear(x, y, z, nx, ny, nz, h):
    n = len(x)
    idx = np.zeros(8 * n, np.int32)
    w = np.zeros(8 * n, np.float32)
    xs, ys, zs = (np.ascontiguousarray(a, np.float32) for a in (x, y, z))
    lib().orc_trilinear_setup(n, ptr(xs), ptr(ys), ptr(zs), nx, ny, nz, h, ptr(idx), ptr(w))
    return idx, w


def conv27(u: np.ndarray, shape, K: np.ndarray) -> np.ndarray:
    nz, ny, nx = shape
    u = np.ascontiguousarray(u, np.float64)
    out = np.zeros_like(u)
    lib().orc_conv27(ptr(u), ptr(out), nx, ny, nz, ptr(np.ascontiguousarray(K, np.float64)))
    return out


def paracrine_cn_solve(u: np.ndarray, shape, h, D, k, dt, abs_tol=1e-6, max_iter=20, quirk_b=1):
    nz, ny, nx = shape
    u = np.ascontiguousarray(u, np.float64).copy()
    rr = C.c_double(0)
    it = lib().orc_paracrine_cn_solve(ptr(u), nx, ny, nz, h, D, k, dt, abs_tol, max_iter, quirk_b, C.byref(rr))
    return u, it, rr.value


def hh_params() -> OrcHHParams:
    p = OrcHHParams()
    lib().orc_hh_params_standard(C.byref(p))
    return p


def steady_state(v: float):
    m, h, n = C.c_double(), C.c_double(), C.c_double()
    lib().orc_hh_steady_state(v, C.byref(m), C.byref(h), C.byref(n))
    return m.value, h.value, n.value


class CSR:
    """Owning wrapper of an orc_csr."""

    def __init__(self, row_ptr, col, weight, delay):
        self.row_ptr = np.ascontiguousarray(row_ptr, np.int64)
        self.col = np.ascontiguousarray(col, np.int32)
        self.weight = np.ascontiguousarray(weight, np.float32)
        self.delay = np.ascontiguousarray(delay, np.uint8)
        self.n = len(self.row_ptr) - 1
        self.s = OrcCSR(self.n, len(self.col), self.row_ptr.ctypes.data, self.col.ctypes.data,
                        self.weight.ctypes.data, self.delay.ctypes.data)


def gen_er(n: int, p: float, wmax: float, seed: int) -> CSR:
    rp = np.zeros(n + 1, np.int64)
    s = OrcCSR(n, 0, rp.ctypes.data, None, None, None)
    lib().orc_gen_er(n, p, wmax, seed, C.byref(s))
    nnz = int(rp[-1])
    col = np.zeros(max(nnz, 1), np.int32)
    w = np.zeros(max(nnz, 1), np.float32)
    d = np.zeros(max(nnz, 1), np.uint8)
    s2 = OrcCSR(n, 0, rp.ctypes.data, col.ctypes.data, w.ctypes.data, d.ctypes.data)
    lib().orc_gen_er(n, p, wmax, seed, C.byref(s2))
    return CSR(rp, col[:nnz], w[:nnz], d[:nnz])


def gen_gauss(n: int, k: int, sigma: float, mu: float, sg: float, dmax: int, seed: int) -> CSR:
    rp = np.zeros(n + 1, np.int64)
    col = np.zeros(n * k, np.int32)
    w = np.zeros(n * k, np.float32)
    d = np.zeros(n * k, np.uint8)
    s = OrcCSR(n, 0, rp.ctypes.data, col.ctypes.data, w.ctypes.data, d.ctypes.data)
    lib().orc_gen_gauss(n, k, sigma, mu, sg, dmax, seed, C.byref(s))
    return CSR(rp, col, w, d)


def gen_block(n: int, k: int, R: int, size_sigma: float, density_sigma: float, dmax: int, mu: float, sg: float,
              seed: int) -> CSR:
    rp = np.zeros(n + 1, np.int64)
    col = np.zeros(n * k, np.int32)
    w = np.zeros(n * k, np.float32)
    d = np.zeros(n * k, np.uint8)
    s = OrcCSR(n, 0, rp.ctypes.data, col.ctypes.data, w.ctypes.data, d.ctypes.data)
    lib().orc_gen_block(n, k, R, size_sigma, density_sigma, dmax, mu, sg, seed, C.byref(s))
    return CSR(rp, col, w, d)


def local_gaussian(x, y, z, stddev: float, n_stddevs: int, seed: int):
    """(offsets, indices) of the local Gaussian-ball network."""
    x, y, z = (np.ascontiguousarray(v, np.float32) for v in (x, y, z))
    n = len(x)
    off = np.zeros(n + 1, np.int32)
    nnz = lib().orc_local_gaussian(n, ptr(x), ptr(y), ptr(z), stddev, n_stddevs, seed, ptr(off), None, 0)
    idx = np.zeros(max(nnz, 1), np.int32)
    lib().orc_local_gaussian(n, ptr(x), ptr(y), ptr(z), stddev, n_stddevs, seed, ptr(off), ptr(idx), nnz)
    return off, idx[:nnz]


def gauss_table(sigma_sites: float) -> np.ndarray:
    t = np.zeros(4096, np.int16)
    lib().orc_gauss_table(sigma_sites, ptr(t))
    return t


def lattice_positions(n: int, seed: int):
    x, y, z = (np.zeros(n, np.float32) for _ in range(3))
    lib().orc_lattice_positions(n, seed, ptr(x), ptr(y), ptr(z))
    return x, y, z


def init_drive(n: int, seed: int, lo: float, hi: float) -> np.ndarray:
    """Drive currents of the device's initial state (nn_sim_init_state)."""
    out = np.zeros(n, np.float32)
    lib().orc_init_drive(n, seed, lo, hi, ptr(out))
    return out


def inh_flags(n: int, frac: float, random: bool, seed: int) -> np.ndarray:
    """Inhibitory flags of the device generators (k_inh)."""
    out = np.zeros(n, np.uint8)
    lib().orc_inh_flags(n, frac, 1 if random else 0, seed, ptr(out))
    return out


def rest_state(n: int, v0: float = -65.0) -> np.ndarray:
    """(6, n) state V, m, h, n, ge, gi at rest: gates at their steady state."""
    m, h, nn_ = steady_state(v0)
    st = np.zeros((6, n), np.float64)
    st[0], st[1], st[2], st[3] = v0, np.float32(m), np.float32(h), np.float32(nn_)
    return st


def voxels(x, y, z, grid: int) -> np.ndarray:
    """Voxel of each position on a grid^3 over the unit cube (k_init_state)."""
    g = np.float32(grid)
    ix = np.clip((np.asarray(x, np.float32) * g).astype(np.int32), 0, grid - 1)
    iy = np.clip((np.asarray(y, np.float32) * g).astype(np.int32), 0, grid - 1)
    iz = np.clip((np.asarray(z, np.float32) * g).astype(np.int32), 0, grid - 1)
    return (ix + grid * (iy + grid * iz)).astype(np.int32)


def csr_to_csc(a: CSR):
    cp = np.zeros(a.n + 1, np.int64)
    nnz = len(a.col)
    src = np.zeros(max(nnz, 1), np.int32)
    w = np.zeros(max(nnz, 1), np.float32)
    d = np.zeros(max(nnz, 1), np.uint8)
    lib().orc_csr_to_csc(C.byref(a.s), ptr(cp), ptr(src), ptr(w), ptr(d), None)
    return cp, src[:nnz], w[:nnz], d[:nnz]


class Sim:
    """FP64 oracle of the simulation step (orc_sim_step)."""

    def __init__(self, net: CSR, is_inh, i_drive, seed: int, D: int, state6: np.ndarray,
                 hp: OrcHHParams | None = None, gna_scale=None, vox=None, grid_cells: int = 0):
        self.net = net
        self.hp = hp or hh_params()
        self.n = net.n
        self.is_inh = np.ascontiguousarray(is_inh, np.uint8)
        self.i_drive = np.ascontiguousarray(i_drive, np.float32)
        self.gna = None if gna_scale is None else np.ascontiguousarray(gna_scale, np.float32)
        self.y = np.ascontiguousarray(np.asarray(state6, np.float64).reshape(6, self.n).T.copy())
        self.ring = np.zeros(2 * D * self.n, np.float64)
        self.vox = None if vox is None else np.ascontiguousarray(vox, np.int32)
        self.src = np.zeros(grid_cells, np.float64) if grid_cells else None
        self._margin = np.zeros(self.n, np.float64)
        self.s = OrcSim(self.hp, self.n, D, C.pointer(net.s), self.is_inh.ctypes.data, self.i_drive.ctypes.data,
                        None if self.gna is None else self.gna.ctypes.data, None, seed, self.y.ctypes.data,
                        self.ring.ctypes.data, None if self.vox is None else self.vox.ctypes.data,
                        None if self.src is None else self.src.ctypes.data, self._margin.ctypes.data)
        self.t = 0
        self._spk = np.zeros(self.n, np.int32)
        self.margins: dict[tuple[int, int], float] = {}  # (step, neuron) -> threshold-crossing margin (mV)

    def step(self) -> np.ndarray:
        ns = lib().orc_sim_step(C.byref(self.s), self.t, ptr(self._spk))
        spk = self._spk[:ns].copy()
        for j in spk:
            self.margins[(self.t, int(j))] = float(self._margin[j])
        self.t += 1
        return spk

    def state(self) -> np.ndarray:
        return self.y.T.copy()  # (6, n): V, m, h, n, ge, gi


def apply7(x: np.ndarray, shape, alpha, beta, D=None) -> np.ndarray:
    nz, ny, nx = shape
    x = np.ascontiguousarray(x, np.float64).ravel()
    y = np.zeros_like(x)
    lib().orc_apply7(ptr(x), ptr(y), nx, ny, nz, alpha, beta,
                     None if D is None else ptr(np.ascontiguousarray(D, np.float32).ravel()))
    return y


def pcg7(b: np.ndarray, x0: np.ndarray, shape, alpha, beta, D=None, rtol=1e-6, max_iter=10000):
    nz, ny, nx = shape
    b = np.ascontiguousarray(b, np.float64).ravel()
    x = np.ascontiguousarray(x0, np.float64).ravel().copy()
    rel = C.c_double(0)
    it = lib().orc_pcg7(ptr(x), ptr(b), nx, ny, nz, alpha, beta,
                        None if D is None else ptr(np.ascontiguousarray(D, np.float32).ravel()),
                        rtol, max_iter, C.byref(rel))
    return x, it, rel.value
