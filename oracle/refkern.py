"""The reference's own CUDA kernels, run through the driver-API harness
(refkern.c).  TEST INFRASTRUCTURE ONLY: used by the GPU parity tests and by
bench.py's reference arm, never by the product package.

``RefKernels.available()`` is False where the cubins were not built (no
reference checkout where ``oracle/build.py`` ran) or no GPU is present.

Noise: Leapfrog_HH draws white noise with ``curand_normal`` on the neuron's
XORWOW state (src/ephys.cu:88).  curand's normal generator returns a cached
second Box-Muller value when the state's ``boxmuller_flag`` is set
(curand_normal.h), so a state array with that flag set and
``boxmuller_extra = z`` makes the reference kernel draw exactly ``z``.
``xorwow_states_with_draw`` builds such an array; the parity tests pass the
same ``z`` to the library's ``nn_hh_leapfrog_step_z``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .build import build_refkern, ref_cubin_path

# curandStateXORWOW (curand_kernel.h): d, v[5], boxmuller_flag,
# boxmuller_flag_double, boxmuller_extra, (padding), boxmuller_extra_double
XORWOW_DTYPE = np.dtype([("d", np.uint32), ("v", np.uint32, 5), ("flag", np.int32), ("flag_double", np.int32),
                         ("extra", np.float32), ("pad", np.uint32), ("extra_double", np.float64)])
assert XORWOW_DTYPE.itemsize == 48

# src/defines.cuh:81-84; the whole-brain variant launches 512 threads per
# block (src_wholebrain/defines.cuh:46-47)
NBLOCKS, NTHREADS, NCHUNKS, N_PER_CHUNK = 32, 64, 2, 7319
WB_NTHREADS = 512
SRC, WHOLEBRAIN = 0, 1
CUBINS = ("ephys", "coupling", "wb_ephys", "wb_coupling")

_lib = None


def xorwow_states_with_draw(z: np.ndarray) -> np.ndarray:
    """One state per neuron whose next curand_normal returns z[i]."""
    st = np.zeros(len(z), XORWOW_DTYPE)
    st["flag"] = 1
    st["extra"] = np.asarray(z, np.float32)
    return st


def _load() -> C.CDLL:
    global _lib
    if _lib is None:
        l = C.CDLL(str(build_refkern()))
        u64, i, f = C.c_uint64, C.c_int, C.c_float
        sig = {
            "rk_last_error": (C.c_char_p, []),
            "rk_load": (i, [i, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p]),
            "rk_leapfrog": (i, [i, u64, i, f, u64, i, i]),
            "rk_init_random": (i, [C.c_uint, i, u64, i, i]),
            "rk_signal_spikes": (i, [i, i, u64, u64, u64, u64, u64, i, i]),
            "rk_signal_spikes_chunked": (i, [i, u64, u64, u64, u64, u64, u64]),
            "rk_time_leapfrog": (i, [i, u64, i, f, u64, i, i, i, C.POINTER(f)]),
            "rk_time_signal_spikes": (i, [i, i, u64, u64, u64, u64, u64, i, i, i, C.POINTER(f)]),
            "rk_malloc": (i, [u64, C.POINTER(u64)]),
            "rk_free": (i, [u64]),
            "rk_h2d": (i, [u64, C.c_void_p, u64]),
            "rk_d2h": (i, [C.c_void_p, u64, u64]),
            "rk_memset": (i, [u64, u64]),
            "rk_num_sms": (i, [C.POINTER(i)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(l, name)
            fn.restype, fn.argtypes = res, args
        _lib = l
    return _lib


class RefKernels:
    """Leapfrog_HH, init_random, signal_spikes_kernel(_chunked) and
    merge_kernel of the reference (variant SRC: src/; WHOLEBRAIN:
    src_wholebrain/, Leapfrog_HH and signal_spikes_kernel only), compiled
    from its sources for sm_103a.  Device pointers are plain integers (from
    any allocator of the primary context)."""

    def __init__(self, device: int = 0):
        self.lib = _load()
        paths = [ref_cubin_path(n) for n in CUBINS]
        missing = [str(p) for p in paths if not p.exists()]
        if missing:
            raise FileNotFoundError("reference kernel cubins not built: " + ", ".join(missing))
        self._check(self.lib.rk_load(device, *[str(p).encode() for p in paths]))

    @staticmethod
    def available() -> bool:
        return all(ref_cubin_path(n).exists() for n in CUBINS)

    def _check(self, rc: int) -> None:
        if rc != 0:
            raise RuntimeError(f"reference kernel harness: {self.lib.rk_last_error().decode()}")

    def leapfrog(self, d_table: int, n: int, dt: float, d_states: int, variant: int = SRC, grid: int = NBLOCKS,
                 block: int | None = None) -> None:
        block = block or (NTHREADS if variant == SRC else WB_NTHREADS)
        self._check(self.lib.rk_leapfrog(variant, d_table, n, dt, d_states, grid, block))

    def init_random(self, seed: int, n: int, d_states: int) -> None:
        self._check(self.lib.rk_init_random(seed, n, d_states, NBLOCKS, NTHREADS))

    def signal_spikes(self, num_firing: int, d_conn: int, d_off: int, d_firing: int, d_spikes: int,
                      d_outputs: int, variant: int = SRC, grid: int = NBLOCKS, block: int | None = None) -> None:
        block = block or (NTHREADS if variant == SRC else WB_NTHREADS)
        self._check(self.lib.rk_signal_spikes(variant, num_firing, d_conn, d_off, d_firing, d_spikes, d_outputs, grid,
                                              block))

    def signal_spikes_chunked(self, num_firing: int, d_conn_chunks: int, d_off_chunks: int, d_firing: int,
                              d_copies: int, d_spikes: int, d_outputs: int) -> None:
        self._check(self.lib.rk_signal_spikes_chunked(num_firing, d_conn_chunks, d_off_chunks, d_firing, d_copies,
                                                      d_spikes, d_outputs))

    def time_leapfrog(self, d_table: int, n: int, dt: float, d_states: int, grid: int, block: int,
                      reps: int, variant: int = SRC) -> float:
        ms = C.c_float()
        self._check(self.lib.rk_time_leapfrog(variant, d_table, n, dt, d_states, grid, block, reps, C.byref(ms)))
        return ms.value

    def time_signal_spikes(self, num_firing: int, d_conn: int, d_off: int, d_firing: int, d_spikes: int,
                           d_outputs: int, grid: int, block: int, reps: int, variant: int = SRC) -> float:
        ms = C.c_float()
        self._check(self.lib.rk_time_signal_spikes(variant, num_firing, d_conn, d_off, d_firing, d_spikes, d_outputs,
                                                   grid, block, reps, C.byref(ms)))
        return ms.value

    # device memory without the product library (the benchmark's reference arm)
    def to_device(self, a: np.ndarray) -> int:
        a = np.ascontiguousarray(a)
        d = C.c_uint64()
        self._check(self.lib.rk_malloc(a.nbytes, C.byref(d)))
        self._check(self.lib.rk_h2d(d.value, a.ctypes.data, a.nbytes))
        return d.value

    def zeros(self, nbytes: int) -> int:
        d = C.c_uint64()
        self._check(self.lib.rk_malloc(nbytes, C.byref(d)))
        self._check(self.lib.rk_memset(d.value, nbytes))
        return d.value

    def to_host(self, dptr: int, shape, dtype) -> np.ndarray:
        out = np.empty(shape, dtype)
        self._check(self.lib.rk_d2h(out.ctypes.data, dptr, out.nbytes))
        return out

    def free(self, dptr: int) -> None:
        self._check(self.lib.rk_free(dptr))

    def num_sms(self) -> int:
        n = C.c_int()
        self._check(self.lib.rk_num_sms(C.byref(n)))
        return n.value
