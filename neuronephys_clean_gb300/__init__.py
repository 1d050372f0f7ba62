"""GB300-native neuronephys simulation path (Python host side).

Mirrors the reference's C++ interfaces over the C ABI in include/neuronephys.h:

* ``HHEphys``            -- Ephys/HHEphys::SimulateEphys (src/ephys.cuh:6-31)
* ``AtomicCoupling``     -- AtomicCoupling::operator() (src/coupling.cuh:17-38)
* ``UniformRandomNetwork`` / ``Network.to_adjacency_list`` /
  ``Network.to_chunked_adjacency_list`` -- src/network_factory.cuh:6-67
* ``ParacrineModule``    -- src/paracrine.cuh:212-267
* ``Simulation``         -- the step loop (src/main.cu:112-182) as one
  device-resident object: RK4 HH, delayed weighted delivery, 7-point PCG field
* ``PCG``                -- standalone 7-point Jacobi-PCG

Every call runs CUDA code in libneuronephys; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from ._lib import HHParams, KernelTimes, LeapfrogParams, NetSpec, ParacrineRefParams, SimConfig, SolveStats

__all__ = ["NNError", "Context", "DeviceArray", "HHEphys", "AtomicCoupling", "AdjacencyList",
           "ChunkedAdjacencyList", "UniformRandomNetwork", "ParacrineModule", "Simulation", "PCG", "MultigridPCG", "LearnedMultigrid",
           "SimConfig", "HHParams", "NetSpec", "LeapfrogParams", "ParacrineRefParams",
           "lib", "NN_SIGNAL_COUNT", "NN_SIGNAL_OUTPUT", "FIELDS"]

NN_SIGNAL_COUNT, NN_SIGNAL_OUTPUT = 0, 1
NN_DELIVERY_PUSH, NN_DELIVERY_PULL, NN_DELIVERY_AUTO = 0, 1, 2
NN_NET_ER, NN_NET_GAUSS, NN_NET_BLOCK = 1, 2, 3
NN_ERR_NOT_CONVERGED = 4
FIELDS = {name: i for i, name in enumerate(
    ["V", "M", "H", "N", "GE", "GI", "IDRIVE", "GNA_SCALE", "X", "Y", "Z", "UPAR"])}
# reference SoA slots (src/defines.cuh:57-78)
SIM_PARAMS = ["V", "M", "N", "H", "LOCAL_Y", "IY", "EY", "LOCAL_OUTPUT", "LOCAL_IN", "LOCAL_COUNT",
              "EOUTPUT", "EIN", "ECOUNT", "IOUTPUT", "IIN", "ICOUNT", "APPCUR"]


def lib() -> C.CDLL:
    return L.load()


class NNError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


def _check(st: int, ctx: "Context | None" = None, what: str = "") -> None:
    if st != 0:
        l = lib()
        detail = l.nn_status_string(st).decode()
        if ctx is not None and ctx.handle:
            le = l.nn_ctx_last_error(ctx.handle).decode()
            if le:
                detail += ": " + le
        raise NNError(st, f"{what}: {detail}" if what else detail)


def _ptr(a: np.ndarray) -> C.c_void_p:
    """Pointer to a contiguous array; the returned object keeps the array alive."""
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


class Context:
    """One CUDA device and stream (nn_ctx)."""

    def __init__(self, device: int = 0):
        self.handle = C.c_void_p()
        _check(lib().nn_ctx_create(device, C.byref(self.handle)), None, "nn_ctx_create")

    def close(self) -> None:
        if self.handle:
            lib().nn_ctx_destroy(self.handle)
            self.handle = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def synchronize(self) -> None:
        _check(lib().nn_ctx_synchronize(self.handle), self, "synchronize")

    @property
    def kernel_launches(self) -> int:
        return int(lib().nn_ctx_kernel_launches(self.handle))

    @property
    def num_sms(self) -> int:
        return int(lib().nn_ctx_num_sms(self.handle))

    def time_begin(self) -> None:
        """Record a CUDA event on the context stream."""
        _check(lib().nn_ctx_time_begin(self.handle), self, "time_begin")

    def time_end(self) -> float:
        """Record a second event, synchronise, return the elapsed ms."""
        ms = C.c_float()
        _check(lib().nn_ctx_time_end(self.handle, C.byref(ms)), self, "time_end")
        return float(ms.value)

    def empty(self, shape, dtype) -> "DeviceArray":
        return DeviceArray(self, shape, dtype)

    def to_device(self, a: np.ndarray) -> "DeviceArray":
        a = np.ascontiguousarray(a)
        d = DeviceArray(self, a.shape, a.dtype)
        d.copy_from(a)
        return d


class PinnedArray:
    """Page-locked host array (nn_host_alloc), viewed as a numpy array."""

    def __init__(self, shape, dtype):
        dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dtype.itemsize
        self.ptr = C.c_void_p()
        _check(lib().nn_host_alloc(max(nbytes, 1), C.byref(self.ptr)), None, "nn_host_alloc")
        buf = (C.c_char * max(nbytes, 1)).from_address(self.ptr.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def free(self) -> None:
        if self.ptr:
            self.array = None
            lib().nn_host_free(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class DeviceArray:
    """Device buffer owned through the C ABI (nn_malloc/nn_free)."""

    def __init__(self, ctx: Context, shape, dtype):
        self.ctx = ctx
        self.shape = tuple(np.atleast_1d(shape).tolist()) if not isinstance(shape, tuple) else shape
        self.dtype = np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        self.ptr = C.c_void_p()
        _check(lib().nn_malloc(ctx.handle, max(self.nbytes, 1), C.byref(self.ptr)), ctx, "nn_malloc")

    @property
    def value(self) -> int:
        return int(self.ptr.value or 0)

    def copy_from(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=self.dtype)
        assert a.nbytes == self.nbytes, (a.nbytes, self.nbytes)
        _check(lib().nn_memcpy_h2d(self.ctx.handle, self.ptr, _ptr(a), a.nbytes), self.ctx, "h2d")

    def numpy(self) -> np.ndarray:
        out = np.empty(self.shape, self.dtype)
        _check(lib().nn_memcpy_d2h(self.ctx.handle, _ptr(out), self.ptr, self.nbytes), self.ctx, "d2h")
        return out

    def zero(self) -> None:
        _check(lib().nn_memset_d(self.ctx.handle, self.ptr, 0, self.nbytes), self.ctx, "memset")

    def free(self) -> None:
        if self.ptr and self.ctx.handle:
            lib().nn_free(self.ctx.handle, self.ptr)
        self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ------------------------------------------------------- reference mirrors --

class HHEphys:
    """HHEphys with the struct-of-arrays it owns (src_wholebrain/ephys.cuh:6-43).

    ``simulate_ephys()`` is HHEphys::SimulateEphys: one Leapfrog_HH step
    (src/ephys.cu:28-103) of all neurons at dt = leapfrog_dt = 0.4 ms.
    """

    def __init__(self, ctx: Context, n: int, variant: int = 0, seed: int = 0, dt: float = 0.4):
        self.ctx, self.n, self.seed, self.dt, self.step = ctx, n, seed, dt, 0
        self.params = LeapfrogParams()
        lib().nn_leapfrog_params_reference(C.byref(self.params), variant)
        self.vars = [ctx.empty((n,), np.float32) for _ in SIM_PARAMS]
        for v in self.vars:
            v.zero()

    def sim_vars_cpu(self) -> list[int]:
        return [v.value for v in self.vars]

    def set(self, name: str, values) -> None:
        self.vars[SIM_PARAMS.index(name)].copy_from(np.broadcast_to(np.asarray(values, np.float32), (self.n,)))

    def get(self, name: str) -> np.ndarray:
        return self.vars[SIM_PARAMS.index(name)].numpy()

    def simulate_ephys(self, z: "DeviceArray | None" = None) -> None:
        """One step; z (device float[n], optional) supplies the standard
        normal draws of the noise term instead of the library's stream."""
        table = (C.c_void_p * len(self.vars))(*[v.value for v in self.vars])
        if z is None:
            _check(lib().nn_hh_leapfrog_step(self.ctx.handle, table, self.n, self.dt, C.byref(self.params),
                                             self.seed, self.step), self.ctx, "SimulateEphys")
        else:
            _check(lib().nn_hh_leapfrog_step_z(self.ctx.handle, table, self.n, self.dt, C.byref(self.params),
                                               C.c_void_p(z.value)), self.ctx, "SimulateEphys")
        self.step += 1


@dataclass
class AdjacencyList:
    """Device CSR, row = presynaptic (src/coupling.cuh:4-8)."""
    indices: DeviceArray
    offset_in_indices: DeviceArray


@dataclass
class ChunkedAdjacencyList:
    """Per-chunk device CSR with chunk-local targets (src/coupling.cuh:10-14)."""
    indices_chunks: list
    offset_in_indices_chunks: list
    n_per_chunk: int
    chunk_nnz: list


class AtomicCoupling:
    """AtomicCoupling (src/coupling.cuh:17-38)."""

    def __init__(self, ctx: Context, n: int):
        self.ctx, self.n = ctx, n
        self.handle = C.c_void_p()
        _check(lib().nn_coupling_create(ctx.handle, n, C.byref(self.handle)), ctx, "AtomicCoupling")

    def __call__(self, connectivity, spikes: DeviceArray, neuron_outputs: DeviceArray,
                 signal_mode: int = NN_SIGNAL_COUNT, read_count: bool = True) -> int | None:
        nf = C.c_int(-1)
        pnf = C.byref(nf) if read_count else None
        if isinstance(connectivity, ChunkedAdjacencyList):
            k = len(connectivity.indices_chunks)
            ci = (C.c_void_p * k)(*[a.value for a in connectivity.indices_chunks])
            co = (C.c_void_p * k)(*[a.value for a in connectivity.offset_in_indices_chunks])
            st = lib().nn_coupling_run_chunked(self.handle, k, connectivity.n_per_chunk, ci, co, spikes.ptr,
                                               neuron_outputs.ptr, pnf)
        else:
            st = lib().nn_coupling_run(self.handle, connectivity.indices.ptr, connectivity.offset_in_indices.ptr,
                                       spikes.ptr, neuron_outputs.ptr, signal_mode, pnf)
        _check(st, self.ctx, "AtomicCoupling()")
        return nf.value if read_count else None

    def get_firing_neurons(self) -> np.ndarray:
        """GetFiringNeurons(): the full n-entry buffer (src/coupling.cuh:37)."""
        out = np.empty(self.n, np.int32)
        p = lib().nn_coupling_firing_list(self.handle)
        _check(lib().nn_memcpy_d2h(self.ctx.handle, _ptr(out), C.c_void_p(p), out.nbytes), self.ctx)
        return out

    def close(self):
        if self.handle:
            lib().nn_coupling_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Network:
    """Host-side CSR (src/network_factory.cuh:6-53)."""

    def __init__(self):
        self.indices = np.zeros(0, np.int32)
        self.offset_in_indices = np.zeros(1, np.int32)

    @property
    def n(self) -> int:
        return len(self.offset_in_indices) - 1

    def to_adjacency_list(self, ctx: Context, tcount: DeviceArray) -> AdjacencyList:
        """ToAdjacencyList(Float*& Tcount) (src/network_factory.cu:5-27)."""
        lst = AdjacencyList(ctx.to_device(self.indices), ctx.to_device(self.offset_in_indices))
        _check(lib().nn_net_tcount(ctx.handle, lst.indices.ptr, len(self.indices), self.n, tcount.ptr), ctx,
               "ToAdjacencyList")
        return lst

    def to_chunked_adjacency_list(self, ctx: Context, tcount: DeviceArray, nchunks: int = 2,
                                  n_per_chunk: int = 7319) -> ChunkedAdjacencyList:
        """ToChunkedAdjacencyList(Float*& Tcount) (src/network_factory.cu:29-85)."""
        d_idx = ctx.to_device(self.indices)
        d_off = ctx.to_device(self.offset_in_indices)
        _check(lib().nn_net_tcount(ctx.handle, d_idx.ptr, len(self.indices), self.n, tcount.ptr), ctx, "Tcount")
        nnz = max(len(self.indices), 1)
        ci = [ctx.empty((nnz,), np.int32) for _ in range(nchunks)]
        co = [ctx.empty((self.n + 1,), np.int32) for _ in range(nchunks)]
        cnt = (C.c_int64 * nchunks)()
        _check(lib().nn_net_to_chunked(ctx.handle, d_idx.ptr, d_off.ptr, self.n, nchunks, n_per_chunk,
                                       (C.c_void_p * nchunks)(*[a.value for a in ci]),
                                       (C.c_void_p * nchunks)(*[a.value for a in co]), cnt), ctx,
               "ToChunkedAdjacencyList")
        return ChunkedAdjacencyList(ci, co, n_per_chunk, list(cnt))


class UniformRandomNetwork(Network):
    """UniformRandomNetwork (src/network_factory.cuh:56-67); the engine is the
    reference's shared default-constructed minstd_rand0 (state 1)."""

    engine = C.c_uint32(1)

    def __init__(self, ncouple: int):
        super().__init__()
        self.ncouple = ncouple

    @classmethod
    def reset_engine(cls, state: int = 1) -> None:
        cls.engine = C.c_uint32(state)

    def generate(self, n: int) -> bool:
        self.indices = np.zeros(n * self.ncouple, np.int32)
        self.offset_in_indices = np.zeros(n + 1, np.int32)
        st = lib().nn_net_uniform_random(n, self.ncouple, C.byref(UniformRandomNetwork.engine),
                                         _ptr(self.indices), _ptr(self.offset_in_indices))
        return st == 0


class ParacrineModule:
    """ParacrineModule (src/paracrine.cuh:212-267)."""

    def __init__(self, ctx: Context, d_g_paracrine: DeviceArray, n: int, params: ParacrineRefParams,
                 x: DeviceArray, y: DeviceArray, z: DeviceArray):
        self.ctx, self.n, self.params = ctx, n, params
        self.handle = C.c_void_p()
        _check(lib().nn_paracrine_ref_create(ctx.handle, C.byref(params), n, x.ptr, y.ptr, z.ptr,
                                             d_g_paracrine.ptr, C.byref(self.handle)), ctx, "ParacrineModule")
        self.G = params.nx * params.ny * params.nz

    @staticmethod
    def default_params() -> ParacrineRefParams:
        p = ParacrineRefParams()
        lib().nn_paracrine_ref_params_default(C.byref(p))
        return p

    def update_on_fine_timescale(self, coupling: AtomicCoupling) -> None:
        _check(lib().nn_paracrine_ref_fine(self.handle, coupling.handle), self.ctx, "update_on_fine_timescale")

    def update_on_own_timescale(self) -> tuple[int, float]:
        it, rr = C.c_int(0), C.c_float(0)
        _check(lib().nn_paracrine_ref_own(self.handle, C.byref(it), C.byref(rr)), self.ctx,
               "update_on_own_timescale")
        return it.value, rr.value

    def _read(self, p: int, count: int) -> np.ndarray:
        out = np.empty(count, np.float32)
        _check(lib().nn_memcpy_d2h(self.ctx.handle, _ptr(out), C.c_void_p(p), out.nbytes), self.ctx)
        return out

    def density(self) -> np.ndarray:
        return self._read(lib().nn_paracrine_density(self.handle), self.G)

    def set_density(self, u: np.ndarray) -> None:
        u = np.ascontiguousarray(u, np.float32).ravel()
        _check(lib().nn_memcpy_h2d(self.ctx.handle, C.c_void_p(lib().nn_paracrine_density(self.handle)), _ptr(u),
                                   u.nbytes), self.ctx)

    def sources(self) -> np.ndarray:
        return self._read(lib().nn_paracrine_sources(self.handle), self.n)

    def set_sources(self, s: np.ndarray) -> None:
        s = np.ascontiguousarray(s, np.float32)
        _check(lib().nn_memcpy_h2d(self.ctx.handle, C.c_void_p(lib().nn_paracrine_sources(self.handle)), _ptr(s),
                                   s.nbytes), self.ctx)

    def close(self):
        if self.handle:
            lib().nn_paracrine_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------- GB300 sim --

def default_config(n: int) -> SimConfig:
    c = SimConfig()
    lib().nn_sim_config_default(C.byref(c), n)
    return c


def default_net_spec(kind: int) -> NetSpec:
    s = NetSpec()
    lib().nn_net_spec_default(C.byref(s), kind)
    return s


class Simulation:
    """Device-resident network simulation (RK4 HH + delayed delivery + field)."""

    def __init__(self, ctx: Context, config: SimConfig):
        self.ctx, self.config, self.n = ctx, config, config.n
        self.handle = C.c_void_p()
        _check(lib().nn_sim_create(ctx.handle, C.byref(config), C.byref(self.handle)), ctx, "nn_sim_create")

    def close(self):
        if self.handle:
            lib().nn_sim_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_network(self, row_ptr, col, weight, delay, is_inh=None) -> None:
        row_ptr = np.ascontiguousarray(row_ptr, np.int64)
        col = np.ascontiguousarray(col, np.int32)
        weight = np.ascontiguousarray(weight, np.float32)
        delay = np.ascontiguousarray(delay, np.uint8)
        inh = None if is_inh is None else np.ascontiguousarray(is_inh, np.uint8)
        _check(lib().nn_sim_set_network(self.handle, _ptr(row_ptr), _ptr(col), _ptr(weight), _ptr(delay), len(col),
                                        None if inh is None else _ptr(inh)), self.ctx, "set_network")

    def generate_network(self, spec: NetSpec) -> int:
        _check(lib().nn_sim_generate_network(self.handle, C.byref(spec)), self.ctx, "generate_network")
        return self.nnz

    @property
    def nnz(self) -> int:
        v = C.c_int64()
        _check(lib().nn_sim_network_size(self.handle, C.byref(v)), self.ctx)
        return v.value

    def get_network(self):
        nnz = self.nnz
        rp = np.empty(self.n + 1, np.int64)
        col = np.empty(nnz, np.int32)
        w = np.empty(nnz, np.float32)
        d = np.empty(nnz, np.uint8)
        inh = np.empty(self.n, np.uint8)
        _check(lib().nn_sim_get_network(self.handle, _ptr(rp), _ptr(col), _ptr(w), _ptr(d), _ptr(inh)), self.ctx)
        return rp, col, w, d, inh

    def get_csc(self):
        nnz = self.nnz
        cp = np.empty(self.n + 1, np.int64)
        src = np.empty(nnz, np.int32)
        w = np.empty(nnz, np.float32)
        d = np.empty(nnz, np.uint8)
        _check(lib().nn_sim_get_csc(self.handle, _ptr(cp), _ptr(src), _ptr(w), _ptr(d)), self.ctx, "get_csc")
        return cp, src, w, d

    def init_state(self, v0: float = -65.0, i_lo: float = 5.0, i_hi: float = 15.0) -> None:
        _check(lib().nn_sim_init_state(self.handle, v0, i_lo, i_hi), self.ctx, "init_state")

    def set_field(self, name: str, values) -> None:
        v = np.ascontiguousarray(np.broadcast_to(np.asarray(values, np.float32), (self.n,)))
        _check(lib().nn_sim_set_field(self.handle, FIELDS[name], _ptr(v)), self.ctx, "set_field")

    def get_field(self, name: str) -> np.ndarray:
        out = np.empty(self.n, np.float32)
        _check(lib().nn_sim_get_field(self.handle, FIELDS[name], _ptr(out)), self.ctx, "get_field")
        return out

    def step(self, nsteps: int = 1) -> None:
        _check(lib().nn_sim_step(self.handle, nsteps), self.ctx, "step")

    def set_instances(self, offsets, grid_sides=None) -> None:
        """A batch of independent networks (see nn_sim_set_instances)."""
        off = np.ascontiguousarray(offsets, np.int32)
        gs = None if grid_sides is None else np.ascontiguousarray(grid_sides, np.int32)
        _check(lib().nn_sim_set_instances(self.handle, len(off) - 1, _ptr(off), None if gs is None else _ptr(gs)),
               self.ctx, "sim_set_instances")
        self.n_inst = len(off) - 1
        self._inst = (off, gs)

    def generate_batch_er(self, p_per_instance, w_max=0.5, inh_fraction: float = 0.2) -> int:
        """Block-diagonal Erdos-Renyi network, one p (and optionally one
        w_max) per instance."""
        spec = default_net_spec(NN_NET_ER)
        self._inst_p = np.ascontiguousarray(p_per_instance, np.float64)
        spec.inst_p = self._inst_p.ctypes.data
        if np.ndim(w_max):
            self._inst_w = np.ascontiguousarray(w_max, np.float32)
            spec.inst_w_max = self._inst_w.ctypes.data
            w_max = 0.0
        spec.w_max, spec.inh_fraction = w_max, inh_fraction
        return self.generate_network(spec)

    def autotune(self, trial_steps: int = 20) -> tuple[int, int, float]:
        """(threads per block, neurons per thread, ms per step) chosen for the neuron update."""
        tpb, npt, ms = C.c_int(), C.c_int(), C.c_float()
        _check(lib().nn_sim_autotune(self.handle, trial_steps, C.byref(tpb), C.byref(npt), C.byref(ms)), self.ctx,
               "sim_autotune")
        return tpb.value, npt.value, ms.value

    def autotune_solver(self, trial_iters: int = 20) -> tuple[int, float]:
        """Field solver block shape (single grid: tile depth of the one-kernel
        PCG iteration; batch: cells per block), timed on scratch vectors.
        Returns (shape, ms per iteration)."""
        shape, ms = C.c_int(0), C.c_float(0.0)
        _check(lib().nn_sim_autotune_solver(self.handle, trial_iters, C.byref(shape), C.byref(ms)), self.ctx,
               "sim_autotune_solver")
        return shape.value, ms.value

    def instance_iterations(self) -> np.ndarray:
        out = np.empty(self.n_inst, np.int32)
        _check(lib().nn_sim_instance_iterations(self.handle, _ptr(out)), self.ctx, "sim_instance_iterations")
        return out

    def deliver_spikes(self, d_list: "DeviceArray", count: int, mode: int = NN_DELIVERY_PUSH) -> None:
        _check(lib().nn_sim_deliver_spikes(self.handle, d_list.ptr, count, mode), self.ctx, "sim_deliver_spikes")

    def pull_gather(self) -> None:
        """The pull gather kernel alone, from the current spike bitmap."""
        _check(lib().nn_sim_pull_gather(self.handle), self.ctx, "sim_pull_gather")

    def pull_info(self) -> tuple[bool, int]:
        """(shared-memory sliced pull kernel in use, columns per block)."""
        a, b = C.c_int(0), C.c_int(0)
        _check(lib().nn_sim_pull_info(self.handle, C.byref(a), C.byref(b)), self.ctx, "sim_pull_info")
        return bool(a.value), b.value

    def set_pull_rate(self, rate: float) -> None:
        """Automatic delivery: pull threshold (spikes per neuron and step) for
        the periods enqueued from now on."""
        _check(lib().nn_sim_set_pull_rate(self.handle, rate), self.ctx, "sim_set_pull_rate")

    def delivery_log(self, reset: bool = False) -> tuple[np.ndarray, np.ndarray]:
        """Automatic delivery: (mode of each period since the last reset, 0 push
        1 pull; the measured spikes per neuron and step that chose it)."""
        cnt = C.c_int(0)
        _check(lib().nn_sim_delivery_log(self.handle, None, None, 0, C.byref(cnt), 0), self.ctx, "sim_delivery_log")
        modes = np.zeros(max(cnt.value, 1), np.int8)
        rates = np.zeros(max(cnt.value, 1), np.float32)
        _check(lib().nn_sim_delivery_log(self.handle, _ptr(modes), _ptr(rates), cnt.value, C.byref(cnt),
                                         1 if reset else 0), self.ctx, "sim_delivery_log")
        return modes[:cnt.value], rates[:cnt.value]

    def run_host(self, state_in: np.ndarray, nsteps: int, state_out: np.ndarray) -> int:
        sp = C.c_int64()
        _check(lib().nn_sim_run_host(self.handle, _ptr(state_in), nsteps, _ptr(state_out), C.byref(sp)), self.ctx,
               "run_host")
        return sp.value

    def set_electrodes(self, regions_inds, regions_offsets, every: int = 1, capacity: int = 1024) -> None:
        """ElectrodeNet fused into the step (nn_sim_set_electrodes): regions
        as index lists (CSR), sampled every `every` steps into a ring of
        `capacity` samples; every = 0 turns it off."""
        ind = np.ascontiguousarray(regions_inds, np.int32)
        off = np.ascontiguousarray(regions_offsets, np.int32)
        self._el_regions = len(off) - 1
        self._el_cap = capacity
        _check(lib().nn_sim_set_electrodes(self.handle, _ptr(ind), _ptr(off), self._el_regions, every, capacity),
               self.ctx, "set_electrodes")

    def read_electrodes(self):
        """(first step, mean potentials [samples, regions], firing counts
        [samples, regions]) of the recorded samples, oldest first."""
        R = getattr(self, "_el_regions", 0)
        cap = max(getattr(self, "_el_cap", 1), 1)
        avg = np.zeros((cap, max(R, 1)), np.float32)
        fire = np.zeros((cap, max(R, 1)), np.int32)
        first, k = C.c_int64(0), C.c_int(0)
        _check(lib().nn_sim_read_electrodes(self.handle, _ptr(avg), _ptr(fire), C.byref(first), C.byref(k)),
               self.ctx, "read_electrodes")
        return int(first.value), avg[:k.value, :R], fire[:k.value, :R]

    def get_ring(self) -> np.ndarray:
        """Delay ring as (D, n, 2) float32: slot t mod D holds the (E, I)
        input of step t."""
        D = int(self.config.max_delay) + 1
        out = np.zeros((D, self.config.n, 2), np.float32)
        _check(lib().nn_sim_get_ring(self.handle, _ptr(out)), self.ctx, "get_ring")
        return out

    def reset_raster(self) -> None:
        _check(lib().nn_sim_reset_raster(self.handle), self.ctx, "reset_raster")

    def counters(self) -> tuple[int, int]:
        s, t = C.c_int64(), C.c_int64()
        _check(lib().nn_sim_counters(self.handle, C.byref(s), C.byref(t)), self.ctx, "counters")
        return s.value, t.value

    def raster(self, cap: int | None = None) -> tuple[np.ndarray, np.ndarray]:
        cap = int(self.config.raster_capacity if cap is None else cap)
        st = np.empty(max(cap, 1), np.int32)
        ne = np.empty(max(cap, 1), np.int32)
        cnt = C.c_int64()
        _check(lib().nn_sim_get_raster(self.handle, cap, _ptr(st), _ptr(ne), C.byref(cnt)), self.ctx, "raster")
        m = min(cap, cnt.value)
        return st[:m].copy(), ne[:m].copy()

    def field_cells(self) -> int:
        c = C.c_int64()
        _check(lib().nn_sim_field_cells(self.handle, C.byref(c)), self.ctx, "field_cells")
        return int(c.value)

    def density(self) -> np.ndarray:
        out = np.empty(self.field_cells(), np.float32)
        _check(lib().nn_sim_get_density(self.handle, _ptr(out)), self.ctx, "density")
        return out

    get_density = density

    def get_vox(self) -> np.ndarray:
        out = np.empty(self.n, np.int32)
        _check(lib().nn_sim_get_vox(self.handle, _ptr(out)), self.ctx, "get_vox")
        return out

    def set_density(self, u: np.ndarray) -> None:
        u = np.ascontiguousarray(u, np.float32).ravel()
        _check(lib().nn_sim_set_density(self.handle, _ptr(u)), self.ctx, "set_density")

    def set_kernel_timing(self, on: bool = True) -> None:
        _check(lib().nn_sim_set_kernel_timing(self.handle, int(on)), self.ctx, "set_kernel_timing")

    def kernel_times(self) -> KernelTimes:
        k = KernelTimes()
        _check(lib().nn_sim_kernel_times(self.handle, C.byref(k)), self.ctx, "kernel_times")
        return k

    def solve_stats(self) -> SolveStats:
        s = SolveStats()
        _check(lib().nn_sim_solve_stats(self.handle, C.byref(s)), self.ctx)
        return s


class BatchedPCG:
    """Jacobi-PCG over many independent cubic grids, each to its own rtol."""

    def __init__(self, ctx: Context, sides, alpha_unit: float, beta: float):
        self.ctx = ctx
        self.sides = np.ascontiguousarray(sides, np.int32)
        self.offsets = np.concatenate([[0], np.cumsum(self.sides.astype(np.int64) ** 3)])
        self.handle = C.c_void_p()
        _check(lib().nn_bpcg_create(ctx.handle, len(self.sides), _ptr(self.sides), alpha_unit, beta,
                                    C.byref(self.handle)), ctx, "nn_bpcg_create")

    def solve(self, b: DeviceArray, x: DeviceArray, rtol: float = 1e-6, max_iter: int = 10000):
        its = np.empty(len(self.sides), np.int32)
        mx, bad = C.c_int(), C.c_int()
        _check(lib().nn_bpcg_solve(self.handle, b.ptr, x.ptr, rtol, max_iter, _ptr(its), C.byref(mx), C.byref(bad)),
               self.ctx, "bpcg_solve")
        return its, bad.value

    def autotune(self, b: DeviceArray, x: DeviceArray, trial_iters: int = 20) -> tuple[int, float]:
        """Time 512 .. 4,096 cells per block on right-hand side b (x: scratch,
        overwritten); keeps the fastest.  Returns (cells per block, ms per iteration)."""
        cpb, ms = C.c_int(0), C.c_float(0.0)
        _check(lib().nn_bpcg_autotune(self.handle, b.ptr, x.ptr, trial_iters, C.byref(cpb), C.byref(ms)), self.ctx,
               "bpcg_autotune")
        return cpb.value, ms.value

    def set_cells_per_block(self, cells: int) -> None:
        _check(lib().nn_bpcg_set_cells_per_block(self.handle, cells), self.ctx, "bpcg_set_cells_per_block")

    def close(self):
        if self.handle:
            lib().nn_bpcg_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PCG:
    """Standalone 7-point Jacobi-PCG (nn_pcg_*)."""

    def __init__(self, ctx: Context, nx: int, ny: int, nz: int, alpha: float, beta: float,
                 Dcell: DeviceArray | None = None):
        self.ctx, self.shape = ctx, (nz, ny, nx)
        self.handle = C.c_void_p()
        _check(lib().nn_pcg_create(ctx.handle, nx, ny, nz, alpha, beta, None if Dcell is None else Dcell.ptr,
                                   C.byref(self.handle)), ctx, "nn_pcg_create")
        self._D = Dcell

    def apply(self, x: DeviceArray, y: DeviceArray) -> None:
        _check(lib().nn_pcg_apply(self.handle, x.ptr, y.ptr), self.ctx, "pcg_apply")

    def solve(self, b: DeviceArray, x: DeviceArray, rtol: float = 1e-6, max_iter: int = 10000) -> tuple[int, float]:
        it, rel = C.c_int(0), C.c_double(0)
        _check(lib().nn_pcg_solve(self.handle, b.ptr, x.ptr, rtol, max_iter, C.byref(it), C.byref(rel)), self.ctx,
               "pcg_solve")
        return it.value, rel.value

    def set_kernel_timing(self, on: bool = True) -> None:
        _check(lib().nn_pcg_set_kernel_timing(self.handle, int(on)), self.ctx, "pcg_set_kernel_timing")

    def kernel_time(self) -> tuple[float, int]:
        """(ms of the iteration kernels, iterations) of the last solve."""
        ms, it = C.c_float(0), C.c_int(0)
        _check(lib().nn_pcg_kernel_time(self.handle, C.byref(ms), C.byref(it)), self.ctx, "pcg_kernel_time")
        return ms.value, it.value

    def close(self):
        if self.handle:
            lib().nn_pcg_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MultigridPCG:
    """Flexible CG preconditioned by a geometric multigrid V-cycle on the
    7-point operator of a PCG object (nn_mg_*).  The PCG object (and its
    cell field) must stay alive while this one is used."""

    def __init__(self, pcg: PCG, levels: int = 0):
        self.ctx, self.pcg = pcg.ctx, pcg
        self.handle = C.c_void_p()
        _check(lib().nn_mg_create(pcg.handle, levels, C.byref(self.handle)), self.ctx, "nn_mg_create")

    @property
    def levels(self) -> int:
        n = C.c_int(0)
        _check(lib().nn_mg_levels(self.handle, C.byref(n)), self.ctx, "nn_mg_levels")
        return n.value

    def apply(self, r: DeviceArray, z: DeviceArray) -> None:
        """z = M r (one V-cycle)."""
        _check(lib().nn_mg_apply(self.handle, r.ptr, z.ptr), self.ctx, "nn_mg_apply")

    def solve(self, b: DeviceArray, x: DeviceArray, rtol: float = 1e-6, max_iter: int = 1000) -> tuple[int, float]:
        it, rel = C.c_int(0), C.c_double(0)
        _check(lib().nn_mg_solve(self.handle, b.ptr, x.ptr, rtol, max_iter, C.byref(it), C.byref(rel)), self.ctx,
               "nn_mg_solve")
        return it.value, rel.value

    def close(self):
        if self.handle:
            lib().nn_mg_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LearnedMultigrid:
    """Multigrid FCG whose coarse level `level` (and everything below it) is
    solved by the learned 3D conv U-Net (nn_lmg_*).  Train with
    add_solves(rhs) + train(); use_network(False) gives the classical
    hierarchy on the same object.  The PCG object must stay alive."""

    def __init__(self, pcg: PCG, level: int = 3, seed: int = 7):
        self.ctx, self.pcg = pcg.ctx, pcg
        self.handle = C.c_void_p()
        _check(lib().nn_lmg_create(pcg.handle, level, seed, C.byref(self.handle)), self.ctx, "nn_lmg_create")

    def add_solves(self, rhs_list) -> int:
        """Solve each right-hand side (host arrays) with the classical hierarchy
        and keep the level's right-hand sides and solutions as training pairs;
        returns the number of pairs added."""
        total = 0
        for b in rhs_list:
            hb = np.ascontiguousarray(b, np.float32).ravel()
            db = self.ctx.to_device(hb)
            dx = self.ctx.empty((hb.size,), np.float32)
            k = C.c_int(0)
            _check(lib().nn_lmg_add_solve(self.handle, db.ptr, dx.ptr, C.byref(k)), self.ctx, "nn_lmg_add_solve")
            total += k.value
        return total

    @property
    def pairs(self) -> int:
        n = C.c_int(0)
        _check(lib().nn_lmg_pairs(self.handle, C.byref(n)), self.ctx, "nn_lmg_pairs")
        return n.value

    def train(self, steps: int, lr: float = 1e-3) -> float:
        loss = C.c_float(0)
        _check(lib().nn_lmg_train(self.handle, steps, lr, C.byref(loss)), self.ctx, "nn_lmg_train")
        return loss.value

    def use_network(self, on: bool = True) -> None:
        _check(lib().nn_lmg_use_network(self.handle, int(on)), self.ctx, "nn_lmg_use_network")

    def set_post_sweeps(self, sweeps: int) -> None:
        """Jacobi sweeps on the network's level after its correction (default 2)."""
        _check(lib().nn_lmg_set_post_sweeps(self.handle, sweeps), self.ctx, "nn_lmg_set_post_sweeps")

    def autotune_post_sweeps(self, rhs, rtol: float = 1e-6) -> tuple[int, float]:
        """Pick the post-network sweeps (2 .. 24) by timing solves of the device
        right-hand sides `rhs` (a list); returns (sweeps, total ms of its solves)."""
        x = self.ctx.empty((int(np.prod(rhs[0].shape)),), np.float32)
        ptrs = (C.c_void_p * len(rhs))(*[r.ptr for r in rhs])
        best, ms = C.c_int(0), C.c_float(0)
        _check(lib().nn_lmg_autotune_post_sweeps(self.handle, ptrs, len(rhs), x.ptr, rtol, C.byref(best),
                                                 C.byref(ms)), self.ctx, "nn_lmg_autotune_post_sweeps")
        return best.value, ms.value

    def solve(self, b: DeviceArray, x: DeviceArray, rtol: float = 1e-6, max_iter: int = 1000) -> tuple[int, float]:
        it, rel = C.c_int(0), C.c_double(0)
        _check(lib().nn_lmg_solve(self.handle, b.ptr, x.ptr, rtol, max_iter, C.byref(it), C.byref(rel)), self.ctx,
               "nn_lmg_solve")
        return it.value, rel.value

    def close(self):
        if self.handle:
            lib().nn_lmg_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------- learned preconditioner layers --

def act_bytes(shape, channels: int) -> int:
    """Bytes of a padded BF16 activation with `channels` channels on shape (nz, ny, nx)."""
    nz, ny, nx = shape
    b = C.c_int64()
    _check(lib().nn_act_layout(nz, ny, nx, channels, None, None, C.byref(b)), None, "nn_act_layout")
    return int(b.value)


class Activation(DeviceArray):
    """Padded channel-blocked BF16 activation (zeros in pads and guards)."""

    def __init__(self, ctx: Context, shape, channels: int):
        super().__init__(ctx, (act_bytes(shape, channels),), np.uint8)
        self.grid, self.channels = tuple(shape), channels
        self.zero()

    def pack(self, dense: DeviceArray) -> None:
        nz, ny, nx = self.grid
        _check(lib().nn_act_pack(self.ctx.handle, nz, ny, nx, self.channels, dense.ptr, self.ptr), self.ctx, "act_pack")

    def unpack(self) -> np.ndarray:
        nz, ny, nx = self.grid
        d = DeviceArray(self.ctx, (self.channels, nz, ny, nx), np.float32)
        _check(lib().nn_act_unpack(self.ctx.handle, nz, ny, nx, self.channels, self.ptr, d.ptr), self.ctx, "act_unpack")
        return d.numpy()


def conv3d_pack_weights(ctx: Context, w: DeviceArray, cin: int, cout: int, adjoint: bool = False) -> DeviceArray:
    out = DeviceArray(ctx, (27 * cin * cout * 2,), np.uint8)
    _check(lib().nn_conv3d_pack_weights(ctx.handle, cin, cout, w.ptr, int(adjoint), out.ptr), ctx, "conv3d_pack")
    return out


def conv3d_forward(ctx: Context, x: Activation, wpacked: DeviceArray, y: Activation, bias: DeviceArray | None = None,
                   relu: bool = False, mask: Activation | None = None, y32: DeviceArray | None = None) -> None:
    nz, ny, nx = x.grid
    _check(lib().nn_conv3d_forward(ctx.handle, nz, ny, nx, x.channels, y.channels, x.ptr, wpacked.ptr,
                                   None if bias is None else bias.ptr, int(relu), None if mask is None else mask.ptr,
                                   y.ptr, None if y32 is None else y32.ptr), ctx, "conv3d_forward")


def conv3d_wgrad(ctx: Context, x: Activation, gy: Activation, dw: DeviceArray, db: DeviceArray | None = None) -> None:
    nz, ny, nx = x.grid
    _check(lib().nn_conv3d_wgrad(ctx.handle, nz, ny, nx, x.channels, gy.channels, x.ptr, gy.ptr, dw.ptr,
                                 None if db is None else db.ptr), ctx, "conv3d_wgrad")


class LearnedPreconditioner:
    """Two-grid preconditioner with a U-Net coarse correction for a PCG's
    operator (nn_learned_*), and the flexible CG that uses it."""

    def __init__(self, pcg: PCG, seed: int = 0):
        self.pcg, self.ctx = pcg, pcg.ctx
        self.handle = C.c_void_p()
        _check(lib().nn_learned_create(pcg.handle, seed, C.byref(self.handle)), self.ctx, "nn_learned_create")

    def add_pair(self, r: DeviceArray, e: DeviceArray) -> None:
        _check(lib().nn_learned_add_pair(self.handle, r.ptr, e.ptr), self.ctx, "learned_add_pair")

    def add_solver_pairs(self, rhs, snapshots=(0, 1, 2, 4, 8, 16, 32, 64), rtol: float = 1e-7) -> int:
        """Training pairs from the plain solver's own iterates: for each
        right-hand side b (host arrays), solve to rtol for x*, then for every
        snapshot k restart from zero for k iterations and add
        (b - A x_k, x* - x_k).  Returns the number of pairs added."""
        pc, ctx = self.pcg, self.ctx
        G = int(np.prod(pc.shape))
        t = ctx.empty((G,), np.float32)
        added = 0
        for b in rhs:
            b = np.ascontiguousarray(b, np.float32).ravel()
            db = ctx.to_device(b)
            xs = ctx.to_device(np.zeros(G, np.float32))
            pc.solve(db, xs, rtol, 100000)
            xstar = xs.numpy()
            for k in snapshots:
                xk = ctx.to_device(np.zeros(G, np.float32))
                if k:
                    try:
                        pc.solve(db, xk, 1e-30, k)
                    except NNError as e:
                        if e.status != NN_ERR_NOT_CONVERGED:
                            raise
                pc.apply(xk, t)
                self.add_pair(ctx.to_device(b - t.numpy()), ctx.to_device(xstar - xk.numpy()))
                added += 1
        return added

    def train(self, steps: int, lr: float = 1e-3) -> float:
        loss = C.c_float(0)
        _check(lib().nn_learned_train(self.handle, steps, lr, C.byref(loss)), self.ctx, "learned_train")
        return loss.value

    def apply(self, r: DeviceArray, z: DeviceArray) -> None:
        _check(lib().nn_learned_apply(self.handle, r.ptr, z.ptr), self.ctx, "learned_apply")

    def use_network(self, on: bool) -> None:
        _check(lib().nn_learned_use_network(self.handle, int(on)), self.ctx, "learned_use_network")

    def solve(self, b: DeviceArray, x: DeviceArray, rtol: float = 1e-6, max_iter: int = 10000) -> tuple[int, float]:
        it, rel = C.c_int(0), C.c_double(0)
        _check(lib().nn_learned_solve(self.handle, b.ptr, x.ptr, rtol, max_iter, C.byref(it), C.byref(rel)),
               self.ctx, "learned_solve")
        return it.value, rel.value

    def num_params(self) -> int:
        n = C.c_int64()
        _check(lib().nn_learned_num_params(self.handle, C.byref(n)), self.ctx, "learned_num_params")
        return int(n.value)

    def get_params(self) -> np.ndarray:
        out = np.empty(self.num_params(), np.float32)
        _check(lib().nn_learned_get_params(self.handle, _ptr(out)), self.ctx, "learned_get_params")
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.num_params()
        _check(lib().nn_learned_set_params(self.handle, _ptr(p)), self.ctx, "learned_set_params")

    def net_gradient(self, rc: DeviceArray, target: DeviceArray):
        """(loss, flat parameter gradient, network output) on a coarse-grid input."""
        g = np.empty(self.num_params(), np.float32)
        loss = C.c_double(0)
        y = DeviceArray(self.ctx, rc.shape, np.float32)
        _check(lib().nn_learned_net_gradient(self.handle, rc.ptr, target.ptr, _ptr(g), C.byref(loss), y.ptr),
               self.ctx, "learned_net_gradient")
        return loss.value, g, y.numpy()

    def close(self):
        if self.handle:
            lib().nn_learned_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------- consumers of the step --

class ElectrodeNet:
    """Mirror of the reference's ElectrodeNet: regions as index lists."""

    def __init__(self, ctx: Context, regions_inds, regions_offsets):
        self.ctx = ctx
        idx = np.ascontiguousarray(regions_inds, np.int32)
        off = np.ascontiguousarray(regions_offsets, np.int32)
        self.n_regions = len(off) - 1
        self.handle = C.c_void_p()
        _check(lib().nn_electrodes_create(ctx.handle, _ptr(idx), _ptr(off), self.n_regions, C.byref(self.handle)),
               ctx, "nn_electrodes_create")

    def do_electrode_measurements(self, V: DeviceArray, is_firing: DeviceArray | None = None):
        avg = np.empty(self.n_regions, np.float32)
        fir = np.empty(self.n_regions, np.int32)
        _check(lib().nn_electrodes_measure(self.handle, V.ptr, None if is_firing is None else is_firing.ptr,
                                           _ptr(avg), _ptr(fir)), self.ctx, "electrodes_measure")
        return avg, (fir if is_firing is not None else None)

    @staticmethod
    def measure_average_entire_network(ctx: Context, V: DeviceArray, n: int) -> float:
        out = C.c_float()
        _check(lib().nn_measure_average(ctx.handle, V.ptr, n, C.byref(out)), ctx, "measure_average")
        return out.value

    def close(self):
        if self.handle:
            lib().nn_electrodes_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SynchronyNet:
    def __init__(self, ctx: Context, region_inds, sub_sample_counts):
        self.ctx = ctx
        idx = np.ascontiguousarray(region_inds, np.int32)
        sub = np.ascontiguousarray(sub_sample_counts, np.int32)
        self.n_sub = len(sub)
        self.handle = C.c_void_p()
        _check(lib().nn_synchrony_create(ctx.handle, _ptr(idx), len(idx), _ptr(sub), len(sub), C.byref(self.handle)),
               ctx, "nn_synchrony_create")

    def measure_variances(self, V: DeviceArray) -> None:
        _check(lib().nn_synchrony_measure(self.handle, V.ptr), self.ctx, "synchrony_measure")

    def get_synchrony_measures(self) -> np.ndarray:
        out = np.empty(self.n_sub, np.float64)
        _check(lib().nn_synchrony_get(self.handle, _ptr(out)), self.ctx, "synchrony_get")
        return out

    def close(self):
        if self.handle:
            lib().nn_synchrony_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Hebbian:
    """Mirror of the reference's Hebbian learner (timer window, increment)."""

    def __init__(self, ctx: Context, window_duration: int, heb_inc: float, nconns: int, n_neurons: int):
        self.ctx, self.nconns = ctx, nconns
        self.handle = C.c_void_p()
        _check(lib().nn_hebbian_create(ctx.handle, window_duration, heb_inc, nconns, n_neurons, C.byref(self.handle)),
               ctx, "nn_hebbian_create")

    def update_weights(self, indices: DeviceArray, offsets: DeviceArray, weights: DeviceArray, is_firing: DeviceArray,
                       firing_inds: DeviceArray | None, num_firing: int) -> None:
        _check(lib().nn_hebbian_update(self.handle, indices.ptr, offsets.ptr, is_firing.ptr,
                                       None if firing_inds is None else firing_inds.ptr, num_firing, weights.ptr),
               self.ctx, "hebbian_update")

    def timers(self) -> np.ndarray:
        out = np.empty(self.nconns, np.int32)
        _check(lib().nn_hebbian_timers(self.handle, _ptr(out)), self.ctx, "hebbian_timers")
        return out

    def close(self):
        if self.handle:
            lib().nn_hebbian_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --------------------------------------------------------- on-disk inputs --

def write_network_file(path: str, row_ptr, col) -> None:
    rp = np.ascontiguousarray(row_ptr, np.int32)
    c = np.ascontiguousarray(col, np.int32)
    _check(lib().nn_net_file_write(str(path).encode(), len(rp) - 1, len(c), _ptr(rp), _ptr(c)), None,
           "nn_net_file_write")


def read_network_file(path: str) -> tuple[np.ndarray, np.ndarray]:
    nr, nz = C.c_int64(), C.c_int64()
    _check(lib().nn_net_file_read(str(path).encode(), C.byref(nr), C.byref(nz), None, None), None, "nn_net_file_read")
    rp = np.empty(nr.value + 1, np.int32)
    col = np.empty(nz.value, np.int32)
    _check(lib().nn_net_file_read(str(path).encode(), C.byref(nr), C.byref(nz), _ptr(rp), _ptr(col)), None,
           "nn_net_file_read")
    return rp, col


class FileNetwork:
    """Mirror of the reference's FileNetwork: connectivity from a file,
    sub-sampled to N neurons on the device."""

    def __init__(self, path: str):
        self.path = str(path)
        self.row_ptr = self.col = None

    def generate(self, ctx: Context, N: int) -> bool:
        try:
            rp, col = read_network_file(self.path)
        except NNError:
            return False
        if N > len(rp) - 1:
            return False
        drp, dcol = ctx.to_device(rp), ctx.to_device(col)
        orp = DeviceArray(ctx, (N + 1,), np.int64)
        ocol = DeviceArray(ctx, (max(len(col), 1),), np.int32)
        nnz = C.c_int64()
        _check(lib().nn_net_subsample(ctx.handle, drp.ptr, dcol.ptr, len(rp) - 1, N, orp.ptr, ocol.ptr, C.byref(nnz)),
               ctx, "nn_net_subsample")
        self.row_ptr = orp.numpy()
        self.col = ocol.numpy()[:nnz.value]
        return True


def write_positions_file(path: str, x, y, z) -> None:
    a = [np.ascontiguousarray(v, np.float32) for v in (x, y, z)]
    _check(lib().nn_positions_file_write(str(path).encode(), len(a[0]), _ptr(a[0]), _ptr(a[1]), _ptr(a[2])), None,
           "nn_positions_file_write")


class FileMorphology:
    """Mirror of the reference's FileMorphology: N positions in [-1, 1]."""

    def __init__(self, path: str):
        self.path = str(path)
        self.positions = None

    def generate(self, ctx: Context, N: int) -> bool:
        n = C.c_int64()
        if lib().nn_positions_file_read(self.path.encode(), C.byref(n), None, None, None) != 0:
            return False
        if N > n.value:
            return False
        xyz = [np.empty(n.value, np.float32) for _ in range(3)]
        _check(lib().nn_positions_file_read(self.path.encode(), C.byref(n), *[_ptr(v) for v in xyz]), None,
               "nn_positions_file_read")
        d = [ctx.to_device(v) for v in xyz]
        o = [DeviceArray(ctx, (N,), np.float32) for _ in range(3)]
        _check(lib().nn_positions_subsample(ctx.handle, d[0].ptr, d[1].ptr, d[2].ptr, n.value, N, o[0].ptr, o[1].ptr,
                                            o[2].ptr), ctx, "nn_positions_subsample")
        self.positions = np.stack([v.numpy() for v in o], axis=1)
        return True


# ------------------------------------------------------- whole-brain step --

class NormalNetwork:
    """NormalNetwork (src_wholebrain/network_factory.cuh:73-91): local
    Gaussian-ball connectivity over device positions, built on the device."""

    def __init__(self, x: DeviceArray, y: DeviceArray, z: DeviceArray, stddev: float, n_stddevs: int = 2,
                 seed: int = 0):
        self.x, self.y, self.z = x, y, z
        self.stddev, self.n_stddevs, self.seed = stddev, n_stddevs, seed

    def to_adjacency_list(self, ctx: Context, tcount: DeviceArray | None = None) -> AdjacencyList:
        n = self.x.shape[0]
        off = DeviceArray(ctx, (n + 1,), np.int32)
        nnz = C.c_int64()
        args = (ctx.handle, n, self.x.ptr, self.y.ptr, self.z.ptr, self.stddev, self.n_stddevs, self.seed, off.ptr)
        _check(lib().nn_net_local_gaussian(*args, None, 0, C.byref(nnz)), ctx, "NormalNetwork count")
        idx = DeviceArray(ctx, (max(nnz.value, 1),), np.int32)
        _check(lib().nn_net_local_gaussian(*args, idx.ptr, nnz.value, C.byref(nnz)), ctx, "NormalNetwork fill")
        if tcount is not None:
            _check(lib().nn_net_tcount(ctx.handle, idx.ptr, nnz.value, n, tcount.ptr), ctx, "Tcount")
        self.nnz = nnz.value
        return AdjacencyList(idx, off)


class MouseCortex:
    """MouseCortex (src_wholebrain/mouse_cortex.cu:8-120): the whole-brain
    HH model with white-matter AMPA / GABA couplings (uniform random, 0.9 and
    0.1 of ncouple out-edges) and optional gray-matter local GABA coupling
    (Gaussian ball of stddev over the positions).  simulate() is
    MouseCortex::Simulate: the couplings in the reference's order (gray GABA,
    white GABA, white AMPA), then one leapfrog step."""

    def __init__(self, ctx: Context, n: int, positions=None, ncouple: int = 1000, use_gray: bool = True,
                 stddev: float = 0.045, seed: int = 0):
        self.ctx, self.n = ctx, n
        self.ephys = HHEphys(ctx, n, variant=1, seed=seed)
        v = self.ephys.vars
        ix = {name: v[SIM_PARAMS.index(name)] for name in SIM_PARAMS}
        e_net, i_net = UniformRandomNetwork(int(0.9 * ncouple)), UniformRandomNetwork(int(0.1 * ncouple))
        e_net.generate(n)
        i_net.generate(n)
        self.e_list = e_net.to_adjacency_list(ctx, ix["ECOUNT"])
        self.i_list = i_net.to_adjacency_list(ctx, ix["ICOUNT"])
        self.white_ampa = AtomicCoupling(ctx, n)
        self.white_gaba = AtomicCoupling(ctx, n)
        self.gray_gaba = None
        if use_gray:
            if positions is None:
                positions = np.random.default_rng(seed).uniform(-1.0, 1.0, (n, 3)).astype(np.float32)
            self.pos = [ctx.to_device(np.ascontiguousarray(positions[:, a], np.float32)) for a in range(3)]
            self.loc_net = NormalNetwork(*self.pos, stddev=stddev, seed=seed)
            self.loc_list = self.loc_net.to_adjacency_list(ctx, ix["LOCAL_COUNT"])
            self.gray_gaba = AtomicCoupling(ctx, n)
        self._ix = ix

    def simulate(self) -> int:
        ix = self._ix
        n_firing = 0
        if self.gray_gaba is not None:
            n_firing = self.gray_gaba(self.loc_list, ix["LOCAL_IN"], ix["LOCAL_OUTPUT"])
        n_firing = self.white_gaba(self.i_list, ix["IIN"], ix["IOUTPUT"])
        n_firing = self.white_ampa(self.e_list, ix["EIN"], ix["EOUTPUT"])
        self.ephys.simulate_ephys()
        return n_firing
