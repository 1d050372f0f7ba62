"""ctypes binding of libneuronephys (include/neuronephys.h).

Loading fails loudly when the CUDA library has not been built: there is no
CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from .build import lib_path

c_int, c_int64, c_uint32, c_uint64 = C.c_int, C.c_int64, C.c_uint32, C.c_uint64
c_float, c_double, c_size_t = C.c_float, C.c_double, C.c_size_t
c_void_p, c_char_p = C.c_void_p, C.c_char_p
P = C.POINTER


class LeapfrogParams(C.Structure):
    _fields_ = [(n, c_float) for n in (
        "gna", "ena", "gk", "ek", "gl", "el", "Tmax", "Vt", "Kp", "Ar", "Ad",
        "g_local", "e_local", "g_gaba", "e_gaba", "g_exc", "e_exc",
        "noise_mean", "noise_intensity")]


class ParacrineRefParams(C.Structure):
    _fields_ = [("nx", c_int), ("ny", c_int), ("nz", c_int), ("h", c_float), ("D", c_float),
                ("decay", c_float), ("par_dt", c_float), ("coup_strength", c_float),
                ("max_iter", c_int), ("abs_tol", c_float), ("quirk_rhs", c_int),
                ("quirk_firing_list", c_int)]


class HHParams(C.Structure):
    _fields_ = [(n, c_float) for n in (
        "C", "gNa", "gK", "gL", "ENa", "EK", "EL", "E_exc", "E_inh", "tau_exc", "tau_inh",
        "v_thresh", "noise_sigma", "dt", "g_par", "E_par")]


class SimConfig(C.Structure):
    _fields_ = [("n", c_int), ("max_delay", c_int), ("seed", c_uint64), ("hp", HHParams),
                ("delivery", c_int), ("raster_capacity", c_int64), ("grid", c_int),
                ("timescale", c_int), ("par_D", c_float), ("par_decay", c_float),
                ("par_rtol", c_double), ("par_max_iter", c_int), ("threads_per_block", c_int),
                ("neurons_per_thread", c_int), ("par_overlap", c_int), ("par_extrapolate", c_int),
                ("pull_rate", c_float)]


class NetSpec(C.Structure):
    _fields_ = [("kind", c_int), ("p", c_double), ("w_max", c_float), ("k", c_int),
                ("sigma", c_double), ("w_mu", c_double), ("w_sigma", c_double), ("dmax", c_int),
                ("inh_fraction", c_double), ("inh_random", c_int), ("n_regions", c_int),
                ("region_size_sigma", c_double), ("density_sigma", c_double),
                ("block_dmax", c_int), ("inst_p", c_void_p), ("inst_w_max", c_void_p)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", c_int), ("relres", c_double), ("solves", c_int),
                ("converged", c_int)]


class KernelTimes(C.Structure):
    _fields_ = [("hh_step_ms", c_float), ("deliver_ms", c_float), ("samples", c_int),
                ("solve_ms", c_float), ("solve_iterations", c_int),
                ("hh_step_median_ms", c_float), ("deliver_median_ms", c_float)]


# name -> (restype, argtypes)
_SIGS = {
    "nn_status_string": (c_char_p, [c_int]),
    "nn_version": (c_int, []),
    "nn_ctx_create": (c_int, [c_int, P(c_void_p)]),
    "nn_ctx_destroy": (c_int, [c_void_p]),
    "nn_ctx_last_error": (c_char_p, [c_void_p]),
    "nn_ctx_synchronize": (c_int, [c_void_p]),
    "nn_ctx_kernel_launches": (c_int64, [c_void_p]),
    "nn_ctx_num_sms": (c_int, [c_void_p]),
    "nn_ctx_stream": (c_void_p, [c_void_p]),
    "nn_ctx_time_begin": (c_int, [c_void_p]),
    "nn_ctx_time_end": (c_int, [c_void_p, P(c_float)]),
    "nn_host_alloc": (c_int, [c_size_t, P(c_void_p)]),
    "nn_host_free": (c_int, [c_void_p]),
    "nn_malloc": (c_int, [c_void_p, c_size_t, P(c_void_p)]),
    "nn_free": (c_int, [c_void_p, c_void_p]),
    "nn_memcpy_h2d": (c_int, [c_void_p, c_void_p, c_void_p, c_size_t]),
    "nn_memcpy_d2h": (c_int, [c_void_p, c_void_p, c_void_p, c_size_t]),
    "nn_memset_d": (c_int, [c_void_p, c_void_p, c_int, c_size_t]),
    "nn_leapfrog_params_reference": (None, [P(LeapfrogParams), c_int]),
    "nn_hh_leapfrog_step": (c_int, [c_void_p, P(c_void_p), c_int, c_float, P(LeapfrogParams),
                                    c_uint64, c_uint64]),
    "nn_hh_leapfrog_step_z": (c_int, [c_void_p, P(c_void_p), c_int, c_float, P(LeapfrogParams), c_void_p]),
    "nn_coupling_create": (c_int, [c_void_p, c_int, P(c_void_p)]),
    "nn_coupling_destroy": (c_int, [c_void_p]),
    "nn_coupling_run": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, P(c_int)]),
    "nn_coupling_run_chunked": (c_int, [c_void_p, c_int, c_int, P(c_void_p), P(c_void_p), c_void_p,
                                        c_void_p, P(c_int)]),
    "nn_coupling_firing_list": (c_void_p, [c_void_p]),
    "nn_coupling_firing_count": (c_void_p, [c_void_p]),
    "nn_net_uniform_random": (c_int, [c_int, c_int, P(c_uint32), c_void_p, c_void_p]),
    "nn_net_tcount": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p]),
    "nn_net_to_chunked": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, P(c_void_p),
                                  P(c_void_p), P(c_int64)]),
    "nn_paracrine_ref_params_default": (None, [P(ParacrineRefParams)]),
    "nn_paracrine_ref_create": (c_int, [c_void_p, P(ParacrineRefParams), c_int, c_void_p, c_void_p,
                                        c_void_p, c_void_p, P(c_void_p)]),
    "nn_paracrine_destroy": (c_int, [c_void_p]),
    "nn_paracrine_ref_fine": (c_int, [c_void_p, c_void_p]),
    "nn_paracrine_ref_own": (c_int, [c_void_p, P(c_int), P(c_float)]),
    "nn_paracrine_density": (c_void_p, [c_void_p]),
    "nn_paracrine_sources": (c_void_p, [c_void_p]),
    "nn_hh_params_standard": (None, [P(HHParams)]),
    "nn_sim_config_default": (None, [P(SimConfig), c_int]),
    "nn_net_spec_default": (None, [P(NetSpec), c_int]),
    "nn_sim_create": (c_int, [c_void_p, P(SimConfig), P(c_void_p)]),
    "nn_sim_destroy": (c_int, [c_void_p]),
    "nn_sim_set_network": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p]),
    "nn_sim_generate_network": (c_int, [c_void_p, P(NetSpec)]),
    "nn_sim_network_size": (c_int, [c_void_p, P(c_int64)]),
    "nn_sim_get_network": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "nn_sim_get_csc": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "nn_sim_set_field": (c_int, [c_void_p, c_int, c_void_p]),
    "nn_sim_get_field": (c_int, [c_void_p, c_int, c_void_p]),
    "nn_sim_field_ptr": (c_void_p, [c_void_p, c_int]),
    "nn_sim_init_state": (c_int, [c_void_p, c_float, c_float, c_float]),
    "nn_sim_step": (c_int, [c_void_p, c_int]),
    "nn_sim_run_host": (c_int, [c_void_p, c_void_p, c_int, c_void_p, P(c_int64)]),
    "nn_sim_set_electrodes": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int]),
    "nn_sim_read_electrodes": (c_int, [c_void_p, c_void_p, c_void_p, P(c_int64), P(c_int)]),
    "nn_sim_get_ring": (c_int, [c_void_p, c_void_p]),
    "nn_sim_reset_raster": (c_int, [c_void_p]),
    "nn_sim_counters": (c_int, [c_void_p, P(c_int64), P(c_int64)]),
    "nn_sim_get_raster": (c_int, [c_void_p, c_int64, c_void_p, c_void_p, P(c_int64)]),
    "nn_sim_get_density": (c_int, [c_void_p, c_void_p]),
    "nn_sim_set_density": (c_int, [c_void_p, c_void_p]),
    "nn_sim_solve_stats": (c_int, [c_void_p, P(SolveStats)]),
    "nn_sim_set_kernel_timing": (c_int, [c_void_p, c_int]),
    "nn_sim_kernel_times": (c_int, [c_void_p, P(KernelTimes)]),
    "nn_pcg_create": (c_int, [c_void_p, c_int, c_int, c_int, c_double, c_double, c_void_p, P(c_void_p)]),
    "nn_pcg_destroy": (c_int, [c_void_p]),
    "nn_pcg_apply": (c_int, [c_void_p, c_void_p, c_void_p]),
    "nn_pcg_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_double, c_int, P(c_int), P(c_double)]),
    "nn_pcg_set_kernel_timing": (c_int, [c_void_p, c_int]),
    "nn_sim_deliver_spikes": (c_int, [c_void_p, c_void_p, c_int, c_int]),
    "nn_sim_pull_info": (c_int, [c_void_p, P(c_int), P(c_int)]),
    "nn_sim_pull_gather": (c_int, [c_void_p]),
    "nn_sim_delivery_log": (c_int, [c_void_p, c_void_p, c_void_p, c_int, P(c_int), c_int]),
    "nn_sim_set_pull_rate": (c_int, [c_void_p, c_float]),
    "nn_sim_autotune_solver": (c_int, [c_void_p, c_int, P(c_int), P(c_float)]),
    "nn_bpcg_autotune": (c_int, [c_void_p, c_void_p, c_void_p, c_int, P(c_int), P(c_float)]),
    "nn_bpcg_set_cells_per_block": (c_int, [c_void_p, c_int]),
    "nn_sim_set_instances": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    "nn_sim_field_cells": (c_int, [c_void_p, P(c_int64)]),
    "nn_sim_get_vox": (c_int, [c_void_p, c_void_p]),
    "nn_sim_autotune": (c_int, [c_void_p, c_int, P(c_int), P(c_int), P(c_float)]),
    "nn_sim_instance_iterations": (c_int, [c_void_p, c_void_p]),
    "nn_bpcg_create": (c_int, [c_void_p, c_int, c_void_p, c_double, c_double, P(c_void_p)]),
    "nn_bpcg_destroy": (c_int, [c_void_p]),
    "nn_bpcg_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_double, c_int, c_void_p, P(c_int), P(c_int)]),
    "nn_net_file_write": (c_int, [C.c_char_p, c_int64, c_int64, c_void_p, c_void_p]),
    "nn_net_file_read": (c_int, [C.c_char_p, P(c_int64), P(c_int64), c_void_p, c_void_p]),
    "nn_net_subsample": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int, c_void_p, c_void_p, P(c_int64)]),
    "nn_positions_file_write": (c_int, [C.c_char_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "nn_positions_file_read": (c_int, [C.c_char_p, P(c_int64), c_void_p, c_void_p, c_void_p]),
    "nn_positions_subsample": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_int, c_void_p, c_void_p,
                                       c_void_p]),
    "nn_net_local_gaussian": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_float, c_int, c_uint64,
                                      c_void_p, c_void_p, c_int64, P(c_int64)]),
    "nn_electrodes_create": (c_int, [c_void_p, c_void_p, c_void_p, c_int, P(c_void_p)]),
    "nn_electrodes_destroy": (c_int, [c_void_p]),
    "nn_electrodes_measure": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "nn_measure_average": (c_int, [c_void_p, c_void_p, c_int, P(c_float)]),
    "nn_synchrony_create": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_int, P(c_void_p)]),
    "nn_synchrony_destroy": (c_int, [c_void_p]),
    "nn_synchrony_measure": (c_int, [c_void_p, c_void_p]),
    "nn_synchrony_get": (c_int, [c_void_p, c_void_p]),
    "nn_hebbian_create": (c_int, [c_void_p, c_int, c_float, c_int64, c_int, P(c_void_p)]),
    "nn_hebbian_destroy": (c_int, [c_void_p]),
    "nn_hebbian_update": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "nn_hebbian_timers": (c_int, [c_void_p, c_void_p]),
    "nn_mg_create": (c_int, [c_void_p, c_int, P(c_void_p)]),
    "nn_mg_destroy": (c_int, [c_void_p]),
    "nn_mg_levels": (c_int, [c_void_p, P(c_int)]),
    "nn_mg_apply": (c_int, [c_void_p, c_void_p, c_void_p]),
    "nn_mg_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_double, c_int, P(c_int), P(c_double)]),
    "nn_lmg_create": (c_int, [c_void_p, c_int, c_uint64, P(c_void_p)]),
    "nn_lmg_destroy": (c_int, [c_void_p]),
    "nn_lmg_add_solve": (c_int, [c_void_p, c_void_p, c_void_p, P(c_int)]),
    "nn_lmg_pairs": (c_int, [c_void_p, P(c_int)]),
    "nn_lmg_train": (c_int, [c_void_p, c_int, c_float, P(c_float)]),
    "nn_lmg_use_network": (c_int, [c_void_p, c_int]),
    "nn_lmg_set_post_sweeps": (c_int, [c_void_p, c_int]),
    "nn_lmg_autotune_post_sweeps": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_double, P(c_int), P(c_float)]),
    "nn_lmg_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_double, c_int, P(c_int), P(c_double)]),
    "nn_learned_create": (c_int, [c_void_p, c_uint64, P(c_void_p)]),
    "nn_learned_destroy": (c_int, [c_void_p]),
    "nn_learned_add_pair": (c_int, [c_void_p, c_void_p, c_void_p]),
    "nn_learned_train": (c_int, [c_void_p, c_int, c_float, P(c_float)]),
    "nn_learned_apply": (c_int, [c_void_p, c_void_p, c_void_p]),
    "nn_learned_use_network": (c_int, [c_void_p, c_int]),
    "nn_learned_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_double, c_int, P(c_int), P(c_double)]),
    "nn_learned_num_params": (c_int, [c_void_p, P(c_int64)]),
    "nn_learned_get_params": (c_int, [c_void_p, c_void_p]),
    "nn_learned_set_params": (c_int, [c_void_p, c_void_p]),
    "nn_learned_net_gradient": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, P(c_double), c_void_p]),
    "nn_act_layout": (c_int, [c_int, c_int, c_int, c_int, P(c_int64), P(c_int64), P(c_int64)]),
    "nn_act_pack": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p]),
    "nn_act_unpack": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_void_p]),
    "nn_conv3d_pack_weights": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int, c_void_p]),
    "nn_conv3d_forward": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int,
                                  c_void_p, c_void_p, c_void_p]),
    "nn_conv3d_wgrad": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                c_void_p]),
    "nn_pcg_kernel_time": (c_int, [c_void_p, P(c_float), P(c_int)]),
    "nn_pcg_solve_noalloc": (c_int, [c_void_p, c_int, c_int, c_int, c_double, c_double, c_void_p, c_void_p,
                                     c_void_p, c_double, c_int, P(c_int), P(c_double)]),
}

_lib = None


def declared_symbols() -> list[str]:
    return sorted(_SIGS)


def load(path: str | Path | None = None) -> C.CDLL:
    """Load (once) and type the shared library; raise if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else lib_path()
    if not p.exists():
        raise RuntimeError(f"libneuronephys is not built ({p}); run __graft_entry__.build() "
                           "-- there is no CPU fallback")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
