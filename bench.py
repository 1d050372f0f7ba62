#!/usr/bin/env python3
"""Benchmark of the per-timestep simulation path on one GB300.

Workload (``--workload c2``, the default): 1,000,000 Hodgkin-Huxley neurons,
RK4 at dt = 0.01 ms, Gaussian distance-dependent connectivity (sigma = 0.1,
100 out-edges per neuron, 1e8 synapses, int32 CSR), lognormal(-1, 1) nS
weights, delays U{1..20} steps, 20 % inhibitory, drive U[6, 12] uA/cm^2,
paracrine field on a 128^3 grid solved every 100 steps by Jacobi-PCG to a
1e-6 relative residual.  All inputs are seeded synthetic data.

One bench "step" is the workload's full run: 1,000 simulation timesteps
(10 paracrine periods of 100 timesteps, each replayed from a CUDA graph, plus
10 field solves).

Output: one JSON line (rank 0).  ``value`` is neuron-steps/s of the device-
resident path; ``e2e`` is the same metric through the C-ABI entry point that
takes host state buffers (host<->device copies inside the timed region).
``parity`` compares the GPU with the FP64 oracle over 50 timesteps started
from the GPU's state inside a population burst (after the timed region), and
``cpu_baseline`` is that oracle's time on the host cores.  Spike delivery is
chosen per period by the measured firing rate (``delivery``).  Two more
workloads ride along in the default line: ``cg_256cube`` (CG time to 1e-6 on
the 256^3 heterogeneous grid: plain, multigrid, learned multigrid) and
``batch256`` (256 independent networks in one simulation, both autotuners).
``--impl reference`` times the CPU oracle port of the same workload on the
host cores instead (the reference has no runnable CPU implementation of the
path); it builds the network and initial state with the oracle's own
generators (bit-exact to the device ones) and loads no GPU code.
Multi-GPU (torchrun): replicas only -- every rank simulates its own copy, no
data-path collective; value = all ranks' neuron-steps / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    "c2": dict(workload="hh_1M_gauss_k100_d20_grid128", n=1_000_000, kind="gauss", k=100, sigma=0.1,
               w_mu=-1.0, w_sigma=1.0, dmax=20, inh=0.2, i_lo=6.0, i_hi=12.0, grid=128, timescale=100,
               par_D=1.0, par_decay=0.0, total_steps=1000),
    "c3": dict(workload="hh_10M_block200_k100_d40_grid192", n=10_000_000, kind="block", k=100, n_regions=200,
               size_sigma=1.0, density_sigma=1.0, w_mu=-1.0, w_sigma=1.0, dmax=40, inh=0.2, i_lo=6.0, i_hi=12.0,
               grid=192, timescale=100, par_D=1.0, par_decay=0.0, total_steps=500),
    "c4": dict(workload="batch256_er_1k-64k_grids32-64", kind="batch", n_inst=256, size_lo=1000, size_hi=64000,
               p_lo=0.005, p_hi=0.05, gna_lo=0.8, gna_hi=1.2, drive_lo=4.0, drive_hi=16.0, w_total=2.5, inh=0.2,
               grid_lo=32, grid_hi=64, timescale=100, par_D=1.0, par_decay=0.0, total_steps=2000),
    "c5": dict(workload="cg_256cube_lognormalD_s1_l8_uptake0.1", kind="cg", grid=256, sigma=1.0, corr=8.0,
               D0=1.0, uptake=0.1, dt_s=1e-3, neurons=20000, rate=2.0,
               # iterations of the FP64 oracle PCG to 1e-6 on this seeded instance
               # (oracle.pcg7 run to convergence once; the CPU arms time a bounded
               # number of iterations and scale by this count)
               fp64_iters=329, train_rhs=6, train_steps=400, lmg_train_steps=3000),
    "c1": dict(workload="hh_1k_er_p0.01_grid32", n=1000, kind="er", p=0.01, w_max=0.5, dmax=1, inh=0.2,
               i_lo=5.0, i_hi=15.0, grid=32, timescale=100, par_D=1.0, par_decay=0.0, total_steps=10000),
}

# Algorithmic bytes per unit of work (what one launch must move at minimum):
HH_BYTES_PER_NEURON_STEP = 60      # R: V,m,h,n,ge,gi,I (28 B) + ring (E,I) slot (8 B); W: 6 state floats (24 B)
# Algorithmic FP32 work of one neuron-step, counted on the FP64 oracle's
# expression tree (oracle.c: hh_rates, hh_rhs, orc_hh_rk4, orc_sim_step), each
# add, subtract, multiply and divide one operation:
#   rates: (V+c)/s for six rates (12), alpha_m 2 + alpha_n 3 (1 - e, u / den,
#          0.1 x), beta_m / alpha_h / beta_n one scale each (3), beta_h 2  -> 22
#   rhs:   n^2 1, ionic current 15, synaptic + field current 9, dV/dt 3,
#          three gates 4 each, two conductance decays 1 each                -> 42
#   RK4:   4 right-hand sides (4 x 64 = 256), three stage points
#          (6 x 2 each = 36), the combination (6 x 7 = 42)                   -> 334
#   step:  synaptic input added (2), drive + noise (2), Box-Muller scaling (2) -> 6
HH_FP32_OPS_PER_NEURON_STEP = 340
# transcendental calls of the same tree: 6 exponentials per right-hand side,
# and log, sqrt, sin, cos per neuron pair for the noise
HH_TRANSCENDENTALS_PER_NEURON_STEP = 26
FP32_LANES_PER_SM = 128            # FP32 lanes per SM (sm_100 family), one fused multiply-add (2 ops) per lane and clock
PCG_BYTES_PER_CELL_ITER = 40       # k_cg_iter R: r,w,s,p,x; W: r,w,s,p,x -> 10 floats per cell
PCG_HET_BYTES_PER_CELL_ITER = 48   # k_cg_iter<HET>: + D and 1/diag reads
PUSH_BYTES_PER_EVENT = 13          # 4 B target + 4 B weight + 1 B delay + 4 B ring read-modify-write
PULL_CSC_BYTES_PER_SYNAPSE = 9     # full CSC sweep: 4 B source + 4 B weight + 1 B delay

# DRAM bytes per unit of work from one ncu capture of the kernel
# (dram__bytes_read.sum + dram__bytes_write.sum per launch / units per launch).
NCU_TRAFFIC_PER_UNIT = {
    "hh_step": 36.03,        # 36.03 MB read + 0 MB written per 1M-neuron launch (writes stay in L2)
    "pcg_iteration": 20.2,   # 41.99 MB read + 0.45 MB written per 128^3 launch (the rest hits L2)
}


def measured_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------- distributed --

def dist_env() -> tuple[int, int, int]:
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def dist_init(world: int):
    if world <= 1:
        return None
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group("gloo")
    return dist


def barrier(dist) -> None:
    if dist is not None:
        dist.barrier()


def reduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def aggregate(units_per_rank: float, seconds_per_rank: float, dist) -> tuple[float, float]:
    """Whole-job throughput: units of all ranks / the slowest rank's time."""
    tmax = reduce_max(dist, seconds_per_rank)
    units = reduce_sum(dist, units_per_rank)
    return units / tmax, tmax


# ------------------------------------------------------------------ clocks --

class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device, self.proc, self.path = device, None, None

    def start(self) -> None:
        try:
            self.path = Path(f"/tmp/nn_clocks_{os.getpid()}.csv")
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        self.path.unlink(missing_ok=True)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# --------------------------------------------------------------- our arm ---

def build_sim(nn, ctx, wl: dict, seed: int = 1, delivery: int = 0, raster: int = 0, tpb: int = 0, npt: int = 0):
    c = nn.default_config(wl["n"])
    c.delivery = delivery
    c.threads_per_block, c.neurons_per_thread = tpb, npt
    c.seed = seed
    c.max_delay = max(1, wl["dmax"])
    c.grid = wl["grid"]
    c.timescale = wl["timescale"]
    c.par_D = wl["par_D"]
    c.par_decay = wl["par_decay"]
    c.par_rtol = 1e-6
    c.par_max_iter = 5000
    c.raster_capacity = raster
    s = nn.Simulation(ctx, c)
    if wl["kind"] == "gauss":
        sp = nn.default_net_spec(nn.NN_NET_GAUSS)
        sp.k, sp.sigma, sp.w_mu, sp.w_sigma, sp.dmax = wl["k"], wl["sigma"], wl["w_mu"], wl["w_sigma"], wl["dmax"]
        sp.inh_fraction, sp.inh_random = wl["inh"], 1
    elif wl["kind"] == "block":
        sp = nn.default_net_spec(nn.NN_NET_BLOCK)
        sp.k, sp.n_regions, sp.block_dmax = wl["k"], wl["n_regions"], wl["dmax"]
        sp.region_size_sigma, sp.density_sigma = wl["size_sigma"], wl["density_sigma"]
        sp.w_mu, sp.w_sigma, sp.inh_fraction, sp.inh_random = wl["w_mu"], wl["w_sigma"], wl["inh"], 1
    else:
        sp = nn.default_net_spec(nn.NN_NET_ER)
        sp.p, sp.w_max, sp.inh_fraction, sp.inh_random = wl["p"], wl["w_max"], wl["inh"], 0
    s.generate_network(sp)
    s.init_state(-65.0, wl["i_lo"], wl["i_hi"])
    return s


def run_ours(args, wl: dict, dist, rank: int, local_rank: int) -> dict | None:
    import neuronephys_clean_gb300 as nn
    ctx = nn.Context(local_rank)
    # the raster records the parity window's spikes (restarted before it)
    sim = build_sim(nn, ctx, wl, raster=2_000_000 if args.cpu_baseline else 0,
                    delivery=DELIVERY_MODES[args.delivery])
    P = wl["total_steps"]  # timesteps per bench step: one full run of the workload
    n = wl["n"]
    el_info = None
    if args.electrodes > 0:
        el_info = set_knn_electrodes(sim, args.electrodes, 50, args.electrode_every)
    # settle: start the timed region in steady tonic firing, not at rest
    sim.step(args.settle)
    # the field solver's tile depth from the autotuner (whole periods with the
    # solve overlapped, in the settled state; the simulation is restored)
    cg_tile = sim.autotune_solver(10) if wl["grid"] else (0, 0.0)
    for _ in range(args.warmup):  # warm-up also captures the period graph
        sim.step(P)
    ctx.synchronize()
    if args.delivery == "auto":
        sim.delivery_log(reset=True)
    launches0 = ctx.kernel_launches
    _, spikes_a = sim.counters()
    clocks = ClockSampler(local_rank)
    barrier(dist)
    clocks.start()
    ctx.time_begin()
    for _ in range(args.steps):
        sim.step(P)
    ms = ctx.time_end()
    clock_info = clocks.stop()
    barrier(dist)
    launches = ctx.kernel_launches - launches0
    _, spikes_b = sim.counters()
    delivery_info = {"mode": args.delivery}
    if args.delivery == "auto":
        modes, rates = sim.delivery_log(reset=True)
        delivery_info.update({
            "pull_rate": float(sim.config.pull_rate),
            "periods_push": int((modes == 0).sum()), "periods_pull": int((modes == 1).sum()),
            "modes": "".join("L" if m else "S" for m in modes.tolist()),
            "max_measured_rate": float(rates.max()) if len(rates) else None,
            "rule": "each period of the timed region: pull (L) when the latest measured period fired at least "
                    "pull_rate spikes per neuron and step, else push (S)"})
    st = sim.solve_stats()
    seconds = ms / 1e3
    units = float(n) * P * args.steps
    value, tmax = aggregate(units, seconds, dist)
    spikes = spikes_b - spikes_a
    nnz = sim.nnz
    events = spikes * (nnz / n)

    # per-kernel durations: CUDA events bracket every neuron-update / delivery
    # launch (event nodes in the period graph) and the solver iterations over
    # one more bench step, with the field solves in line so that each kernel
    # runs alone (overlapped, the neuron update's launches also wait for the
    # solver's CTAs to leave their SMs).  The neuron update's roofline uses the
    # median launch: the bytes it counts are the state's, and the launches of a
    # burst also scatter the spikes' edges.
    sim.set_kernel_timing(True)
    sim.step(P)
    kt = sim.kernel_times()
    sim.set_kernel_timing(False)
    # the delivery slot between the second and third event of each step holds
    # the pull gather in pull periods; in push periods it is empty (the
    # scatter runs inside k_hh_step) and its time is the events' own interval
    if args.delivery == "auto":
        modes_t, _ = sim.delivery_log(reset=True)
        any_pull = bool((modes_t == 1).any())
    else:
        any_pull = args.delivery == "pull"
    hbm_peak, peak_kind = measured_peaks()
    G = wl["grid"] ** 3
    hh_ms = kt.hh_step_median_ms if kt.hh_step_median_ms > 0 else kt.hh_step_ms
    hh_ach = n * HH_BYTES_PER_NEURON_STEP / (hh_ms * 1e-3) / 1e9 if hh_ms > 0 else None
    it_ms = kt.solve_ms / kt.solve_iterations if kt.solve_iterations else None
    pcg_ach = G * PCG_BYTES_PER_CELL_ITER / (it_ms * 1e-3) / 1e9 if it_ms else None
    # time per bench step: P neuron updates and P / timescale solves
    per_period_hh = hh_ms * P
    per_period_pcg = kt.solve_ms * (P // wl["timescale"])
    hh_roof = {"bound": "hbm", "kernel": "k_hh_step", "achieved": hh_ach, "peak": hbm_peak, "unit": "GB/s",
               "frac": hh_ach / hbm_peak if hh_ach else None,
               "traffic": (NCU_TRAFFIC_PER_UNIT["hh_step"] * n) if NCU_TRAFFIC_PER_UNIT["hh_step"] else None,
               "algorithmic_bytes": n * HH_BYTES_PER_NEURON_STEP, "launch_ms": hh_ms,
               "launch_ms_of": "median launch of the last period of one bench step after the timed region, solves in line",
               "peak_source": peak_kind}
    pcg_roof = {"bound": "hbm", "kernel": "k_cg_iter (one PCG iteration)", "achieved": pcg_ach,
                "peak": hbm_peak, "unit": "GB/s", "frac": pcg_ach / hbm_peak if pcg_ach else None,
                "traffic": (NCU_TRAFFIC_PER_UNIT["pcg_iteration"] * G) if NCU_TRAFFIC_PER_UNIT["pcg_iteration"] else None,
                "algorithmic_bytes": G * PCG_BYTES_PER_CELL_ITER, "launch_ms": it_ms, "peak_source": peak_kind}
    dominant, other = (hh_roof, pcg_roof) if per_period_hh >= per_period_pcg else (pcg_roof, hh_roof)
    # the neuron update's own bound is FP32 arithmetic and instruction issue:
    # its algorithmic operations against the FP32 peak at the sampled clock
    clk_mhz = clock_info.get("sm_mhz") or 2070.0
    fp32_peak = ctx.num_sms * FP32_LANES_PER_SM * 2 * clk_mhz * 1e6 / 1e12
    hh_tflops = n * HH_FP32_OPS_PER_NEURON_STEP / (hh_ms * 1e-3) / 1e12 if hh_ms > 0 else None
    hh_fp32 = {"bound": "fp32", "kernel": "k_hh_step", "achieved": hh_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
               "frac": hh_tflops / fp32_peak if hh_tflops else None,
               "ops_per_neuron_step": HH_FP32_OPS_PER_NEURON_STEP,
               "transcendentals_per_neuron_step": HH_TRANSCENDENTALS_PER_NEURON_STEP,
               "peak_formula": f"{ctx.num_sms} SMs x {FP32_LANES_PER_SM} FP32 lanes x 2 (fused multiply-add) x "
                               f"{clk_mhz:.0f} MHz (median sampled SM clock)",
               "launch_ms": hh_ms,
               "ncu": "profiles/k_hh_step_hh1M.md: FMA-pipe busy cycles and issue-active share of the same kernel"}

    # end to end through the host-buffer C-ABI call
    e2e = None
    if args.e2e_steps > 0:
        pin_in = nn.PinnedArray((6, n), np.float32)
        pin_out = nn.PinnedArray((6, n), np.float32)
        for q, k in enumerate(("V", "M", "H", "N", "GE", "GI")):
            pin_in.array[q] = sim.get_field(k)
        sim.run_host(pin_in.array, P, pin_out.array)  # warm
        pin_in, pin_out = pin_out, pin_in
        barrier(dist)
        # each step continues from the previous one's state (host buffers in
        # and out every step), so the window spans as much of the network's
        # dynamics as the timed region does
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            sim.run_host(pin_in.array, P, pin_out.array)
            pin_in, pin_out = pin_out, pin_in
        e2e_s = time.perf_counter() - t0
        e2e_val, _ = aggregate(float(n) * P * args.e2e_steps, e2e_s, dist)
        e2e = {"value": e2e_val, "unit": "neuron-steps/s", "h2d_bytes_per_step": 6 * 4 * n,
               "d2h_bytes_per_step": 6 * 4 * n + 8 * 2, "steps": args.e2e_steps}
        pin_in.free()
        pin_out.free()

    if rank != 0:
        return None
    line = {
        "metric": "neuron-steps/s", "value": value, "unit": "neuron-steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tmax * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded counter-based generators)",
        "config": workload_config(wl, nnz, args.delivery),
        "delivery": delivery_info,
        "autotuned": {"cg_tile": f"32 x 16 x {cg_tile[0]}", "trial_ms_per_timestep": cg_tile[1],
                      "how": "each tile depth timed over six periods with the solve overlapping the neuron "
                             "updates, from a snapshot restored afterwards"},
        "electrodes": el_info,
        "synaptic_events_per_s": events / seconds if seconds else None,
        "spikes_in_timed_region": spikes,
        "cg": {"iterations_last_solve": st.iterations, "relres_last_solve": st.relres,
               "time_to_tol_ms": kt.solve_ms, "grid": wl["grid"]},
        "roofline": dominant, "roofline_other": other, "roofline_fp32": hh_fp32,
        "kernel_ms": {"k_hh_step": kt.hh_step_ms, "k_hh_step_median": kt.hh_step_median_ms,
                      ("k_deliver_pull" if any_pull else "empty_delivery_slot"): kt.deliver_ms,
                      "delivery": ("pull gather after the neuron update (mean over the steps, push steps "
                                   "included)" if any_pull else
                                   "push scatter fused into k_hh_step; empty_delivery_slot is the interval "
                                   "between two timing events with no kernel between them"),
                      "pcg_solve": kt.solve_ms, "samples": kt.samples},
        "gpu_launches": int(launches),
        "clocks": clock_info,
        "e2e": e2e,
    }
    if args.cpu_baseline:
        line["parity"], line["cpu_baseline"] = parity_and_cpu_baseline(sim, wl, args)
    sim.close()
    if args.c5 and rank == 0 and args.gpus == 1 and wl["workload"] == WORKLOADS["c2"]["workload"]:
        line["cg_256cube"] = c5_leg(nn, ctx, args)
    ctx.close()
    if args.c4 and rank == 0 and args.gpus == 1 and wl["workload"] == WORKLOADS["c2"]["workload"]:
        line["batch256"] = c4_leg(args, local_rank)
    return line


def c4_leg(args, local_rank: int) -> dict:
    """The batched configuration (256 networks of 1k-64k neurons, their own
    32^3-64^3 grids) in the default line: the `--workload c4` measurement with
    3 timed steps of 2,000 timesteps after 1 warm-up step, both autotuners run
    first."""
    a = argparse.Namespace(**vars(args))
    a.steps, a.warmup, a.e2e_steps = 3, 1, 1
    r = run_batch(a, WORKLOADS["c4"], None, 0, local_rank)
    keep = ("value", "unit", "steps", "warmup", "ms_per_step", "config", "spikes_in_timed_region", "cg", "timestep",
            "gpu_launches", "clocks", "e2e")
    return {k: r[k] for k in keep if k in r}


def c5_leg(nn, ctx, args) -> dict:
    """The workload's third metric, CG time to a 1e-6 relative residual, on
    the configuration-5 system (256^3 cells, lognormal D with sigma 1 and an
    8-cell correlation length, uptake 0.1), in the default line:
    * plain Jacobi-PCG (the baseline), the classical multigrid FCG, and the
      multigrid whose 32^3 level is solved by the learned U-Net (trained here
      on the GPU, on the coarse problems of six training right-hand sides);
    * each timed on the bench right-hand side and on four held-out ones
      (spike-source fields of seeds not used in training);
    * each bench solution's error against the FP64 oracle's CG solution of
      the same system to a 1e-10 relative residual (16 host cores)."""
    import oracle
    from neuronephys_clean_gb300 import fields
    wl = WORKLOADS["c5"]
    shape, D, b, alpha, beta = cg_problem(wl)
    G = int(np.prod(shape))
    pc = nn.PCG(ctx, shape[2], shape[1], shape[0], alpha, beta, ctx.to_device(D.ravel()))
    bench_rhs = ctx.to_device(b)
    held_out = [ctx.to_device(fields.spike_sources(shape, wl["neurons"], wl["rate"], seed=5000 + j))
                for j in range(4)]
    dx = ctx.empty((G,), np.float32)

    def timed(solve, rhs, reps=2):
        solve(rhs, dx)  # warm (graph capture, first touches)
        ms, its = [], []
        for _ in range(reps):
            dx.zero()
            ctx.time_begin()
            it, rel = solve(rhs, dx)
            ms.append(ctx.time_end())
            its.append(it)
        return statistics.mean(ms), statistics.mean(its), rel

    def held(solve):
        r = [timed(solve, h, reps=1) for h in held_out]
        return {"ms_mean": statistics.mean(x[0] for x in r), "iterations_mean": statistics.mean(x[1] for x in r)}

    out, sols = {}, {}
    plain = lambda rb, x: pc.solve(rb, x, 1e-6, 20000)  # noqa: E731
    ms, it, rel = timed(plain, bench_rhs)
    sols["jacobi_pcg"] = dx.numpy().astype(np.float64)
    out["jacobi_pcg"] = {"ms_to_tol": ms, "iterations": it, "relres": rel, "held_out": held(plain)}
    mg = nn.MultigridPCG(pc)
    classical = lambda rb, x: mg.solve(rb, x, 1e-6)  # noqa: E731
    ms, it, rel = timed(classical, bench_rhs)
    sols["multigrid"] = dx.numpy().astype(np.float64)
    out["multigrid"] = {"ms_to_tol": ms, "iterations": it, "relres": rel, "levels": mg.levels,
                        "held_out": held(classical)}
    mg.close()
    lm = nn.LearnedMultigrid(pc, level=3, seed=7)
    t0 = time.perf_counter()
    pairs = lm.add_solves([fields.spike_sources(shape, wl["neurons"], wl["rate"], seed=2000 + j)
                           for j in range(wl["train_rhs"])])
    loss = lm.train(wl["lmg_train_steps"], 1e-3)
    t_train = time.perf_counter() - t0
    # Jacobi sweeps after the network's correction, chosen by timing a solve
    # of one training right-hand side
    post_sweeps, _ = lm.autotune_post_sweeps(
        [ctx.to_device(fields.spike_sources(shape, wl["neurons"], wl["rate"], seed=2000 + j))
         for j in range(wl["train_rhs"])])
    learned = lambda rb, x: lm.solve(rb, x, 1e-6)  # noqa: E731
    ms, it, rel = timed(learned, bench_rhs)
    sols["learned_multigrid"] = dx.numpy().astype(np.float64)
    out["learned_multigrid"] = {"ms_to_tol": ms, "iterations": it, "relres": rel, "network_level_grid": 32,
                                "post_sweeps": post_sweeps, "held_out": held(learned),
                                "training": {"right_hand_sides": wl["train_rhs"], "pairs": pairs,
                                             "adam_steps": wl["lmg_train_steps"], "s": t_train, "final_loss": loss}}
    lm.close()
    pc.close()
    t1 = time.perf_counter()
    xs, it_o, rel_o = oracle.pcg7(b, np.zeros(G), shape, alpha, beta, D, rtol=1e-10, max_iter=5000)
    t_oracle = time.perf_counter() - t1
    nref = float(np.linalg.norm(xs))
    for k, x in sols.items():
        out[k]["error_vs_fp64"] = float(np.linalg.norm(x - xs) / nref)
    plain_ms = out["jacobi_pcg"]["ms_to_tol"]
    for k in ("multigrid", "learned_multigrid"):
        out[k]["vs_plain_time"] = out[k]["ms_to_tol"] / plain_ms
        out[k]["held_out"]["vs_plain_time"] = out[k]["held_out"]["ms_mean"] / out["jacobi_pcg"]["held_out"]["ms_mean"]
    out["workload"] = wl["workload"]
    out["fp64_oracle"] = {"iterations": it_o, "relres": rel_o, "s": t_oracle,
                          "cores": int(oracle.lib().orc_num_threads())}
    out["tolerance"] = "relative residual 1e-6 (FP64 reductions); error = |x - x_fp64| / |x_fp64|"
    return out


def set_knn_electrodes(sim, count: int, k: int, every: int = 1, seed: int = 11) -> dict:
    """ElectrodeNet's regions (Morphology::GenSphericalRegions,
    src/morphology.cpp:48-72): the k nearest neurons of each of `count`
    randomly chosen electrode neurons, recorded every `every` steps by the
    fused recording."""
    x, y, z = (sim.get_field(f).astype(np.float64) for f in ("X", "Y", "Z"))
    n = len(x)
    centers = np.random.default_rng(seed).choice(n, count, replace=False)
    regions = []
    for c in centers:
        d2 = (x - x[c]) ** 2 + (y - y[c]) ** 2 + (z - z[c]) ** 2
        regions.append(np.argpartition(d2, k)[:k])
    idx = np.concatenate(regions).astype(np.int32)
    off = (np.arange(count + 1) * k).astype(np.int32)
    sim.set_electrodes(idx, off, every=every, capacity=1024)
    return {"regions": count, "neurons_per_region": k, "every_steps": every}


DELIVERY_MODES = {"push": 0, "pull": 1, "auto": 2}


def workload_config(wl: dict, nnz: int, delivery: str) -> dict:
    """The `config` object of both arms' lines for a single-network workload."""
    n = wl["n"]
    return {"workload": wl["workload"], "neurons": n, "synapses": int(nnz), "timesteps_per_step": wl["total_steps"],
            "dt_ms": 0.01, "grid": wl["grid"], "delivery": delivery, "parallelism": "replicas",
            "l2": f"inputs larger than L2 (CSR {nnz * 9 / 1e9:.1f} GB, ring "
                  f"{(wl['dmax'] + 1) * n * 8 / 1e6:.0f} MB, state {n * 28 / 1e6:.0f} MB per step)"}


# ---------------------------------------------------------- CPU baseline ---

def parity_and_cpu_baseline(sim, wl: dict, args) -> tuple[dict, dict]:
    """The GPU against the FP64 oracle at the benchmarked configuration.

    Both start from the GPU's state at a period boundary inside a population
    burst (neuron fields, delay ring and step counter: the complete state a
    step depends on) and advance args.parity_steps timesteps (>= 20, so that
    spikes of the window arrive through the delay ring within it).  Reported:
    raster equality (one-step shifts of crossings within 0.01 mV of the
    threshold counted apart), the per-neuron trajectory criterion of
    oracle/parity.py and the largest relative V error away from spikes.  The
    oracle's time for the window is the CPU baseline (OpenMP over the host
    cores), plus one PCG solve of the 128^3 field amortised over its period."""
    import oracle
    from oracle.parity import find_burst, window_parity
    n, k = wl["n"], args.parity_steps
    P = wl["timescale"]
    periods = find_burst(sim, P, n)
    res = window_parity(sim, k)
    o, t_steps, t0 = res.pop("_oracle"), res.pop("_t_oracle_s"), res["start_step"]
    parity = dict(res, settle_periods_to_burst=periods,
                  tolerance="V, m, h, n within 1e-4 relative (floors 1 mV / 1e-3) away from spikes, within a 1 us "
                            "spike-time shift in a spike; rasters identical except one-step shifts of crossings "
                            "within 0.01 mV of the threshold and the differences they cause downstream (cascade); "
                            "the neurons those reach leave the trajectory check (max_rel_excluded reports them)",
                  oracle="FP64 C restatement (oracle/oracle.c), started from the GPU's neuron fields, delay ring "
                         "and step counter")
    g = wl["grid"]
    t_solve = 0.0
    if g:
        # the period's field solve: b = u + deposits of the window's spikes,
        # warm-started from u, as the simulation forms it
        dt_s = wl["timescale"] * 0.01 * 1e-3
        alpha, beta = dt_s * wl["par_D"] * g * g, dt_s * wl["par_decay"]
        vox = oracle.voxels(sim.get_field("X"), sim.get_field("Y"), sim.get_field("Z"), g)
        u = sim.density().astype(np.float64)
        fired = np.fromiter((j for (_, j) in o.margins), np.int64, len(o.margins))
        b = u + np.bincount(vox[fired], minlength=g ** 3)
        t1 = time.perf_counter()
        oracle.pcg7(b, u, (g, g, g), alpha, beta, rtol=1e-6)
        t_solve = time.perf_counter() - t1
    per_step = t_steps / k + t_solve / P
    cpu = {"value": n / per_step, "unit": "neuron-steps/s", "cores": int(oracle.lib().orc_num_threads()),
           "kind": "port", "t_steps_s": t_steps, "t_solve_s": t_solve,
           "sample": f"{k} timesteps of all {n} neurons from the GPU's state at step {t0} inside a population "
                     f"burst ({parity['spikes_oracle']} spikes delivered; FP64 oracle, OpenMP) + one {g}^3 PCG "
                     f"solve amortised over {P} timesteps"}
    return parity, cpu


def run_delivery_sweep(args, wl: dict, rank: int, local_rank: int) -> dict | None:
    """Spike delivery alone on the workload's network at firing fractions
    1e-4 .. 3e-1 of the neurons per step: push scatter (13 B per synaptic
    event) and pull gather (the chunked layout: one 4-byte entry word per
    synapse, the weights of the synapses whose source fired, 8 B ring write
    per neuron), CUDA-event timed, achieved algorithmic GB/s against the
    measured HBM peak."""
    if rank != 0:
        return None
    import neuronephys_clean_gb300 as nn
    ctx = nn.Context(local_rank)
    wl = dict(wl, grid=0)
    sim = build_sim(nn, ctx, wl, delivery=nn.NN_DELIVERY_PULL)
    n, nnz = wl["n"], sim.nnz
    rp, _, _, dly, _ = sim.get_network()
    sliced, cols = sim.pull_info()
    dmax = wl["dmax"]
    # past the longest delay, so that the gather covers every delay slice
    # (before step d a delay-d synapse reaches back before step 0)
    sim.step(dmax + 1)
    d1cum = np.concatenate([[0], np.cumsum(dly == 1)])  # delay-1 synapses before each CSR position
    hbm_peak, peak_kind = measured_peaks()
    rng = np.random.default_rng(5)
    rows = []
    for frac in (1e-4, 3e-4, 1e-3, 3e-3, 1e-2, 3e-2, 1e-1, 3e-1):
        cnt = max(1, int(frac * n))
        lst = np.sort(rng.choice(n, cnt, replace=False)).astype(np.int32)
        events = int((rp[lst + 1] - rp[lst]).sum())
        dl = ctx.to_device(lst)
        res = {"fraction": frac, "spikes": cnt, "events": events}
        # the list fires at the current step, so only its delay-1 synapses
        # arrive in the gathered step: the weights the sliced pull reads
        hits = int((d1cum[rp[lst + 1]] - d1cum[rp[lst]]).sum()) if sliced else 0
        for mode, name, reps in ((nn.NN_DELIVERY_PUSH, "push", 20), (nn.NN_DELIVERY_PULL, "pull", 5)):
            sim.deliver_spikes(dl, cnt, mode)
            ctx.time_begin()
            for _ in range(reps):
                sim.deliver_spikes(dl, cnt, mode)
            ms = ctx.time_end() / reps
            if mode == nn.NN_DELIVERY_PUSH:
                nbytes = events * PUSH_BYTES_PER_EVENT
            elif sliced:
                # entry words + weights of arriving synapses + ring slot
                # written + the D - 1 bitmap rows read
                nbytes = nnz * 4 + hits * 4 + n * 8 + dmax * (n // 8)
            else:
                nbytes = nnz * PULL_CSC_BYTES_PER_SYNAPSE + n * 8 + n // 8
            res[name] = {"ms": ms, "GBs": nbytes / (ms * 1e-3) / 1e9, "frac_of_peak": nbytes / (ms * 1e-3) / 1e9 / hbm_peak}
            if mode == nn.NN_DELIVERY_PULL:
                # the gather kernel alone (the bitmap built above stays): the
                # simulation's pull mode runs only this kernel, its bitmap
                # written by the neuron update
                sim.pull_gather()
                ctx.time_begin()
                for _ in range(reps):
                    sim.pull_gather()
                gms = ctx.time_end() / reps
                res[name]["gather_ms"] = gms
                res[name]["gather_frac_of_peak"] = nbytes / (gms * 1e-3) / 1e9 / hbm_peak
                csc = nnz * PULL_CSC_BYTES_PER_SYNAPSE + n * 8 + n // 8
                res[name]["bytes"] = nbytes
                # the rate at which a sweep over the 9-byte CSC entries would
                # have to run to finish in the same time
                res[name]["GBs_csc9_equivalent"] = csc / (ms * 1e-3) / 1e9
                res[name]["synapses_per_s"] = nnz / (ms * 1e-3)
        rows.append(res)
    cross = next((r["fraction"] for r in rows if r["pull"]["ms"] < r["push"]["ms"]), None)
    sim.close()
    ctx.close()
    # "ms": list in, delivery out (the pull rebuilds the bitmap from the list
    # first); "gather_ms": the pull gather kernel by itself
    return {"metric": "spike delivery GB/s vs firing fraction", "workload": wl["workload"], "neurons": n,
            "synapses": nnz, "peak_GBs": hbm_peak, "peak_source": peak_kind,
            "pull_kernel": (f"k_deliver_pull_sliced (chunked entries and bitmap ranges staged by bulk copies, "
                            f"{cols} columns per block; bytes: 4 per synapse + 4 per arriving synapse + 8 per "
                            "neuron + the bitmap rows)")
            if sliced else "k_deliver_pull (warp per column; bytes: the 9-byte CSC entry per synapse)",
            "sweep": rows,
            "push_pull_crossover_fraction": cross}


def run_launch_shapes(args, wl: dict, rank: int, local_rank: int) -> dict | None:
    """The neuron update's launch shapes on the workload: for every
    (neurons per thread, threads per block) the autotuner considers, a
    simulation from the same seed (the shapes give bit-identical neurons, so
    every one follows the same trajectory) settles, warms up and times
    args.steps bench steps with CUDA events, field solve included; one more
    bench step with kernel timing gives the median neuron-update launch.
    Four neurons per thread load the state as 128-bit float4 vectors, two as
    float2, one as float."""
    if rank != 0:
        return None
    import neuronephys_clean_gb300 as nn
    ctx = nn.Context(local_rank)
    P, n = wl["total_steps"], wl["n"]
    rows = []
    for npt in (1, 2, 4):
        for tpb in (64, 128, 256):
            sim = build_sim(nn, ctx, wl, delivery=DELIVERY_MODES[args.delivery], tpb=tpb, npt=npt)
            sim.step(args.settle)
            for _ in range(args.warmup):
                sim.step(P)
            ctx.time_begin()
            for _ in range(args.steps):
                sim.step(P)
            ms = ctx.time_end()
            sim.set_kernel_timing(True)
            sim.step(P)
            kt = sim.kernel_times()
            sim.set_kernel_timing(False)
            rows.append({"neurons_per_thread": npt, "threads_per_block": tpb,
                         "load": {1: "float", 2: "float2", 4: "float4"}[npt],
                         "ms_per_timestep": ms / (args.steps * P),
                         "neuron_steps_per_s": n * P * args.steps / (ms * 1e-3),
                         "k_hh_step_median_us": kt.hh_step_median_ms * 1e3})
            sim.close()
    ctx.close()
    best = min(rows, key=lambda r: r["ms_per_timestep"])
    return {"metric": "neuron-steps/s by neuron-update launch shape", "workload": wl["workload"], "neurons": n,
            "steps": args.steps, "warmup": args.warmup, "timesteps_per_step": P, "shapes": rows,
            "fastest": {"neurons_per_thread": best["neurons_per_thread"],
                        "threads_per_block": best["threads_per_block"]}}


def batch_layout(wl: dict, seed: int = 4):
    """Seeded instance sizes (log-uniform), ER p, gNa scale, drive and grid
    sides (32 at 1k neurons to 64 at 64k, growing as size^(1/6))."""
    rng = np.random.default_rng(seed)
    B = wl["n_inst"]
    sizes = np.exp(rng.uniform(np.log(wl["size_lo"]), np.log(wl["size_hi"]), B)).astype(np.int64)
    p = rng.uniform(wl["p_lo"], wl["p_hi"], B)
    gna = rng.uniform(wl["gna_lo"], wl["gna_hi"], B).astype(np.float32)
    drive = rng.uniform(wl["drive_lo"], wl["drive_hi"], B).astype(np.float32)
    sides = np.clip(np.rint(wl["grid_lo"] * (sizes / wl["size_lo"]) ** (1 / 6)), wl["grid_lo"], wl["grid_hi"])
    return sizes, p, gna, drive, sides.astype(np.int32)


def run_batch(args, wl: dict, dist, rank: int, local_rank: int) -> dict | None:
    """A batch of independent networks in one simulation: one neuron-update
    launch per step for all instances, per-instance paracrine grids solved by
    the batched PCG, launch shape chosen by the autotuner."""
    import neuronephys_clean_gb300 as nn
    ctx = nn.Context(local_rank)
    sizes, p, gna, drive, sides = batch_layout(wl)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    n = int(off[-1])
    c = nn.default_config(n)
    c.seed, c.grid, c.timescale, c.par_D, c.par_decay = 1, 0, wl["timescale"], wl["par_D"], wl["par_decay"]
    c.par_rtol, c.par_max_iter, c.raster_capacity = 1e-6, 5000, 0
    sim = nn.Simulation(ctx, c)
    sim.set_instances(off, sides)
    t0 = time.perf_counter()
    # weight ceiling per instance: the expected total synaptic weight onto a
    # neuron (in-degree p * size times mean weight w_max / 2) stays that of the
    # 1k-neuron configuration (10 inputs, weights U[0, 0.5]: 2.5 nS), so large
    # dense instances are not driven into an unstable conductance regime
    w_inst = (wl["w_total"] * 2.0 / (p * sizes)).astype(np.float32)
    nnz = sim.generate_batch_er(p, w_max=w_inst, inh_fraction=wl["inh"])
    t_gen = time.perf_counter() - t0
    sim.init_state(-65.0, 0.0, 0.0)
    sim.set_field("GNA_SCALE", np.repeat(gna, sizes))
    sim.set_field("IDRIVE", np.repeat(drive, sizes))
    sim.step(args.settle)
    tpb, npt, tune_ms = sim.autotune(20)
    cpb, pcg_iter_ms = sim.autotune_solver(10)
    P = wl["total_steps"]
    for _ in range(args.warmup):
        sim.step(P)
    ctx.synchronize()
    launches0 = ctx.kernel_launches
    _, spikes_a = sim.counters()
    clocks = ClockSampler(local_rank)
    barrier(dist)
    clocks.start()
    ctx.time_begin()
    for _ in range(args.steps):
        sim.step(P)
    ms = ctx.time_end()
    clock_info = clocks.stop()
    barrier(dist)
    launches = ctx.kernel_launches - launches0
    _, spikes_b = sim.counters()
    # per-kernel durations over one more bench step, each kernel alone (see run_ours)
    sim.set_kernel_timing(True)
    sim.step(P)
    kt = sim.kernel_times()
    sim.set_kernel_timing(False)
    value, tmax = aggregate(float(n) * P * args.steps, ms / 1e3, dist)
    iters = sim.instance_iterations()
    hbm_peak, peak_kind = measured_peaks()
    hh_ms = kt.hh_step_median_ms if kt.hh_step_median_ms > 0 else kt.hh_step_ms  # median launch (see run_ours)
    hh_ach = n * HH_BYTES_PER_NEURON_STEP / (hh_ms * 1e-3) / 1e9 if hh_ms > 0 else None
    # end to end: state from / to pinned host memory around each bench step
    pin_in = nn.PinnedArray((6, n), np.float32)
    pin_out = nn.PinnedArray((6, n), np.float32)
    for q, k in enumerate(("V", "M", "H", "N", "GE", "GI")):
        pin_in.array[q] = sim.get_field(k)
    t1 = time.perf_counter()
    for _ in range(max(1, args.e2e_steps)):
        sim.run_host(pin_in.array, P, pin_out.array)
        pin_in, pin_out = pin_out, pin_in  # the next step continues from this one
    e2e_s = time.perf_counter() - t1
    e2e_val, _ = aggregate(float(n) * P * max(1, args.e2e_steps), e2e_s, dist)
    pin_in.free()
    pin_out.free()
    if rank != 0:
        return None
    line = {
        "metric": "neuron-steps/s", "value": value, "unit": "neuron-steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tmax * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded counter-based generators)",
        "config": {"workload": wl["workload"], "instances": int(wl["n_inst"]), "neurons": n, "synapses": int(nnz),
                   "timesteps_per_step": P, "grid_cells": int(sim.field_cells()),
                   "weights": "U[0, w_b], w_b = 2 * 2.5 nS / (p_b * size_b) per instance",
                   "autotuned": {"threads_per_block": tpb, "neurons_per_thread": npt, "trial_ms_per_step": tune_ms,
                                 "pcg_cells_per_block": cpb, "pcg_trial_ms_per_timestep": pcg_iter_ms,
                                 "pcg_how": "each block size timed over six periods with the batched solve "
                                            "overlapping the neuron updates, from a snapshot restored afterwards"},
                   "network_generation_s": t_gen, "l2": "inputs larger than L2"},
        "spikes_in_timed_region": spikes_b - spikes_a,
        "cg": {"instances": int(wl["n_inst"]), "iterations_last_solve_max": int(iters.max()),
               "iterations_last_solve_median": float(np.median(iters)), "solve_ms": kt.solve_ms},
        # one neuron-update launch per timestep for all instances, replayed from
        # a graph: the timestep's wall time against the launch's own duration
        # (events around each launch) shows what launching costs
        "timestep": {"wall_us": tmax * 1e6 / (args.steps * P), "k_hh_step_mean_us": kt.hh_step_ms * 1e3,
                     "k_hh_step_median_us": hh_ms * 1e3,
                     "solve_us_per_timestep": kt.solve_ms * 1e3 / wl["timescale"]},
        "roofline": {"bound": "hbm", "kernel": "k_hh_step", "achieved": hh_ach, "peak": hbm_peak, "unit": "GB/s",
                     "frac": hh_ach / hbm_peak if hh_ach else None,
                     "traffic": NCU_TRAFFIC_PER_UNIT["hh_step"] * n, "algorithmic_bytes": n * HH_BYTES_PER_NEURON_STEP,
                     "launch_ms": hh_ms, "launch_ms_of": "median launch of the last period of one bench step after the timed region, solves in line",
                     "peak_source": peak_kind},
        "gpu_launches": int(launches),
        "clocks": clock_info,
        "e2e": {"value": e2e_val, "unit": "neuron-steps/s", "h2d_bytes_per_step": 6 * 4 * n,
                "d2h_bytes_per_step": 6 * 4 * n + 8 * 2},
    }
    sim.close()
    ctx.close()
    return line


def cg_problem(wl: dict):
    from neuronephys_clean_gb300 import fields
    g = wl["grid"]
    shape = (g, g, g)
    D = fields.lognormal_diffusivity(shape, wl["sigma"], wl["corr"], seed=1)
    b = fields.spike_sources(shape, wl["neurons"], wl["rate"], seed=2)
    alpha, beta = fields.be_coefficients(g, wl["dt_s"], wl["D0"], wl["uptake"])
    return shape, D, b, alpha, beta


def run_cg(args, wl: dict, dist, rank: int, local_rank: int) -> dict | None:
    """One bench step = one solve of A x = b from x = 0 to a 1e-6 relative
    residual on the 256^3 heterogeneous grid (Jacobi-PCG, single-kernel TMA
    iteration)."""
    import neuronephys_clean_gb300 as nn
    ctx = nn.Context(local_rank)
    shape, D, b, alpha, beta = cg_problem(wl)
    G = int(np.prod(shape))
    dD, db, dx = ctx.to_device(D.ravel()), ctx.to_device(b), ctx.empty((G,), np.float32)
    pc = nn.PCG(ctx, shape[2], shape[1], shape[0], alpha, beta, dD)
    pc.set_kernel_timing(True)
    for _ in range(args.warmup):
        dx.zero()
        pc.solve(db, dx, 1e-6, 20000)
    ctx.synchronize()
    launches0 = ctx.kernel_launches
    clocks = ClockSampler(local_rank)
    barrier(dist)
    clocks.start()
    times, iters, kern_ms, rel = [], [], [], 0.0
    for _ in range(args.steps):
        ctx.time_begin()
        dx.zero()
        it, rel = pc.solve(db, dx, 1e-6, 20000)
        times.append(ctx.time_end())
        ms_k, _ = pc.kernel_time()
        kern_ms.append(ms_k)
        iters.append(it)
    clock_info = clocks.stop()
    barrier(dist)
    launches = ctx.kernel_launches - launches0
    total_ms = sum(times)
    per_solve, tmax = aggregate(1.0, total_ms / 1e3 / args.steps, dist)
    ms_solve = tmax * 1e3
    it_mean = statistics.mean(iters)
    it_ms = statistics.mean(kern_ms) / it_mean
    hbm_peak, peak_kind = measured_peaks()
    ach = G * PCG_HET_BYTES_PER_CELL_ITER / (it_ms * 1e-3) / 1e9
    x = dx.numpy()
    # e2e: rhs from pinned host memory, solution back to pinned host memory
    pin_b = nn.PinnedArray((G,), np.float32)
    pin_x = nn.PinnedArray((G,), np.float32)
    pin_b.array[:] = b
    e2e_s = []
    for _ in range(max(1, args.e2e_steps)):
        t0 = time.perf_counter()
        db.copy_from(pin_b.array)
        dx.zero()
        pc.solve(db, dx, 1e-6, 20000)
        lib_x = dx.numpy()
        pin_x.array[:] = lib_x
        e2e_s.append(time.perf_counter() - t0)
    pin_b.free()
    pin_x.free()
    if rank != 0:
        return None
    line = {
        "metric": "CG time-to-1e-6", "value": ms_solve, "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_solve, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (FP64 reductions)", "data": "synthetic (seeded lognormal D, Poisson sources)",
        "config": {"workload": wl["workload"], "grid": wl["grid"], "alpha": alpha, "beta": beta,
                   "preconditioner": "jacobi", "l2": "inputs larger than L2 (9 x 67 MB vectors)"},
        "cg": {"iterations": it_mean, "relres": rel, "ms_per_iteration": it_ms,
               "solution_norm": float(np.linalg.norm(x.astype(np.float64)))},
        "roofline": {"bound": "hbm", "kernel": "k_cg_iter<HET> (one PCG iteration)", "achieved": ach,
                     "peak": hbm_peak, "unit": "GB/s", "frac": ach / hbm_peak, "traffic": None,
                     "algorithmic_bytes": G * PCG_HET_BYTES_PER_CELL_ITER, "launch_ms": it_ms,
                     "peak_source": peak_kind},
        "gpu_launches": int(launches),
        "clocks": clock_info,
        "e2e": {"value": 1e3 * statistics.mean(e2e_s), "unit": "ms", "h2d_bytes_per_step": 4 * G,
                "d2h_bytes_per_step": 4 * G},
    }
    line["multigrid"] = multigrid_cg(nn, ctx, pc, G, db, ms_solve, it_mean, args)
    line["learned_multigrid"] = learned_multigrid_cg(nn, ctx, pc, wl, shape, G, db, ms_solve, it_mean, args)
    if args.learned:
        line["learned"] = learned_cg(nn, ctx, pc, wl, shape, db, ms_solve, it_mean, args)
    if args.cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_cg(wl, shape, D, b, alpha, beta, wl["fp64_iters"], args.cpu_steps)
    pc.close()
    ctx.close()
    return line


def multigrid_cg(nn, ctx, pc, G, db, plain_ms, plain_iters, args) -> dict:
    """Flexible CG preconditioned by the geometric multigrid V-cycle on the
    same problem, from x = 0 to the same relative residual."""
    mg = nn.MultigridPCG(pc)
    dx = ctx.empty((G,), np.float32)
    for _ in range(max(1, args.warmup)):
        dx.zero()
        mg.solve(db, dx, 1e-6)
    times, its, rel = [], [], 0.0
    for _ in range(args.steps):
        dx.zero()
        ctx.time_begin()
        it, rel = mg.solve(db, dx, 1e-6)
        times.append(ctx.time_end())
        its.append(it)
    levels = mg.levels
    mg.close()
    ms = statistics.mean(times)
    return {"ms_to_tol": ms, "iterations": statistics.mean(its), "relres": rel, "levels": levels,
            "ms_per_iteration": ms / statistics.mean(its), "vs_plain_time": ms / plain_ms,
            "vs_plain_iterations": statistics.mean(its) / plain_iters,
            "solution_norm": float(np.linalg.norm(dx.numpy().astype(np.float64)))}


def learned_multigrid_cg(nn, ctx, pc, wl, shape, G, db, plain_ms, plain_iters, args) -> dict:
    """Multigrid FCG whose 32^3 level (and all below) is solved by the U-Net:
    training pairs from classical solves of fresh right-hand sides, Adam on
    the GPU, then timed solves of the bench right-hand side.  Beside it: the
    classical hierarchy on the same object, and the hierarchy cut at 32^3
    (eight Jacobi sweeps there instead of the levels below)."""
    from neuronephys_clean_gb300 import fields
    level = 3
    lm = nn.LearnedMultigrid(pc, level=level, seed=7)
    t0 = time.perf_counter()
    rhs = [fields.spike_sources(shape, wl["neurons"], wl["rate"], seed=2000 + j) for j in range(wl["train_rhs"])]
    pairs = lm.add_solves(rhs)
    t_pairs = time.perf_counter() - t0
    t0 = time.perf_counter()
    loss = lm.train(wl["lmg_train_steps"], 1e-3)
    t_train = time.perf_counter() - t0
    post_sweeps, _ = lm.autotune_post_sweeps([ctx.to_device(r) for r in rhs])
    dx = ctx.empty((G,), np.float32)

    def timed(solve):
        for _ in range(max(1, args.warmup)):
            dx.zero()
            solve(db, dx)
        times, its, rel = [], [], 0.0
        for _ in range(args.steps):
            dx.zero()
            ctx.time_begin()
            it, rel = solve(db, dx)
            times.append(ctx.time_end())
            its.append(it)
        return statistics.mean(times), statistics.mean(its), rel

    # held-out right-hand sides (seeds disjoint from the training ones)
    test = [ctx.to_device(fields.spike_sources(shape, wl["neurons"], wl["rate"], seed=5000 + j))
            for j in range(args.c5_test_rhs)]

    def test_set(solve) -> dict:
        ms_t, its = [], []
        for h in test:
            dx.zero()
            ctx.time_begin()
            it_h, _ = solve(h, dx)
            ms_t.append(ctx.time_end())
            its.append(it_h)
        return {"right_hand_sides": len(test), "iterations_mean": statistics.mean(its),
                "iterations_max": max(its), "ms_mean": statistics.mean(ms_t)}

    ms, it, rel = timed(lambda b, x: lm.solve(b, x, 1e-6))
    test_learned = test_set(lambda b, x: lm.solve(b, x, 1e-6)) if test else None
    lm.use_network(False)
    ms_c, it_c, _ = timed(lambda b, x: lm.solve(b, x, 1e-6))
    test_classical = test_set(lambda b, x: lm.solve(b, x, 1e-6)) if test else None
    lm.close()
    # the same training with four times the right-hand sides (pairs), judged
    # on the same held-out set
    more = None
    if test and args.c5_more_training:
        lm4 = nn.LearnedMultigrid(pc, level=level, seed=7)
        rhs4 = [fields.spike_sources(shape, wl["neurons"], wl["rate"], seed=2000 + j)
                for j in range(4 * wl["train_rhs"])]
        pairs4 = lm4.add_solves(rhs4)
        loss4 = lm4.train(wl["lmg_train_steps"], 1e-3)
        sweeps4, _ = lm4.autotune_post_sweeps([ctx.to_device(r) for r in rhs4])
        dx.zero()
        lm4.solve(db, dx, 1e-6)  # warm (graph capture)
        more = {"right_hand_sides": len(rhs4), "pairs": pairs4, "final_loss": loss4, "post_sweeps": sweeps4,
                "held_out": test_set(lambda b, x: lm4.solve(b, x, 1e-6))}
        lm4.close()
    test.clear()
    cut = nn.MultigridPCG(pc, level + 1)
    ms_t, it_t, _ = timed(lambda b, x: cut.solve(b, x, 1e-6))
    cut.close()
    return {"ms_to_tol": ms, "iterations": it, "relres": rel, "vs_plain_time": ms / plain_ms,
            "vs_plain_iterations": it / plain_iters, "network_level_grid": shape[0] >> level,
            "post_sweeps": post_sweeps,
            "held_out": test_learned,
            "classical_hierarchy": {"ms_to_tol": ms_c, "iterations": it_c, "held_out": test_classical},
            "cut_at_network_level": {"ms_to_tol": ms_t, "iterations": it_t},
            "training": {"right_hand_sides": len(rhs), "pairs": pairs, "pair_generation_s": t_pairs,
                         "adam_steps": wl["lmg_train_steps"], "train_s": t_train, "final_loss": loss},
            "four_times_the_training_pairs": more}


def learned_cg(nn, ctx, pc, wl, shape, db, plain_ms, plain_iters, args) -> dict:
    """The learned two-grid preconditioner inside flexible CG on the same
    problem: pairs from the plain solver's iterates on fresh right-hand sides,
    Adam training on the GPU, then timed solves of the bench right-hand side."""
    from neuronephys_clean_gb300 import fields
    G = int(np.prod(shape))
    lp = nn.LearnedPreconditioner(pc, seed=7)
    t0 = time.perf_counter()
    rhs = [fields.spike_sources(shape, wl["neurons"], wl["rate"], seed=1000 + j) for j in range(wl["train_rhs"])]
    pairs = lp.add_solver_pairs(rhs)
    ctx.synchronize()
    t_pairs = time.perf_counter() - t0
    t0 = time.perf_counter()
    loss = lp.train(wl["train_steps"], 1e-3)
    t_train = time.perf_counter() - t0
    dx = ctx.empty((G,), np.float32)
    times, its = [], []
    for _ in range(max(1, args.steps // 2)):
        dx.zero()
        ctx.time_begin()
        it, rel = lp.solve(db, dx, 1e-6, 5000)
        times.append(ctx.time_end())
        its.append(it)
    lp.use_network(False)
    dx.zero()
    it_smooth, _ = lp.solve(db, dx, 1e-6, 5000)
    lp.close()
    ms = statistics.mean(times)
    return {"ms_to_tol": ms, "iterations": statistics.mean(its), "relres": rel, "vs_plain_time": ms / plain_ms,
            "vs_plain_iterations": statistics.mean(its) / plain_iters, "iterations_without_network": it_smooth,
            "training": {"pairs": pairs, "pair_generation_s": t_pairs, "adam_steps": wl["train_steps"],
                         "train_s": t_train, "final_loss": loss}}


def cpu_baseline_cg(wl, shape, D, b, alpha, beta, iterations, sample_iters) -> dict:
    """FP64 oracle PCG on the host cores: two bounded runs (k and 4k
    iterations) separate the setup from the per-iteration time, scaled to the
    iteration count of the full solve."""
    import oracle
    G = int(np.prod(shape))
    k = max(1, sample_iters) * 4
    t = []
    for m in (k, 4 * k):
        t0 = time.perf_counter()
        oracle.pcg7(b, np.zeros(G), shape, alpha, beta, D, rtol=1e-30, max_iter=m)
        t.append(time.perf_counter() - t0)
    per_it = (t[1] - t[0]) / (3 * k)
    setup = max(0.0, t[0] - k * per_it)
    ms = 1e3 * (setup + per_it * iterations)
    return {"value": ms, "unit": "ms", "cores": int(oracle.lib().orc_num_threads()), "kind": "port",
            "sample": f"{k} and {4 * k} FP64 PCG iterations on the same {shape[0]}^3 problem "
                      f"(setup {1e3 * setup:.0f} ms, {1e3 * per_it:.1f} ms/iteration), scaled to {iterations:.0f}"}


def run_cg_reference(args, wl: dict, rank: int) -> dict | None:
    if rank != 0:
        return None
    shape, D, b, alpha, beta = cg_problem(wl)
    times = []
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline_cg(wl, shape, D, b, alpha, beta, wl["fp64_iters"], args.cpu_steps)
        if i >= args.warmup:
            times.append(cb["value"])
    ms_solve = statistics.mean(times)
    return {"metric": "CG time-to-1e-6", "value": ms_solve, "unit": "ms", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_solve, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": "synthetic (seeded lognormal D, Poisson sources)",
            "config": {"workload": wl["workload"], "grid": wl["grid"]},
            "cpu_baseline": dict(cb, value=ms_solve),
            "e2e": {"value": ms_solve, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def oracle_network(wl: dict, seed: int):
    """The workload's network, inhibitory flags, drive and voxels from the
    oracle's generators, bit-exact to the device generators (tests
    test_gauss_generator_bit_exact, test_block_generator_bit_exact,
    test_er_generator_bit_exact, test_init_state_drive_and_types)."""
    import oracle
    n = wl["n"]
    if wl["kind"] == "gauss":
        net = oracle.gen_gauss(n, wl["k"], wl["sigma"], wl["w_mu"], wl["w_sigma"], wl["dmax"], seed)
        inh = oracle.inh_flags(n, wl["inh"], True, seed)
    elif wl["kind"] == "block":
        net = oracle.gen_block(n, wl["k"], wl["n_regions"], wl["size_sigma"], wl["density_sigma"], wl["dmax"],
                               wl["w_mu"], wl["w_sigma"], seed)
        inh = oracle.inh_flags(n, wl["inh"], True, seed)
    else:
        net = oracle.gen_er(n, wl["p"], wl["w_max"], seed)
        inh = oracle.inh_flags(n, wl["inh"], False, seed)
    idr = oracle.init_drive(n, seed, wl["i_lo"], wl["i_hi"])
    vox = oracle.voxels(*oracle.lattice_positions(n, seed), wl["grid"]) if wl["grid"] else None
    return net, inh, idr, vox


def run_reference(args, wl: dict, rank: int) -> dict | None:
    """The reference arm: the CPU oracle port of the same workload on the host
    cores (OpenMP over all of them).  It loads no GPU code: the network,
    inhibitory flags, drive and positions come from the oracle's generators,
    bit-exact to the device ones, and the state starts at rest as the GPU
    arm's does.  One timed step is a bounded sample of the workload:
    args.ref_sample_steps timesteps (one paracrine period) of all neurons with
    spike delivery through the delay ring and the deposits, then the period's
    PCG solve of the field (b = u + deposits, warm-started from u).  The
    warm-up samples run on a copy of the initial state and are discarded, so
    the timed samples simulate the workload from its first step; they contain
    its first population burst (all neurons spike within a few ms, ~2 ms after
    the start), the GPU arm's timed region contains later bursts."""
    if rank != 0:
        return None
    import oracle
    seed, n, S = 1, wl["n"], args.ref_sample_steps
    t0 = time.perf_counter()
    net, inh, idr, vox = oracle_network(wl, seed)
    t_gen = time.perf_counter() - t0
    g, D = wl["grid"], max(1, wl["dmax"]) + 1
    dt_s = wl["timescale"] * 0.01 * 1e-3
    alpha, beta = dt_s * wl["par_D"] * g * g, dt_s * wl["par_decay"]

    def new_sim():
        return oracle.Sim(net, inh, idr, seed, D, oracle.rest_state(n), vox=vox, grid_cells=g ** 3 if g else 0)

    def sample(o, u):
        spikes = events = 0
        t = time.perf_counter()
        for _ in range(S):
            sp = o.step()
            spikes += len(sp)
            events += int((net.row_ptr[sp + 1] - net.row_ptr[sp]).sum()) if len(sp) else 0
        if g:
            x, _, _ = oracle.pcg7(u + o.src, u, (g, g, g), alpha, beta, rtol=1e-6)
            u[:] = x
            o.src[:] = 0.0
        return time.perf_counter() - t, spikes, events

    o, u = new_sim(), np.zeros(g ** 3 if g else 0)
    for _ in range(args.warmup):
        sample(o, u)
    o, u = new_sim(), np.zeros(g ** 3 if g else 0)
    times, spikes, events = [], 0, 0
    for _ in range(args.steps):
        dt, sp, ev = sample(o, u)
        times.append(dt)
        spikes += sp
        events += ev
    per_sample = statistics.mean(times)
    value = n * S / per_sample
    cb = {"value": value, "unit": "neuron-steps/s", "cores": int(oracle.lib().orc_num_threads()), "kind": "port",
          "sample": f"{S} timesteps of all {n} neurons (FP64 oracle, OpenMP, spike delivery through the delay ring) "
                    f"+ the period's {g}^3 PCG solve, per timed step; {args.steps} consecutive samples from the "
                    f"initial state ({spikes} spikes, {events} synaptic events); network generation {t_gen:.1f} s "
                    f"untimed"}
    return {"metric": "neuron-steps/s", "value": value, "unit": "neuron-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_sample * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded counter-based generators)", "impl": "reference",
            "config": workload_config(wl, len(net.col), args.delivery),
            "spikes_in_timed_region": spikes, "synaptic_events_per_s": events / sum(times),
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "neuron-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ------------------------------------------- reference kernels on GB300 ---

# slots of the reference's HH struct-of-arrays (src/defines.cuh:57-78)
REF_SOA = ["V", "M", "N", "H", "LOCAL_Y", "IY", "EY", "LOCAL_OUTPUT", "LOCAL_IN", "LOCAL_COUNT",
           "EOUTPUT", "EIN", "ECOUNT", "IOUTPUT", "IIN", "ICOUNT", "APPCUR"]
REFKERN = dict(workload="leapfrog_1M_dt0.4_coupling_count_1M_k100_fire1pct", n=1_000_000, k=100, fire=0.01,
               dt=0.4, reps=20)


def refkern_inputs(seed: int = 3):
    """Shared inputs of the reference-kernel comparison: the reference SoA of
    1M HH neurons in a physiological state (gates at their steady state,
    src/ephys.cu:57-63 rates), and a 1M-neuron network of 100 uniformly random
    out-edges per neuron (int32 CSR, as UniformRandomNetwork builds) with 1 %
    of the neurons firing (output 0.5 > 0.1, the rest 0.05)."""
    w = REFKERN
    n, k = w["n"], w["k"]
    rng = np.random.default_rng(seed)
    V = rng.uniform(-75.0, -40.0, n)
    am = (3.5 + 0.1 * V) / (1 - np.exp(-3.5 - 0.1 * V))
    an = (-0.5 - 0.01 * V) / (np.exp(-5 - 0.1 * V) - 1)
    ah, bm = 0.07 * np.exp(-V / 20 - 3), 4 * np.exp(-(V + 60) / 18)
    bn, bh = 0.125 * np.exp(-(V + 60) / 80), 1 / (np.exp(-3 - 0.1 * V) + 1)
    st = {q: np.zeros(n, np.float32) for q in REF_SOA}
    st["V"], st["M"] = V.astype(np.float32), (am / (am + bm)).astype(np.float32)
    st["N"], st["H"] = (an / (an + bn)).astype(np.float32), (ah / (ah + bh)).astype(np.float32)
    for q in ("LOCAL", "E", "I"):
        cnt = rng.integers(0, 12, n).astype(np.float32)
        st["LOCAL_COUNT" if q == "LOCAL" else f"{q}COUNT"] = cnt
        st["LOCAL_IN" if q == "LOCAL" else f"{q}IN"] = (cnt * rng.uniform(0, 1, n)).astype(np.float32)
    st["APPCUR"] = rng.uniform(0.0, 5.0, n).astype(np.float32)
    idx = rng.integers(0, n, n * k).astype(np.int32)
    off = (np.arange(n + 1, dtype=np.int64) * k).astype(np.int32)
    out = np.full(n, 0.05, np.float32)
    fire = np.sort(rng.choice(n, int(w["fire"] * n), replace=False)).astype(np.int32)
    out[fire] = 0.5
    return [st[q] for q in REF_SOA], idx, off, out, fire


def refkern_line(impl: str, rows: dict) -> dict:
    w = REFKERN
    return {"metric": "reference-semantics kernels on GB300 (leapfrog neuron-steps/s, count-coupling events/s)",
            "impl": impl, "config": {"workload": w["workload"], "neurons": w["n"], "out_degree": w["k"],
                                     "firing_fraction": w["fire"], "dt_ms": w["dt"], "launches_timed": w["reps"]},
            "data": "synthetic (seeded)", **rows}


def run_reference_kernels(args, rank: int) -> dict | None:
    """The reference's own Leapfrog_HH and signal_spikes_kernel (compiled from
    its sources, run by the driver-API harness in oracle/; no product code),
    at the reference's launch shape <<<32, 64>>> (src/defines.cuh:81-82) and on
    a grid that fills the GPU.  The thrust threshold/compaction of
    AtomicCoupling::operator() is host glue the harness does not time: only
    the kernels."""
    if rank != 0:
        return None
    from oracle import refkern
    if not refkern.RefKernels.available():
        return {"impl": "reference", "unavailable": "reference kernel cubins not built (no reference checkout "
                                                    "where oracle/build.py ran)"}
    w = REFKERN
    n, reps = w["n"], w["reps"]
    vars17, idx, off, out, fire = refkern_inputs()
    rk = refkern.RefKernels(0)
    d_vars = [rk.to_device(a) for a in vars17]
    d_table = rk.to_device(np.array(d_vars, np.uint64))
    d_states = rk.zeros(n * refkern.XORWOW_DTYPE.itemsize)
    rk.init_random(0, n, d_states)                       # Ephys::Ephys (src/ephys.cu:20-26)
    full = (n + 255) // 256
    rows = {"leapfrog": {}, "signal_spikes": {}}
    for name, grid, block in (("reference_grid_32x64", 32, 64), ("full_grid", full, 256)):
        rk.leapfrog(d_table, n, w["dt"], d_states, grid=grid, block=block)  # warm
        ms = rk.time_leapfrog(d_table, n, w["dt"], d_states, grid, block, reps)
        rows["leapfrog"][name] = {"grid": grid, "block": block, "ms_per_launch": ms,
                                  "neuron_steps_per_s": n / (ms * 1e-3)}
    d_idx, d_off, d_out, d_fire = rk.to_device(idx), rk.to_device(off), rk.to_device(out), rk.to_device(fire)
    d_in = rk.zeros(4 * n)
    events = len(fire) * w["k"]
    for name, grid, block in (("reference_grid_32x64", 32, 64), ("full_grid", (len(fire) + 63) // 64, 64)):
        rk.signal_spikes(len(fire), d_idx, d_off, d_fire, d_in, d_out, grid=grid, block=block)
        ms = rk.time_signal_spikes(len(fire), d_idx, d_off, d_fire, d_in, d_out, grid, block, reps)
        rows["signal_spikes"][name] = {"grid": grid, "block": block, "ms_per_launch": ms,
                                       "synaptic_events_per_s": events / (ms * 1e-3)}
    return refkern_line("reference", rows)


def run_our_reference_kernels(args, rank: int, local_rank: int) -> dict | None:
    """The library's drop-ins for the same calls on the same inputs:
    nn_hh_leapfrog_step (HHEphys::SimulateEphys; same FP64 rate arithmetic, a
    counter-based noise draw instead of curand) and nn_coupling_run in count
    mode (AtomicCoupling::operator(): zeroing, threshold, ordered compaction
    and the scatter, all timed)."""
    if rank != 0:
        return None
    import neuronephys_clean_gb300 as nn
    w = REFKERN
    n, reps = w["n"], w["reps"]
    vars17, idx, off, out, fire = refkern_inputs()
    ctx = nn.Context(local_rank)
    eph = nn.HHEphys(ctx, n, variant=0, dt=w["dt"])
    assert list(nn.SIM_PARAMS) == REF_SOA
    for q, a in zip(REF_SOA, vars17):
        eph.set(q, a)
    eph.simulate_ephys()
    ctx.time_begin()
    for _ in range(reps):
        eph.simulate_ephys()
    ms = ctx.time_end() / reps
    rows = {"leapfrog": {"k_leapfrog": {"ms_per_launch": ms, "neuron_steps_per_s": n / (ms * 1e-3)}}}
    coup = nn.AtomicCoupling(ctx, n)
    lst = nn.AdjacencyList(ctx.to_device(idx), ctx.to_device(off))
    d_out, d_in = ctx.to_device(out), ctx.empty((n,), np.float32)
    nf = coup(lst, d_in, d_out)
    assert nf == len(fire)
    ctx.time_begin()
    for _ in range(reps):
        coup(lst, d_in, d_out, read_count=False)
    ms = ctx.time_end() / reps
    rows["signal_spikes"] = {"nn_coupling_run": {"ms_per_launch": ms,
                                                 "synaptic_events_per_s": len(fire) * w["k"] / (ms * 1e-3),
                                                 "includes": "zeroing of the inputs, threshold, compaction, scatter"}}
    coup.close()
    ctx.close()
    return refkern_line("ours", rows)


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="c2")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--settle", type=int, default=2000, help="untimed timesteps before the warm-up")
    ap.add_argument("--cpu-steps", type=int, default=3, help="CG workload: FP64 PCG iterations per CPU sample unit")
    ap.add_argument("--parity-steps", type=int, default=50,
                    help="timesteps of the GPU-vs-oracle parity window (and the CPU baseline's sample)")
    ap.add_argument("--ref-sample-steps", type=int, default=100,
                    help="reference arm: timesteps per timed sample (one paracrine period)")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--delivery-sweep", action="store_true",
                    help="time push / pull spike delivery alone over firing fractions (one JSON line)")
    ap.add_argument("--launch-shapes", action="store_true",
                    help="time the workload at every neuron-update launch shape (neurons per thread x threads "
                         "per block; one JSON line)")
    ap.add_argument("--reference-kernels", action="store_true",
                    help="time the reference-semantics leapfrog and count coupling at 1M neurons: the reference's "
                         "own kernels with --impl reference, the library's drop-ins otherwise (one JSON line)")
    ap.add_argument("--electrodes", type=int, default=0,
                    help="record this many KNN electrode regions (50 neurons each), fused into the update")
    ap.add_argument("--delivery", choices=sorted(DELIVERY_MODES), default="auto",
                    help="spike delivery: push, pull, or auto (per period by the measured firing rate)")
    ap.add_argument("--electrode-every", type=int, default=1,
                    help="electrode sampling interval in steps (40 = 0.4 ms, the reference's leapfrog step)")
    ap.add_argument("--no-c4", dest="c4", action="store_false",
                    help="default workload: skip the batched-networks leg")
    ap.add_argument("--no-c5", dest="c5", action="store_false",
                    help="default workload: skip the 256^3 CG time-to-tolerance leg")
    ap.add_argument("--c5-test-rhs", type=int, default=64,
                    help="CG workload: held-out right-hand sides the learned and classical multigrid solve")
    ap.add_argument("--no-c5-more-training", dest="c5_more_training", action="store_false",
                    help="CG workload: skip the learned multigrid trained on four times the pairs")
    ap.add_argument("--no-learned", dest="learned", action="store_false",
                    help="CG workload: skip the learned-preconditioner comparison")
    args = ap.parse_args()
    rank, world, local_rank = dist_env()
    wl = WORKLOADS[args.workload]
    if args.reference_kernels and args.impl == "reference":
        line = run_reference_kernels(args, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if args.impl == "reference":
        if wl.get("kind") == "batch":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the batched workload has no counterpart in "
                                  "the reference and no CPU port here"}), flush=True)
            return
        line = (run_cg_reference if wl.get("kind") == "cg" else run_reference)(args, wl, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if args.warmup < 3:
        args.warmup = 3
    from neuronephys_clean_gb300.build import build
    if rank == 0 or world == 1:
        build()
    dist = dist_init(world)
    barrier(dist)
    if rank != 0:
        build()  # no-op once rank 0 built it
    args.cpu_baseline = args.cpu_baseline and rank == 0 and world == 1
    if args.reference_kernels:
        line = run_our_reference_kernels(args, rank, local_rank)
    elif args.delivery_sweep:
        line = run_delivery_sweep(args, wl, rank, local_rank)
    elif args.launch_shapes:
        line = run_launch_shapes(args, wl, rank, local_rank)
    else:
        runner = {"cg": run_cg, "batch": run_batch}.get(wl.get("kind"), run_ours)
        line = runner(args, wl, dist, rank, local_rank)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
