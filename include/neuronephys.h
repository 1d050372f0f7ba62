/*
 * neuronephys.h -- C ABI of the GB300-native neuronephys simulation path.
 *
 * One process, one GB300 (sm_103a).  Every entry point takes plain pointers
 * and sizes, returns an nn_status (never exits the process), and records a
 * message retrievable with nn_ctx_last_error().  Pointers documented as
 * "device" are CUDA device pointers (cudaMalloc'd by the caller or through
 * nn_malloc); "host" pointers are ordinary host memory.
 *
 * Each block of declarations names the reference interface it replaces
 * (file:line in NingyuanWang/neuronephys_clean).  The C++ adaptor classes in
 * neuronephys.hpp keep the reference's class names and signatures on top of
 * these functions, so a main.cu-style step loop compiles against them.
 *
 * Threading: one nn_ctx per host thread.  All work of a context is ordered on
 * the context's CUDA stream.
 */
#ifndef NEURONEPHYS_H
#define NEURONEPHYS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#define NN_EXTERN extern "C"
#else
#define NN_EXTERN extern
#endif
#define NN_API NN_EXTERN __attribute__((visibility("default")))

/* ------------------------------------------------------------ status ---- */
/* Replaces gpuErrchk/cusparseErrchk's print-and-exit (src/defines.cuh:24-41). */
typedef enum nn_status {
    NN_OK = 0,
    NN_ERR_INVALID_ARG = 1,
    NN_ERR_OOM = 2,
    NN_ERR_CUDA = 3,
    NN_ERR_NOT_CONVERGED = 4,
    NN_ERR_NUMERIC = 5,      /* non-finite neuron state detected on the device */
    NN_ERR_TIMEOUT = 6,      /* a bounded device-side wait gave up */
    NN_ERR_UNSUPPORTED = 7,
    NN_ERR_NO_DEVICE = 8
} nn_status;

NN_API const char* nn_status_string(nn_status s);
NN_API int nn_version(void);

/* ----------------------------------------------------------- context ---- */
typedef struct nn_ctx nn_ctx;
NN_API nn_status nn_ctx_create(int device, nn_ctx** out);
NN_API nn_status nn_ctx_destroy(nn_ctx* ctx);
NN_API const char* nn_ctx_last_error(const nn_ctx* ctx);
NN_API nn_status nn_ctx_synchronize(nn_ctx* ctx);
/* Number of kernels this context has launched (graph replays count their nodes). */
NN_API int64_t nn_ctx_kernel_launches(const nn_ctx* ctx);
/* Streaming multiprocessors of the context's device. */
NN_API int nn_ctx_num_sms(const nn_ctx* ctx);

/* The context's CUDA stream (a cudaStream_t), for callers that interoperate. */
NN_API void* nn_ctx_stream(nn_ctx* ctx);
/* Wall time on the context stream: records a CUDA event now ... */
NN_API nn_status nn_ctx_time_begin(nn_ctx* ctx);
/* ... and here; synchronises and returns the elapsed milliseconds. */
NN_API nn_status nn_ctx_time_end(nn_ctx* ctx, float* ms);
/* Page-locked host memory (cudaMallocHost / cudaFreeHost). */
NN_API nn_status nn_host_alloc(size_t bytes, void** hptr);
NN_API nn_status nn_host_free(void* hptr);

/* Device memory helpers, ordered on the context stream. */
NN_API nn_status nn_malloc(nn_ctx* ctx, size_t bytes, void** dptr);
NN_API nn_status nn_free(nn_ctx* ctx, void* dptr);
NN_API nn_status nn_memcpy_h2d(nn_ctx* ctx, void* dst, const void* src, size_t bytes);
NN_API nn_status nn_memcpy_d2h(nn_ctx* ctx, void* dst, const void* src, size_t bytes);
NN_API nn_status nn_memset_d(nn_ctx* ctx, void* dst, int value, size_t bytes);

/* ============================================================================
 * Reference-semantics primitives (drop-in for the reference's classes)
 * ========================================================================== */

/* SoA slots of the HH sim_vars table (src/defines.cuh:57-78). */
enum {
    NN_HH_V = 0, NN_HH_M = 1, NN_HH_N = 2, NN_HH_H = 3,
    NN_HH_LOCAL_Y = 4, NN_HH_IY = 5, NN_HH_EY = 6,
    NN_HH_LOCAL_OUTPUT = 7, NN_HH_LOCAL_IN = 8, NN_HH_LOCAL_COUNT = 9,
    NN_HH_EOUTPUT = 10, NN_HH_EIN = 11, NN_HH_ECOUNT = 12,
    NN_HH_IOUTPUT = 13, NN_HH_IIN = 14, NN_HH_ICOUNT = 15,
    NN_HH_APPCUR = 16, NN_HH_NUM_VARS = 17
};

/* Constants of the reference HH model: hh_params (src/defines.cuh:87-102) and
 * the whole-brain HH namespace (src_wholebrain/ephys.cuh:45-61). */
typedef struct nn_leapfrog_params {
    float gna, ena, gk, ek, gl, el;
    float Tmax, Vt, Kp, Ar, Ad;
    float g_local, e_local, g_gaba, e_gaba, g_exc, e_exc;
    float noise_mean, noise_intensity;
} nn_leapfrog_params;
/* variant 0: src/ (SCN/cortex benchmarks); 1: src_wholebrain/. */
NN_API void nn_leapfrog_params_reference(nn_leapfrog_params* p, int variant);

/* HHEphys::SimulateEphys(Float** sim_vars) (src/ephys.cu:98-103;
 * src_wholebrain/ephys.cu:219-224): one semi-implicit Crank-Nicolson step of
 * the reference HH model (kernel Leapfrog_HH, src/ephys.cu:28-96).
 * vars: host array of NN_HH_NUM_VARS device pointers, each float[n].
 * Noise: N(0,1) per neuron from the counter-based stream (seed, step); the
 * reference's per-neuron curand XORWOW state is replaced by this stateless
 * stream. */
NN_API nn_status nn_hh_leapfrog_step(nn_ctx* ctx, float* const* vars, int n, float dt,
                                     const nn_leapfrog_params* p, uint64_t seed, uint64_t step);
/* The same step with the noise draws supplied by the caller: d_z (device,
 * float[n]) holds one standard normal per neuron, so that white noise =
 * noise_intensity * z + noise_mean as in src/ephys.cu:88, where z comes from
 * curand_normal on the neuron's XORWOW state.  A caller that keeps the
 * reference's curand stream passes its draws here. */
NN_API nn_status nn_hh_leapfrog_step_z(nn_ctx* ctx, float* const* vars, int n, float dt,
                                       const nn_leapfrog_params* p, const float* d_z);

/* AtomicCoupling (src/coupling.cuh:17-38, src_wholebrain/coupling.cuh:26-43). */
typedef struct nn_coupling nn_coupling;
enum { NN_SIGNAL_COUNT = 0,   /* add 1 per firing presynaptic neuron (src/coupling.cu:46) */
       NN_SIGNAL_OUTPUT = 1   /* add the presynaptic output (src_wholebrain/coupling.cu:31) */ };
NN_API nn_status nn_coupling_create(nn_ctx* ctx, int n, nn_coupling** out);
NN_API nn_status nn_coupling_destroy(nn_coupling* c);
/* AtomicCoupling::operator()(AdjacencyList const&, Float* spikes, Float const*
 * neuron_outputs) (src/coupling.cu:111-141) / PerformCoupling
 * (src_wholebrain/coupling.cu:43-69): inputs[] is zeroed, neurons whose output
 * exceeds 0.1 fire (src/coupling.cu:103-109), their ascending index list is
 * stored, and every CSR entry of a firing row adds the signal to its target.
 * d_indices/d_offsets: device CSR (row = presynaptic).  num_firing (host) may
 * be NULL, which keeps the call free of host synchronisation. */
NN_API nn_status nn_coupling_run(nn_coupling* c, const int* d_indices, const int* d_offsets,
                                 float* d_inputs, const float* d_outputs, int signal_mode,
                                 int* num_firing);
/* AtomicCoupling::operator()(ChunkedAdjacencyList const&, ...)
 * (src/coupling.cu:143-178): chunk c holds target indices local to
 * [c*n_per_chunk, (c+1)*n_per_chunk).  d_chunk_indices/d_chunk_offsets are
 * host arrays of nchunks device pointers.  Equivalent result to
 * nn_coupling_run on the unchunked list, for any n. */
NN_API nn_status nn_coupling_run_chunked(nn_coupling* c, int nchunks, int n_per_chunk,
                                         const int* const* d_chunk_indices,
                                         const int* const* d_chunk_offsets,
                                         float* d_inputs, const float* d_outputs, int* num_firing);
/* GetFiringNeurons() (src/coupling.cuh:37): device pointer to the n-entry
 * buffer whose first num_firing entries are the ascending firing indices
 * (entries beyond keep earlier calls' values, as the reference's do). */
NN_API const int* nn_coupling_firing_list(const nn_coupling* c);
/* Device pointer to the int count of the last call's firing neurons. */
NN_API const int* nn_coupling_firing_count(const nn_coupling* c);

/* Network construction (src/network_factory.cuh:6-67). */
/* UniformRandomNetwork::Generate (src/network_factory.cu:96-131): host-side,
 * bit-identical to the reference's std::default_random_engine (minstd_rand0)
 * + libstdc++ uniform_int_distribution draw.  engine_state is the shared
 * engine (1 = default-constructed, the reference's UnseededRandomEngine,
 * src/defines.cu:4-10) and is advanced in place.  h_indices: n*ncouple ints,
 * h_offsets: n+1 ints. */
NN_API nn_status nn_net_uniform_random(int n, int ncouple, uint32_t* engine_state,
                                       int* h_indices, int* h_offsets);
/* Network::ToAdjacencyList(Float*& Tcount) (src/network_factory.cu:5-27):
 * in-degree of every neuron as float, computed on the device. */
NN_API nn_status nn_net_tcount(nn_ctx* ctx, const int* d_indices, int64_t nnz, int n, float* d_tcount);
/* Network::ToChunkedAdjacencyList (src/network_factory.cu:29-85) on the
 * device.  d_chunk_indices[c] must hold nnz ints and d_chunk_offsets[c] n+1
 * ints (host arrays of device pointers); chunk_nnz (host) receives each
 * chunk's entry count. */
NN_API nn_status nn_net_to_chunked(nn_ctx* ctx, const int* d_indices, const int* d_offsets, int n,
                                   int nchunks, int n_per_chunk, int* const* d_chunk_indices,
                                   int* const* d_chunk_offsets, int64_t* chunk_nnz);

/* ParacrineModule (src/paracrine.cuh:212-267) with the reference's
 * Crank-Nicolson / 27-point compact-Laplacian CG (src/paracrine.cu:19-134)
 * and trilinear scatter/interpolation (src/paracrine.cu:136-296). */
typedef struct nn_paracrine nn_paracrine;
typedef struct nn_paracrine_ref_params {
    int nx, ny, nz;
    float h;              /* spatial_gridsize */
    float D, decay;       /* diffusion_coef, decay_coef */
    float par_dt;         /* solver time step */
    float coup_strength;  /* source added per firing neuron */
    int max_iter;         /* 20 in the reference (src/paracrine.cu:106) */
    float abs_tol;        /* absolute ||r||^2 bound, 1e-6 (src/paracrine.cuh:164) */
    int quirk_rhs;        /* 1: right-hand side uses h where dt belongs (src/paracrine.cu:105) */
    int quirk_firing_list;/* 1: fine update keyed on the compacted list buffer (src/paracrine.cuh:250-252) */
} nn_paracrine_ref_params;
NN_API void nn_paracrine_ref_params_default(nn_paracrine_ref_params* p);
/* ParacrineModule(Float*& d_g_paracrine, N, nx, ny, nz, par_dt, timescale,
 * coup, h, D, decay, x, y, z) (src/paracrine.cuh:230-244).  d_x/d_y/d_z:
 * centred neuron positions (device, float[n]); d_g_paracrine (device,
 * float[n]) receives the interpolated density. */
NN_API nn_status nn_paracrine_ref_create(nn_ctx* ctx, const nn_paracrine_ref_params* p, int n,
                                         const float* d_x, const float* d_y, const float* d_z,
                                         float* d_g_paracrine, nn_paracrine** out);
NN_API nn_status nn_paracrine_destroy(nn_paracrine* pm);
/* update_on_fine_timescale(AtomicCoupling const&) (src/paracrine.cuh:246-253). */
NN_API nn_status nn_paracrine_ref_fine(nn_paracrine* pm, const nn_coupling* c);
/* update_on_own_timescale() (src/paracrine.cuh:255-265): scatter, CN solve,
 * interpolate, reset sources, copy to d_g_paracrine.  iters/final_rr (host)
 * may be NULL. */
NN_API nn_status nn_paracrine_ref_own(nn_paracrine* pm, int* iters, float* final_rr);
/* get_grid().density() (src/paracrine.cuh:266, :170-172): device pointer to
 * the nx*ny*nz density (x fastest). */
NN_API float* nn_paracrine_density(nn_paracrine* pm);
/* Device pointer to the per-neuron source accumulator (float[n]). */
NN_API float* nn_paracrine_sources(nn_paracrine* pm);

/* ============================================================================
 * GB300 simulation step: RK4 Hodgkin-Huxley + weighted, delayed spike delivery
 * + 7-point backward-Euler paracrine field with Jacobi-PCG.
 * The step loop of the reference (_RunAndPrintSimulation, src/main.cu:112-182;
 * MouseCortex::Simulate, src_wholebrain/mouse_cortex.cu:104-120) becomes one
 * device-resident object whose step sequence is captured in a CUDA graph.
 * ========================================================================== */

typedef struct nn_hh_params {
    float C, gNa, gK, gL, ENa, EK, EL;     /* uF/cm^2, mS/cm^2, mV */
    float E_exc, E_inh, tau_exc, tau_inh;  /* synapse reversal (mV) and decay (ms) */
    float v_thresh;                        /* upward-crossing spike threshold (mV) */
    float noise_sigma;                     /* N(0, sigma^2) current per step, uA/cm^2 */
    float dt;                              /* ms */
    float g_par, E_par;                    /* paracrine conductance per unit density, reversal */
} nn_hh_params;
NN_API void nn_hh_params_standard(nn_hh_params* p);

/* Spike delivery (SignalSpikes / signal_spikes_kernel, src/coupling.cu:111-178,
 * is push only).  NN_DELIVERY_AUTO chooses per period of steps: pull when the
 * last measured period fired at least pull_rate of the neurons per step, else
 * push; the spikes in flight are carried across a change of mode. */
enum { NN_DELIVERY_PUSH = 0, NN_DELIVERY_PULL = 1, NN_DELIVERY_AUTO = 2 };

typedef struct nn_sim_config {
    int n;                 /* neurons */
    int max_delay;         /* largest synaptic delay in steps (>= 1) */
    uint64_t seed;         /* master seed of every counter-based stream */
    nn_hh_params hp;
    int delivery;          /* NN_DELIVERY_PUSH, NN_DELIVERY_PULL or NN_DELIVERY_AUTO */
    int64_t raster_capacity; /* spikes recorded as (step, neuron); 0 = off */
    /* paracrine field: grid^3 cells over the unit cube, solved every
     * `timescale` steps with dt_solve = timescale * dt */
    int grid;              /* 0 = no paracrine field */
    int timescale;
    float par_D;           /* diffusivity, (unit cube)^2 / s */
    float par_decay;       /* linear uptake, 1/s */
    double par_rtol;       /* relative residual target */
    int par_max_iter;
    int threads_per_block; /* 0 = autotuned default */
    int neurons_per_thread;/* 1, 2 or 4; 0 = autotuned default */
    int par_overlap;       /* 1 (default): when the field does not feed back (g_par == 0), each period's
                              field solve runs on its own stream, overlapping the next period's steps */
    int par_extrapolate;   /* 1: initial guess 2 u_n - u_(n-1) from the second solve on; 0 (default): u_n.
                              Helps when the sources change slowly; with spike deposits that are new every
                              period it costs iterations (95 -> 103 on the 1M-neuron workload). */
    float pull_rate;       /* NN_DELIVERY_AUTO: spikes per neuron and step at or above which a period runs
                              pull delivery (default 0.025, the crossover measured on the 1M-neuron workload) */
} nn_sim_config;
NN_API void nn_sim_config_default(nn_sim_config* c, int n);

typedef struct nn_sim nn_sim;
NN_API nn_status nn_sim_create(nn_ctx* ctx, const nn_sim_config* cfg, nn_sim** out);
NN_API nn_status nn_sim_destroy(nn_sim* s);

/* Network (CSR, row = presynaptic neuron): host arrays, copied to the device.
 * Replaces Network::ToAdjacencyList + AtomicCoupling construction; the CSC
 * transpose used by pull delivery is built on the device. */
NN_API nn_status nn_sim_set_network(nn_sim* s, const int64_t* h_row_ptr, const int32_t* h_col,
                                    const float* h_weight, const uint8_t* h_delay, int64_t nnz,
                                    const uint8_t* h_is_inh);

/* Counter-based network generators run on the device (replace the host-serial
 * UniformRandomNetwork / NormalNetwork generators, src/network_factory.cu:96-131,
 * src_wholebrain/network_factory.cu:95-138). */
enum { NN_NET_ER = 1, NN_NET_GAUSS = 2, NN_NET_BLOCK = 3 };
typedef struct nn_net_spec {
    int kind;
    double p;              /* ER: connection probability (no self-loops) */
    float w_max;           /* ER: weights U[0, w_max] nS */
    int k;                 /* GAUSS / BLOCK: out-degree per neuron */
    double sigma;          /* GAUSS: kernel standard deviation (unit cube) */
    double w_mu, w_sigma;  /* GAUSS / BLOCK: lognormal weights (nS) */
    int dmax;              /* GAUSS: delays U{1..dmax}; ER: 0 or 1 = delay 1 */
    double inh_fraction;   /* fraction of inhibitory neurons */
    int inh_random;        /* 0: the last fraction of indices; 1: per-neuron draw */
    int n_regions;         /* BLOCK: regions of lognormal size */
    double region_size_sigma, density_sigma;
    int block_dmax;        /* BLOCK: delays 1..block_dmax by centroid distance */
    const double* inst_p;  /* ER on a batch (nn_sim_set_instances): one p per instance, else NULL */
    const float* inst_w_max; /* ER on a batch: one w_max per instance (NULL: w_max for all) */
} nn_net_spec;
NN_API void nn_net_spec_default(nn_net_spec* sp, int kind);
NN_API nn_status nn_sim_generate_network(nn_sim* s, const nn_net_spec* spec);
/* No counterpart in the reference.  A batch of independent networks in one
 * simulation (one launch per step for all of them): instance b owns neurons
 * h_offsets[b] .. h_offsets[b+1]-1 (h_offsets[0] = 0, h_offsets[n_inst] = n).
 * h_grid_sides (nullable) gives each instance its own cubic paracrine grid
 * (the simulation must be created with grid = 0); the fields are solved by
 * the batched PCG, each instance to par_rtol.  Call before generating the
 * network (ER then draws within instances, nn_net_spec.inst_p giving each its
 * p) and before nn_sim_init_state (positions and voxels per instance). */
NN_API nn_status nn_sim_set_instances(nn_sim* s, int n_inst, const int* h_offsets, const int* h_grid_sides);
/* No counterpart in the reference.  Launch-shape autotuner of the neuron
 * update: times trial_steps steps of every (threads per block 64/128/256,
 * neurons per thread 1/2/4) candidate on the simulation's own network and
 * state, keeps the fastest and restores the state the trials touched. */
NN_API nn_status nn_sim_autotune(nn_sim* s, int trial_steps, int* best_tpb, int* best_npt, float* best_ms);
/* Autotuner of the field solver's block shape: for a single grid the z-depth
 * of the 32 x 16 tiles of the one-kernel PCG iteration (4 .. 32;
 * NN_ERR_UNSUPPORTED when the grid runs the two-kernel PCG), for a batch the
 * batched PCG's cells per block.  When the solve overlaps the neuron updates
 * (par_overlap, no field feedback) each shape is timed over six whole periods
 * from a snapshot of the simulation, which is restored afterwards;
 * *ms_per_iter then holds the time per timestep.  Otherwise the solver is
 * timed alone on scratch vectors and *ms_per_iter is its iteration time.
 * *shape: the chosen depth or cells per block. */
NN_API nn_status nn_sim_autotune_solver(nn_sim* s, int trial_iters, int* shape, float* ms_per_iter);
/* Per-instance solver iteration counts of the last paracrine solve (n_inst entries). */
NN_API nn_status nn_sim_instance_iterations(nn_sim* s, int* h_iters);
NN_API nn_status nn_sim_network_size(nn_sim* s, int64_t* nnz);
/* Download the device network (any pointer may be NULL). */
NN_API nn_status nn_sim_get_network(nn_sim* s, int64_t* h_row_ptr, int32_t* h_col, float* h_weight,
                                    uint8_t* h_delay, uint8_t* h_is_inh);
/* Download the device CSC (columns = postsynaptic; within a column, entries
 * in ascending CSR position). */
NN_API nn_status nn_sim_get_csc(nn_sim* s, int64_t* h_col_ptr, int32_t* h_src, float* h_weight,
                                uint8_t* h_delay);

/* Per-neuron fields. */
enum { NN_F_V = 0, NN_F_M, NN_F_H, NN_F_N, NN_F_GE, NN_F_GI, NN_F_IDRIVE, NN_F_GNA_SCALE,
       NN_F_X, NN_F_Y, NN_F_Z, NN_F_UPAR, NN_F_COUNT };
NN_API nn_status nn_sim_set_field(nn_sim* s, int field, const float* h_values);
NN_API nn_status nn_sim_get_field(nn_sim* s, int field, float* h_values);
/* Device pointer of a field (for zero-copy callers). */
NN_API float* nn_sim_field_ptr(nn_sim* s, int field);
/* Default initial state: V = v0, gates at their steady state, synapses 0,
 * drive I ~ U[i_lo, i_hi] from the seed, positions on the jittered lattice. */
NN_API nn_status nn_sim_init_state(nn_sim* s, float v0, float i_lo, float i_hi);

/* Advance nsteps on the device (no host synchronisation). */
NN_API nn_status nn_sim_step(nn_sim* s, int nsteps);
/* Deliver an explicit list of spiking neurons (device int array, current
 * step) through the network: mode NN_DELIVERY_PUSH scatters their out-edges
 * into the delay ring as the step kernel does; NN_DELIVERY_PULL (simulation
 * created in pull mode) sets them in the current step's bitmap and runs the
 * CSC gather of the next step's input, for measuring the gather (the next
 * nn_sim_step recomputes that input from the simulation's own spikes).  The
 * reference's counterpart is
 * AtomicCoupling::operator() given a firing list (src/coupling.cu:103-141);
 * here it serves callers with spikes from elsewhere and measurement of the
 * delivery path alone.  Asynchronous on the context stream. */
NN_API nn_status nn_sim_deliver_spikes(nn_sim* s, const int* d_list, int count, int mode);
/* Pull delivery layout of a pull-mode simulation: *sliced = 1 when the
 * shared-memory kernel over the delay-sliced CSC runs (bitmap of one step in
 * shared memory; *cols = columns per block), 0 for the warp-per-column
 * kernel.  No counterpart in the reference. */
NN_API nn_status nn_sim_pull_info(nn_sim* s, int* sliced, int* cols);
/* The pull gather alone, from the spike bitmap as it stands (for example
 * after nn_sim_deliver_spikes with NN_DELIVERY_PULL): the input of the next
 * step rewritten.  For timing the gather kernel by itself; asynchronous. */
NN_API nn_status nn_sim_pull_gather(nn_sim* s);
/* NN_DELIVERY_AUTO: the delivery mode of each period run since the last call
 * with reset != 0 (0 push, 1 pull) and the firing rate that chose it (spikes
 * per neuron and step of the latest period measured when it was enqueued;
 * -1 before the first measurement).  Up to cap entries are written, *count
 * receives the number of periods logged. */
NN_API nn_status nn_sim_delivery_log(nn_sim* s, int8_t* h_modes, float* h_rates, int cap, int* count, int reset);
/* NN_DELIVERY_AUTO: change the pull threshold (config field pull_rate) for the
 * periods enqueued from now on. */
NN_API nn_status nn_sim_set_pull_rate(nn_sim* s, float pull_rate);
/* End-to-end call: copy the state (6*n floats: V,m,h,n,ge,gi planes) from
 * host memory, advance nsteps, copy the state back and return the number of
 * spikes emitted. */
NN_API nn_status nn_sim_run_host(nn_sim* s, const float* h_state_in, int nsteps, float* h_state_out,
                                 int64_t* h_spikes);
/* Current step index and total spikes so far (synchronises). */
NN_API nn_status nn_sim_counters(nn_sim* s, int64_t* step, int64_t* total_spikes);
/* ElectrodeNet (src/electrode_net.cu:3-49; src_wholebrain/electrode_net.cu:3-54),
 * fused into the step: regions as ElectrodeNet takes them (h_indices: the
 * neurons of each region, h_offsets[n_regions + 1]; regions may overlap).
 * On every step t with t % every == 0 (from the next such step on) the neuron
 * update records the new membrane potential and the spike of step t of every
 * neuron listed in a region; nn_sim_read_electrodes turns them into each
 * region's mean potential (FP64 sum) and firing count after that step, as
 * DoElectrodeMeasurements computes them.  Samples are kept in a ring of
 * `capacity` slots (the oldest are overwritten).  every = 0 turns the
 * recording off. */
NN_API nn_status nn_sim_set_electrodes(nn_sim* s, const int* h_indices, const int* h_offsets, int n_regions,
                                       int every, int capacity);
/* The recorded samples, oldest first: h_avg / h_firing (host, [capacity]
 * [n_regions], either may be NULL) get mean potentials and firing counts,
 * *first_step the step of the first returned sample, *n_samples their number. */
NN_API nn_status nn_sim_read_electrodes(nn_sim* s, float* h_avg, int* h_firing, int64_t* first_step,
                                        int* n_samples);
/* Download the delay ring: D = max_delay + 1 slots of n (excitatory,
 * inhibitory) input pairs, h_ring float[D * n * 2]; slot (t mod D) holds the
 * input the neurons take at step t.  With the step counter and the neuron
 * fields it is the complete state a step depends on.  No counterpart in the
 * reference (its inputs have a one-step delay and live in the SoA table). */
NN_API nn_status nn_sim_get_ring(nn_sim* s, float* h_ring);
/* Restart the spike raster: the next recorded spike is entry 0 again. */
NN_API nn_status nn_sim_reset_raster(nn_sim* s);
/* Recorded raster (ascending (step, neuron) after sorting on the host). */
NN_API nn_status nn_sim_get_raster(nn_sim* s, int64_t cap, int32_t* h_step, int32_t* h_neuron,
                                   int64_t* count);
/* Paracrine density (grid^3 floats, x fastest) and last solve statistics. */
NN_API nn_status nn_sim_get_density(nn_sim* s, float* h_u);
NN_API nn_status nn_sim_set_density(nn_sim* s, const float* h_u);
/* Cells of the paracrine field (grid^3, or the sum over a batch's grids) and
 * the field cell of every neuron's deposits (n entries). */
NN_API nn_status nn_sim_field_cells(nn_sim* s, int64_t* cells);
NN_API nn_status nn_sim_get_vox(nn_sim* s, int32_t* h_vox);
typedef struct nn_solve_stats { int iterations; double relres; int solves; int converged; } nn_solve_stats;
NN_API nn_status nn_sim_solve_stats(nn_sim* s, nn_solve_stats* st);
/* Kernel timing: when enabled, CUDA events bracket every neuron-update and
 * delivery launch (also inside the captured graph) and every paracrine solve's
 * iterations.  nn_sim_kernel_times returns the mean durations (ms) over the
 * launches of the most recent graph replay / eager steps and the last solve. */
NN_API nn_status nn_sim_set_kernel_timing(nn_sim* s, int enable);
typedef struct nn_kernel_times {
    float hh_step_ms;      /* mean k_hh_step duration */
    float deliver_ms;      /* mean delivery-kernel duration */
    int samples;           /* launches averaged */
    float solve_ms;        /* last paracrine solve, all iterations */
    int solve_iterations;
    float hh_step_median_ms;   /* median k_hh_step duration (a step without a burst of spikes) */
    float deliver_median_ms;   /* median delivery-kernel duration */
} nn_kernel_times;
NN_API nn_status nn_sim_kernel_times(nn_sim* s, nn_kernel_times* out);

/* ============================================================================
 * Standalone 7-point Jacobi-PCG (backward-Euler diffusion with uptake).
 * A = (1 + beta) I + alpha * L_D, L_D the 7-point operator with harmonic-mean
 * face coefficients of the cell field Dcell (or 1 when Dcell is NULL), zero
 * values outside the grid.  Vectors FP32; dot products and norms FP64.
 * ========================================================================== */
typedef struct nn_pcg nn_pcg;
NN_API nn_status nn_pcg_create(nn_ctx* ctx, int nx, int ny, int nz, double alpha, double beta,
                               const float* d_Dcell, nn_pcg** out);
NN_API nn_status nn_pcg_destroy(nn_pcg* pc);
/* y = A x (device vectors). */
NN_API nn_status nn_pcg_apply(nn_pcg* pc, const float* d_x, float* d_y);
/* Solve A x = b to ||r|| <= rtol ||b||; d_x holds the initial guess. */
NN_API nn_status nn_pcg_solve(nn_pcg* pc, const float* d_b, float* d_x, double rtol, int max_iter,
                              int* iters, double* relres);
/* No counterpart in the reference (it has no timing hooks).  With timing on,
 * each solve brackets its iteration kernels with CUDA events;
 * nn_pcg_kernel_time returns their total (ms) and the iteration count of
 * the last solve. */
NN_API nn_status nn_pcg_set_kernel_timing(nn_pcg* pc, int enable);
NN_API nn_status nn_pcg_kernel_time(nn_pcg* pc, float* ms, int* iters);

/* No counterpart in the reference.  Batched Jacobi-PCG for the per-instance
 * paracrine fields of a batch of networks: n_inst independent cubic grids of
 * sides h_sides[b] (cells concatenated in instance order, x fastest), operator
 * (1 + beta) I + alpha_unit * side_b^2 * L (alpha_unit = dt * D on the unit
 * cube), each instance solved to its own relative residual rtol; converged
 * instances stop costing work.  h_iters (nullable): n_inst iteration counts;
 * *unconverged: instances that stopped short of rtol. */
typedef struct nn_bpcg nn_bpcg;
NN_API nn_status nn_bpcg_create(nn_ctx* ctx, int n_inst, const int* h_sides, double alpha_unit, double beta,
                                nn_bpcg** out);
NN_API nn_status nn_bpcg_destroy(nn_bpcg* bp);
NN_API nn_status nn_bpcg_solve(nn_bpcg* bp, const float* d_b, float* d_x, double rtol, int max_iter, int* h_iters,
                               int* max_iters, int* unconverged);
/* Block-size autotuner: times iterations with 512, 1,024, 2,048 and 4,096
 * cells per block (2, 4, 8, 16 per thread) on the batch's own operators,
 * right-hand side d_b and d_x as scratch (overwritten), and keeps the fastest
 * layout for later solves. */
NN_API nn_status nn_bpcg_autotune(nn_bpcg* bp, const float* d_b, float* d_x, int trial_iters, int* cells_per_block,
                                  float* ms_per_iter);
/* Fix the block layout instead: 512, 1024, 2048 (the default) or 4096 cells per block. */
NN_API nn_status nn_bpcg_set_cells_per_block(nn_bpcg* bp, int cells_per_block);

/* No counterpart in the reference.  The same solve as nn_pcg_create +
 * nn_pcg_solve + nn_pcg_destroy for callers that may not allocate device
 * memory: a host framework that owns the GPU's memory budget and forbids
 * allocations by the code it calls, or a real-time loop that cannot take the
 * device-wide synchronisation of cudaMalloc/cudaFree.  It allocates nothing:
 * its work vectors and reduction scratch live in one fixed device array of
 * about 5.4 MB that every GPU loading this library holds until the process
 * exits.  The caller passes the inputs (d_Dcell may be NULL, d_b) and the
 * output d_x (initial guess in, solution out), all device pointers, and the
 * cudaStream_t to run on (NULL = the legacy default stream).
 * Limit: nx*ny*nz <= NN_PCG_NOALLOC_MAX_CELLS (64^3); larger grids return
 * NN_ERR_UNSUPPORTED without launching anything.  Returns NN_ERR_NOT_CONVERGED
 * if rtol is not reached in max_iter iterations.
 * The first call on a device looks up the scratch's device address (which
 * also loads the library's kernels on that device) and keeps it for the
 * process: make that first call before any stream capture, and do not call
 * this entry point on a device after cudaDeviceReset there (the kept address
 * would belong to the context the reset destroyed).  Each process has its
 * own scratch; within a process, all calls on a device share the one
 * scratch, so calls whose work overlaps on the GPU (from different streams or
 * host threads) race: serialise them.  The call synchronises the caller's
 * stream at each convergence check.  Only the status code reports a failure:
 * no message is kept (there is no context to keep it in). */
#define NN_PCG_NOALLOC_MAX_CELLS (64 * 64 * 64)
NN_API nn_status nn_pcg_solve_noalloc(void* stream, int nx, int ny, int nz, double alpha, double beta,
                                      const float* d_Dcell, const float* d_b, float* d_x, double rtol,
                                      int max_iter, int* iters, double* relres);


/* ==========================================================================
 * Learned preconditioner building blocks (no counterpart in the reference).
 * Activations use a zero-padded, channel-blocked BF16 layout (nn_act_layout
 * gives the bytes of a tensor with `channels` channels on an nz x ny x nx
 * grid; channels a multiple of 8).  3x3x3 "same" convolutions run on the
 * tensor cores with FP32 accumulation.  Weights are FP32 w[27][cin][cout]
 * (tap = (dz+1)*9 + (dy+1)*3 + dx+1) packed to BF16 by
 * nn_conv3d_pack_weights; with adjoint set the packed operator is the
 * input-gradient convolution (taps mirrored, cin and cout exchanged), run by
 * nn_conv3d_forward with the channel counts exchanged.  Supported
 * (cin, cout): (16,16) (16,32) (32,32) (32,64) (64,64) (96,32) (48,16) and
 * their exchanges.
 * ========================================================================== */
NN_API nn_status nn_act_layout(int nz, int ny, int nx, int channels, int64_t* block_stride, int64_t* guard,
                               int64_t* bytes);
/* dense FP32 [channels][nz][ny][nx] <-> padded BF16 activation (the
 * activation's pads must be zero: allocate with nn_malloc + nn_memset_d). */
NN_API nn_status nn_act_pack(nn_ctx* ctx, int nz, int ny, int nx, int channels, const float* d_dense, void* d_act);
NN_API nn_status nn_act_unpack(nn_ctx* ctx, int nz, int ny, int nx, int channels, const void* d_act,
                               float* d_dense);
/* d_packed: 27 * cin * cout * 2 bytes, 16-byte aligned. */
NN_API nn_status nn_conv3d_pack_weights(nn_ctx* ctx, int cin, int cout, const float* d_w, int adjoint,
                                        void* d_packed);
/* y = relu?(conv(x) + bias), then zeroed where d_mask (same layout as y,
 * nullable) is <= 0; d_bias and d_y32 (dense FP32 copy of channel 0) nullable.
 * Synchronises; NN_ERR_TIMEOUT if a pipeline wait gave up. */
NN_API nn_status nn_conv3d_forward(nn_ctx* ctx, int nz, int ny, int nx, int cin, int cout, const void* d_x,
                                   const void* d_wpacked, const float* d_bias, int relu, const void* d_mask,
                                   void* d_y, float* d_y32);
/* d_dw[27][cin][cout] += sum_o x(o + tap) gy(o); d_db[cout] += sum_o gy(o)
 * (nullable).  FP32 accumulation. */
NN_API nn_status nn_conv3d_wgrad(nn_ctx* ctx, int nz, int ny, int nx, int cin, int cout, const void* d_x,
                                 const void* d_gy, float* d_dw, float* d_db);


/* Geometric multigrid for the 7-point operator of an nn_pcg (no counterpart
 * in the reference).  Cell-centred hierarchy (2x per axis while the sides stay
 * even; levels = 0 picks the depth that leaves about 16^3 coarsest cells),
 * 7-point coarse operators from the fine conductances, damped-Jacobi
 * smoothing, trilinear prolongation.  nn_mg_apply runs one V-cycle (z = M r);
 * nn_mg_solve runs flexible CG preconditioned by one V-cycle per iteration
 * to the same relative residual as nn_pcg_solve (x holds the initial guess;
 * NN_ERR_NOT_CONVERGED after max_iter iterations).  The nn_pcg (and its cell
 * field) must outlive the nn_mg. */
typedef struct nn_mg nn_mg;
NN_API nn_status nn_mg_create(nn_pcg* pc, int levels, nn_mg** out);
NN_API nn_status nn_mg_destroy(nn_mg* mg);
NN_API nn_status nn_mg_levels(nn_mg* mg, int* levels);
NN_API nn_status nn_mg_apply(nn_mg* mg, const float* d_r, float* d_z);
NN_API nn_status nn_mg_solve(nn_mg* mg, const float* d_b, float* d_x, double rtol, int max_iter, int* iters,
                             double* relres);

/* Multigrid with a learned coarse-level solver (no counterpart in the
 * reference).  The geometric hierarchy of nn_mg_create in which one coarse
 * level (level >= 1; its sides multiples of 4) and everything below it are
 * replaced by the 3D conv U-Net of the learned preconditioner: the level's
 * right-hand side b goes in divided by its RMS, together with the log of the
 * level's diagonal; the output times that RMS is the level's correction,
 * followed by the V-cycle's post-smoothing there.  nn_lmg_add_solve solves
 * A x = b with the classical hierarchy from x = 0 (d_x receives the solution)
 * and stores, for every V-cycle, the right-hand side that reached the level
 * and its solution on that level as a training pair (*pairs_added);
 * nn_lmg_train runs Adam steps over the stored pairs; nn_lmg_solve runs
 * flexible CG to the same relative residual as nn_pcg_solve.
 * nn_lmg_use_network(lm, 0) switches back to the classical hierarchy, for
 * comparisons.  The nn_pcg (and its cell field) must outlive the nn_lmg. */
typedef struct nn_lmg nn_lmg;
NN_API nn_status nn_lmg_create(nn_pcg* pc, int level, uint64_t seed, nn_lmg** out);
NN_API nn_status nn_lmg_destroy(nn_lmg* lm);
NN_API nn_status nn_lmg_add_solve(nn_lmg* lm, const float* d_b, float* d_x, int* pairs_added);
NN_API nn_status nn_lmg_pairs(nn_lmg* lm, int* n);
NN_API nn_status nn_lmg_train(nn_lmg* lm, int steps, float lr, float* mean_loss);
NN_API nn_status nn_lmg_use_network(nn_lmg* lm, int enable);
/* Jacobi sweeps on the network's level after its correction (default 2). */
NN_API nn_status nn_lmg_set_post_sweeps(nn_lmg* lm, int sweeps);
/* Choose that number (2, 4, 8, 12, 16, 20 or 24) by timing, for each, solves of the
 * nb right-hand sides d_bs[k] (host array of device pointers) from zero to
 * rtol (d_x: scratch); the smallest total is kept, *best_ms. */
NN_API nn_status nn_lmg_autotune_post_sweeps(nn_lmg* lm, const float* const* d_bs, int nb, float* d_x, double rtol,
                                             int* best, float* best_ms);
NN_API nn_status nn_lmg_solve(nn_lmg* lm, const float* d_b, float* d_x, double rtol, int max_iter, int* iters,
                              double* relres);

/* Learned two-grid preconditioner for the 7-point operator of an nn_pcg
 * (grid sides multiples of 8): Jacobi smoothing on the fine grid and a
 * coarse-grid correction by a 3-level 3D conv U-Net (16/32/64 channels, BF16
 * tensor-core convolutions) on the 2x coarser grid, inside flexible CG.
 * Training data: nn_learned_add_pair(r, e) with A e = r on the fine grid
 * (e.g. r = b - A x_k and e = x* - x_k from any solve); nn_learned_train
 * runs Adam steps over the stored pairs.  nn_learned_solve iterates to the
 * same relative residual as nn_pcg_solve.  The nn_pcg (and its cell field)
 * must outlive the nn_learned. */
typedef struct nn_learned nn_learned;
NN_API nn_status nn_learned_create(nn_pcg* pc, uint64_t seed, nn_learned** out);
NN_API nn_status nn_learned_destroy(nn_learned* lp);
NN_API nn_status nn_learned_add_pair(nn_learned* lp, const float* d_r, const float* d_e);
NN_API nn_status nn_learned_train(nn_learned* lp, int steps, float lr, float* mean_loss);
/* z = M r (device vectors of the fine grid). */
NN_API nn_status nn_learned_apply(nn_learned* lp, const float* d_r, float* d_z);
/* 0: leave the network out of M (smoothing only), for comparisons. */
NN_API nn_status nn_learned_use_network(nn_learned* lp, int enable);
NN_API nn_status nn_learned_solve(nn_learned* lp, const float* d_b, float* d_x, double rtol, int max_iter,
                                  int* iters, double* relres);
/* Parameters as one flat FP32 host vector (per layer w[27][cin][cout], b[cout]). */
NN_API nn_status nn_learned_num_params(nn_learned* lp, int64_t* n);
NN_API nn_status nn_learned_get_params(nn_learned* lp, float* h_out);
NN_API nn_status nn_learned_set_params(nn_learned* lp, const float* h_in);
/* Gradient check: forward + backward of the network on a coarse-grid input
 * d_rc and target d_target; loss = 0.5 sum (y - t/s)^2 (s = rms of d_rc),
 * parameter gradients to h_grad (flat order), network output y to d_y
 * (both nullable).  No parameter update. */
NN_API nn_status nn_learned_net_gradient(nn_learned* lp, const float* d_rc, const float* d_target, float* h_grad,
                                         double* loss, float* d_y);


/* ==========================================================================
 * Consumers of the step (reference: ElectrodeNet, SynchronyNet, Hebbian).
 * ========================================================================== */
/* ElectrodeNet(regions_inds, regions_offsets) (src/electrode_net.cuh:8-24,
 * src_wholebrain/electrode_net.cuh:9-29): regions as index lists. */
typedef struct nn_electrodes nn_electrodes;
NN_API nn_status nn_electrodes_create(nn_ctx* ctx, const int* h_indices, const int* h_offsets, int n_regions,
                                      nn_electrodes** out);
NN_API nn_status nn_electrodes_destroy(nn_electrodes* e);
/* DoElectrodeMeasurements(V, is_firing) (src_wholebrain/electrode_net.cu:33-48):
 * per-region mean of d_V and, if d_is_firing (int per neuron) is given, the
 * firing count; copied to h_avg / h_firing when those are non-NULL. */
NN_API nn_status nn_electrodes_measure(nn_electrodes* e, const float* d_V, const int* d_is_firing, float* h_avg,
                                       int* h_firing);
/* MeasureAverageEntireNetwork(V, N) (src/electrode_net.cu:46-49). */
NN_API nn_status nn_measure_average(nn_ctx* ctx, const float* d_V, int n, float* out);
/* SynchronyNet (src_wholebrain/electrode_net.cuh:33-60, .cu:56-124). */
typedef struct nn_synchrony nn_synchrony;
NN_API nn_status nn_synchrony_create(nn_ctx* ctx, const int* h_region_inds, int n_inds, const int* h_sub_counts,
                                     int n_sub, nn_synchrony** out);
NN_API nn_status nn_synchrony_destroy(nn_synchrony* s);
NN_API nn_status nn_synchrony_measure(nn_synchrony* s, const float* d_V);  /* MeasureVariances */
NN_API nn_status nn_synchrony_get(nn_synchrony* s, double* h_chi);        /* GetSynchronyMeasures */
/* Hebbian(window, inc, Nconns) (src_wholebrain/hebbian.cuh:3-23). */
typedef struct nn_hebbian nn_hebbian;
NN_API nn_status nn_hebbian_create(nn_ctx* ctx, int window, float inc, int64_t nconns, int n_neurons,
                                   nn_hebbian** out);
NN_API nn_status nn_hebbian_destroy(nn_hebbian* h);
/* UpdateWeights(connectivity, is_firing, firing_inds) (src_wholebrain/hebbian.cu:53-69):
 * CSR (row = presynaptic) indices / offsets, int is_firing per neuron, the
 * list of num_firing neurons whose synapse timers are set, weights updated
 * in place.  Asynchronous on the context stream. */
NN_API nn_status nn_hebbian_update(nn_hebbian* h, const int* d_indices, const int* d_offsets,
                                   const int* d_is_firing, const int* d_firing_inds, int num_firing,
                                   float* d_weights);
NN_API nn_status nn_hebbian_timers(nn_hebbian* h, int* h_timers);


/* ==========================================================================
 * On-disk inputs (reference: FileNetwork, src/network_factory.cu:154-211;
 * FileMorphology, src/morphology.cpp:260-330).  The reference reads HDF5
 * datasets /row_ptr, /col_idx (int32) and /x, /y, /z (float32); with no HDF5
 * library here the same datasets travel in a raw little-endian container:
 *   "NNCSR001" | int64 n_rows | int64 nnz | int32 row_ptr[n_rows+1] | int32 col_idx[nnz]
 *   "NNPOS001" | int64 n | float32 x[n] | float32 y[n] | float32 z[n]
 * The *_read calls return the sizes when the arrays are NULL.
 * ========================================================================== */
NN_API nn_status nn_net_file_write(const char* path, int64_t n_rows, int64_t nnz, const int32_t* h_row_ptr,
                                   const int32_t* h_col);
NN_API nn_status nn_net_file_read(const char* path, int64_t* n_rows, int64_t* nnz, int32_t* h_row_ptr,
                                  int32_t* h_col);
/* FileNetwork::Generate(N): keep rows i * sparsity (sparsity = n_rows / N)
 * and their targets divisible by sparsity, renumbered target / sparsity, in
 * file order.  Device arrays in and out; d_out_col needs the input nnz. */
NN_API nn_status nn_net_subsample(nn_ctx* ctx, const int32_t* d_row_ptr, const int32_t* d_col, int64_t n_rows,
                                  int N, int64_t* d_out_row_ptr, int32_t* d_out_col, int64_t* out_nnz);
NN_API nn_status nn_positions_file_write(const char* path, int64_t n, const float* h_x, const float* h_y,
                                         const float* h_z);
NN_API nn_status nn_positions_file_read(const char* path, int64_t* n, float* h_x, float* h_y, float* h_z);
/* FileMorphology::Generate(N): points stride * i (stride = n / N), mapped by
 * the bounding box of all n points onto [-1, 1] (FP32, the reference's
 * operation order). */
NN_API nn_status nn_positions_subsample(nn_ctx* ctx, const float* d_x, const float* d_y, const float* d_z,
                                        int64_t n, int N, float* d_ox, float* d_oy, float* d_oz);


/* NormalNetwork(morphology, stddev, n_stddevs).Generate(N)
 * (src_wholebrain/network_factory.cu:95-138) on the device: neuron i couples
 * to every j within n_stddevs * stddev with probability
 * exp(-|x_i - x_j|^2 / (2 stddev^2)); counter-based draws per pair (the
 * reference draws from its unseeded engine in kd-tree order: same
 * distribution, other edges).  d_offsets (n + 1) is always written; with
 * d_indices non-NULL and capacity >= *nnz the targets are written too. */
NN_API nn_status nn_net_local_gaussian(nn_ctx* ctx, int n, const float* d_x, const float* d_y, const float* d_z,
                                       float stddev, int n_stddevs, uint64_t seed, int* d_offsets, int* d_indices,
                                       int64_t capacity, int64_t* nnz);

#endif
