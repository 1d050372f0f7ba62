/*
 * oracle.h -- CPU restatement of the neuronephys per-timestep simulation path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code; it is used by tests/, by __graft_entry__.smoke() as the
 * checker, and by bench.py's CPU baseline leg.
 *
 * Two families of functions live here:
 *
 *  REFERENCE semantics (restated from the reference sources, cited file:line
 *  relative to the reference project root):
 *    - std::minstd_rand0 + libstdc++ uniform_int_distribution and the
 *      UniformRandomNetwork generator            src/network_factory.cu:96-131
 *    - in-degree Tcount / chunked adjacency list src/network_factory.cu:5-85
 *    - Leapfrog_HH (FP64 rate arithmetic, as the reference's double literals
 *      promote it)                                src/ephys.cu:28-96
 *    - AtomicCoupling threshold + compaction + push
 *                                                 src/coupling.cu:34-48,103-178
 *                                                 src_wholebrain/coupling.cu:12-33,43-69
 *    - paracrine trilinear scatter/interpolate, 27-point compact Laplacian,
 *      Crank-Nicolson CG                          src/paracrine.cu:19-296
 *
 *  Parity pinning: the network-factory functions are pinned bit-exactly to
 *  golden vectors produced by running the reference's own host code
 *  (tests/golden/).  Leapfrog_HH, the coupling push and the paracrine solver
 *  are CUDA/ArrayFire code in the reference that cannot execute in this
 *  container; their restatements are checked against the reference's
 *  in-code identities (stencil sum, mass conservation) and are otherwise
 *  "parity unpinned" against the reference itself.
 *
 *  Model semantics of the GB300 build (RK4 Hodgkin-Huxley with standard
 *  parameters, exponential conductance synapses with integer delays,
 *  7-point backward-Euler diffusion with Jacobi-PCG, counter-based network
 *  generators).  These have no counterpart in the reference (it has no RK4
 *  HH, no weighted/delayed synapses and no 7-point solver) and are FP64
 *  oracles of the same algorithms the CUDA kernels run.
 */
#ifndef NN_ORACLE_H
#define NN_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ RNG -- */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void orc_philox2x32_10(const uint32_t ctr[2], uint32_t key, uint32_t out[2]);
/* Standard normal of neuron i at a step: one Philox draw per neuron pair,
 * counter (i>>1, step, step>>32, purpose), Box-Muller with the cos branch for
 * even i and the sin branch for odd i. */
double orc_normal_ctr(uint64_t seed, uint32_t i, uint64_t step, uint32_t purpose);

/* std::minstd_rand0 (libstdc++ std::default_random_engine): x <- 16807 x mod (2^31-1). */
uint32_t orc_minstd_next(uint32_t* state);
/* libstdc++ std::uniform_int_distribution<int>(a, b) drawing from minstd_rand0. */
int orc_uniform_int(uint32_t* state, int a, int b);

/* ------------------------------------------- reference network factory -- */
/* UniformRandomNetwork::Generate (src/network_factory.cu:96-131).
 * indices: n*ncouple ints, offsets: n+1 ints.  *engine is the shared engine
 * state (1 = freshly default-constructed), advanced in place. */
void orc_uniform_random_network(int n, int ncouple, uint32_t* engine, int* indices, int* offsets);
/* Tcount = in-degree as float (src/network_factory.cu:19-22). */
void orc_tcount(const int* indices, int64_t nnz, int n, float* tcount);
/* ToChunkedAdjacencyList split (src/network_factory.cu:45-63):
 * chunk c gets local index (idx % n_per_chunk) of every edge with
 * idx / n_per_chunk == c.  chunk_indices[c] must hold nnz ints,
 * chunk_offsets[c] n+1 ints; chunk_nnz[c] receives the count. */
void orc_chunked(const int* indices, const int* offsets, int n, int nchunks, int n_per_chunk,
                 int** chunk_indices, int** chunk_offsets, int64_t* chunk_nnz);

/* --------------------------------------------------- reference ephys ---- */
/* SoA slots of the reference's sim_vars table (src/defines.cuh:57-78). */
enum {
    ORC_V = 0, ORC_M, ORC_N, ORC_H, ORC_LOCAL_Y, ORC_IY, ORC_EY,
    ORC_LOCAL_OUTPUT, ORC_LOCAL_IN, ORC_LOCAL_COUNT,
    ORC_EOUTPUT, ORC_EIN, ORC_ECOUNT,
    ORC_IOUTPUT, ORC_IIN, ORC_ICOUNT,
    ORC_APPCUR, ORC_NUM_SIM_PARAMS
};
/* Parameter block of the reference HH model (src/defines.cuh:87-102 and the
 * whole-brain variant src_wholebrain/ephys.cuh:47-61). */
typedef struct {
    float gna, ena, gk, ek, gl, el, Tmax, Vt, Kp, Ar, Ad;
    float g_local, e_local, g_gaba, e_gaba, g_exc, e_exc;
    float noise_mean, noise_intensity;
} orc_leapfrog_params;
void orc_leapfrog_params_src(orc_leapfrog_params* p);        /* src/ */
void orc_leapfrog_params_wholebrain(orc_leapfrog_params* p); /* src_wholebrain/ */
/* One Leapfrog_HH step over n neurons (src/ephys.cu:28-96).  vars[17] are
 * float arrays of length n, updated in place; z[i] is the standard normal
 * draw of neuron i for this step. */
void orc_hh_leapfrog(float* const* vars, int n, float dt, const orc_leapfrog_params* p, const double* z);

/* ------------------------------------------------ reference coupling ---- */
/* AtomicCoupling::operator() (src/coupling.cu:111-141): inputs are zeroed,
 * neurons with output > 0.1 fire (CheckFiringOperator, :103-109), every CSR
 * entry of a firing row adds 1 (signal_mode 0, src/coupling.cu:46) or the
 * row's output (signal_mode 1, src_wholebrain/coupling.cu:31) to its target.
 * firing_list (n ints) receives the ascending firing indices.  Returns the
 * number firing. */
int orc_coupling_push(int n, const int* indices, const int* offsets, const float* outputs,
                      float* inputs, int signal_mode, int* firing_list);

/* ----------------------------------------------- reference paracrine ---- */
/* Trilinear neuron->grid weights (src/paracrine.cu:136-270).  Positions are
 * centred (x in [-L/2, L/2), L = (nx-1) h).  idx8/w8 hold 8 entries per
 * neuron in the reference's corner order. */
void orc_trilinear_setup(int n, const float* x, const float* y, const float* z,
                         int nx, int ny, int nz, float h, int* idx8, float* w8);
/* scatter_to_grid (src/paracrine.cu:276-287): grid[idx] += w * s. */
void orc_scatter(int n, const int* idx8, const float* w8, const double* s, double* grid);
/* interpolate_at_location (src/paracrine.cu:288-296): out[i] = sum w * grid[idx]. */
void orc_interp(int n, const int* idx8, const float* w8, const double* grid, double* out);
/* Zero-padded 3x3x3 correlation, x fastest (af::convolve3 AF_CONV_DEFAULT). */
void orc_conv27(const double* in, double* out, int nx, int ny, int nz, const double K[27]);
/* Density_on_grid_3d::update_density (src/paracrine.cu:63-134), FP64.
 * u: density (in/out).  quirk_b != 0 reproduces the reference's right-hand
 * side, which uses the grid spacing where the time step belongs (:105).
 * Returns the number of CG iterations run; *final_rr the last ||r||^2. */
int orc_paracrine_cn_solve(double* u, int nx, int ny, int nz, double h, double D, double k,
                           double dt, double abs_tol, int max_iter, int quirk_b, double* final_rr);

/* ------------------------------------------- GB300 model semantics ------ */
typedef struct {
    double C, gNa, gK, gL, ENa, EK, EL, E_exc, E_inh, tau_exc, tau_inh;
    double v_thresh, noise_sigma, dt, g_par, E_par;
} orc_hh_params;
void orc_hh_params_standard(orc_hh_params* p);
/* Steady-state gates at voltage v. */
void orc_hh_steady_state(double v, double* m, double* h, double* n);
/* RK4 step of (V,m,h,n,ge,gi) with the external current held over the stages. */
void orc_hh_rk4(const orc_hh_params* p, double gna_scale, double i_ext, double u_par, double y[6]);

/* Network in CSR (row = presynaptic): row_ptr int64[n+1], col int32, weight
 * float, delay uint8 (steps, >= 1). */
typedef struct {
    int n;
    int64_t nnz;
    int64_t* row_ptr;
    int32_t* col;
    float* weight;
    uint8_t* delay;
} orc_csr;

/* CSC transpose, columns ordered by ascending CSR edge position (stable). */
void orc_csr_to_csc(const orc_csr* a, int64_t* col_ptr, int32_t* src, float* w, uint8_t* d, int64_t* edge_of);

/* Generators (must match the CUDA generators bit for bit in col/delay). */
/* Erdos-Renyi: edge i->j (j != i) iff u32(philox) < floor(p * 2^32);
 * weight = wmax * u01, delay = 1.  Two calls: first with col == NULL fills
 * row_ptr, second fills col/weight/delay. */
void orc_gen_er(int n, double p, float wmax, uint64_t seed, orc_csr* out);
/* Gaussian distance-dependent on a jittered lattice: fixed out-degree k,
 * lattice offsets from a discretised Gaussian table (sigma in lattice units),
 * lognormal(mu, s) weights, delay 1 + floor(u * dmax). */
void orc_gauss_table(double sigma_sites, int16_t* table4096);
int64_t orc_local_gaussian(int n, const float* x, const float* y, const float* z, float stddev, int n_stddevs,
                           uint64_t seed, int* offsets, int* indices, int64_t capacity);
void orc_block_tables(int n, int R, double size_sigma, double density_sigma, int dmax, uint64_t seed,
                      int* start, int* size, uint32_t* cum, uint8_t* pdelay);
void orc_gen_block(int n, int k, int R, double size_sigma, double density_sigma, int dmax, double w_mu,
                   double w_sigma, uint64_t seed, orc_csr* out);
void orc_init_drive(int n, uint64_t seed, float lo, float hi, float* out);
void orc_inh_flags(int n, double frac, int random, uint64_t seed, uint8_t* out);
void orc_gen_gauss(int n, int k, double sigma, double w_mu, double w_sigma, int dmax,
                   uint64_t seed, orc_csr* out);
void orc_lattice_positions(int n, uint64_t seed, float* x, float* y, float* z);

/* Whole simulation (FP64 state).  ring: double[2 * D * n] (E,I interleaved per
 * slot).  Returns spikes emitted this step; spikes[] receives their ids. */
typedef struct {
    orc_hh_params hp;
    int n, D;
    const orc_csr* net;
    const uint8_t* is_inh;
    const float* i_drive;
    const float* gna_scale;   /* may be NULL (1.0) */
    const double* u_par;      /* may be NULL */
    uint64_t seed;
    double* y;                /* 6 * n : V,m,h,n,ge,gi per neuron (AoS) */
    double* ring;             /* 2 * D * n */
    /* paracrine deposit: vox[n] voxel per neuron, src[G] accumulator (may be NULL) */
    const int32_t* vox;
    double* src;
    /* optional (may be NULL), n doubles: for each neuron that spiked this step,
     * min(threshold - V before, V after - threshold), the crossing's margin */
    double* margin;
} orc_sim;
int orc_sim_step(orc_sim* s, uint64_t step, int32_t* spikes);

/* 7-point backward-Euler operator A = (1 + dt k) I - dt div(D grad)/h^2 with
 * zero Dirichlet ghosts.  Dface: NULL for constant D (= D0), else a cell field
 * of D with harmonic-mean face coefficients. */
void orc_apply7(const double* x, double* y, int nx, int ny, int nz, double alpha /* dt D0 / h^2 */,
                double beta /* dt k */, const float* Dcell);
/* Jacobi-PCG on A x = b to ||r|| <= rtol ||b||; x holds the initial guess.
 * Returns iterations, -1 if max_iter reached. */
int orc_pcg7(double* x, const double* b, int nx, int ny, int nz, double alpha, double beta,
             const float* Dcell, double rtol, int max_iter, double* relres);

/* OpenMP threads the oracle uses (1 without OpenMP). */
int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
