// Reference-semantics primitives: the reference HH leapfrog step, the
// AtomicCoupling threshold/compaction/push, the network factory's in-degree
// and chunked lists, and the ParacrineModule (trilinear scatter/interpolation
// + Crank-Nicolson 27-point CG).  Each function cites the reference code whose
// behaviour it reproduces.
#include <cmath>
#include <cstring>
#include <vector>

#include "nn_hh.cuh"
#include "nn_internal.cuh"

// =============================================================== leapfrog ==

extern "C" void nn_leapfrog_params_reference(nn_leapfrog_params* p, int variant)
{
    if (!p) return;
    // src/defines.cuh:87-102
    p->gna = 120.0f; p->ena = 55.0f; p->gk = 36.0f; p->ek = -72.0f; p->gl = 0.3f; p->el = -50.0f;
    p->Tmax = 1.0f; p->Vt = -20.0f; p->Kp = 3.0f; p->Ar = 5.0f; p->Ad = 0.18f;
    p->g_local = 0.1f; p->e_local = 0.0f; p->g_gaba = 0.1f; p->e_gaba = -70.0f;
    p->g_exc = 0.1f; p->e_exc = 0.0f;
    p->noise_mean = 3.0f; p->noise_intensity = 1.5f;
    if (variant == 1) {
        // src_wholebrain/ephys.cuh:56-61: grey AMPA only, zero-mean noise of intensity 2
        p->g_local = 0.1f; p->g_gaba = 0.0f; p->g_exc = 0.0f;
        p->noise_mean = 0.0f; p->noise_intensity = 2.0f;
    }
}

namespace {
struct LFVars { float* v[NN_HH_NUM_VARS]; };

// Leapfrog_HH (src/ephys.cu:28-96), evaluated in the precision the
// reference's expressions have.  Its double literals (3.5, 0.1, 0.07, 0.125,
// 1.0) promote alpha_m, alpha_n, beta_h, the products 0.07 * e^x and
// 0.125 * e^x, and the output sigmoid to FP64, each rounded to float on
// assignment; exponentials of float arguments (alpha_h, beta_m, beta_n, the
// sigmoid's) are FP32 calls; the gate, synapse and membrane updates are FP32
// (Float = float, src/defines.cuh:50-55).  The expressions keep the
// reference's operand order, so each rounds as the reference's does.  The
// removable singularities of alpha_m (V = -35) and alpha_n (V = -50), 0/0 in
// the reference, take their limits (1 and 0.1) there.  V = -35 and V = -50
// are the only float inputs whose FP64 argument 3.5 + 0.1 V (or -5 - 0.1 V)
// lies within 1e-9 of zero, fused or not (the neighbouring floats give
// 3.8e-7), so the test is an FP32 compare, off the FP64 pipe that bounds
// this kernel.
__device__ __forceinline__ float lf_rate_am(float V)
{
    if (V == -35.0f) return 1.0f;
    return (float)((3.5 + 0.1 * V) / (1 - exp(-3.5 - 0.1 * V)));
}

__device__ __forceinline__ float lf_rate_an(float V)
{
    if (V == -50.0f) return 0.1f;
    return (float)((-0.5 - 0.01 * V) / (exp(-5 - 0.1 * V) - 1));
}

// One neuron's step (zi: its standard-normal noise draw).
__device__ __forceinline__ void lf_neuron(const LFVars& s, int i, float timestep, const nn_leapfrog_params& p,
                                          float zi)
{
    {
        const float local_in = s.v[NN_HH_LOCAL_IN][i], local_num_in = s.v[NN_HH_LOCAL_COUNT][i];
        const float Iin = s.v[NN_HH_IIN][i], Inum_in = s.v[NN_HH_ICOUNT][i];
        const float Ein = s.v[NN_HH_EIN][i], Enum_in = s.v[NN_HH_ECOUNT][i];
        const float appcur = s.v[NN_HH_APPCUR][i];
        const float V = s.v[NN_HH_V][i], M = s.v[NN_HH_M][i], N = s.v[NN_HH_N][i], H = s.v[NN_HH_H][i];
        const float local_Y = s.v[NN_HH_LOCAL_Y][i], IY = s.v[NN_HH_IY][i], EY = s.v[NN_HH_EY][i];

        const float Am = lf_rate_am(V);
        const float An = lf_rate_an(V);
        const float Ah = (float)(0.07 * expf(-V / 20 - 3));
        const float Bm = 4 * expf(-(V + 60) / 18);
        const float Bn = (float)(0.125 * expf(-(V + 60) / 80));
        const float Bh = (float)(1 / (exp(-3 - 0.1 * V) + 1));

        const float new_M = (Am * timestep + (1 - timestep / 2 * (Am + Bm)) * M) / (timestep / 2 * (Am + Bm) + 1);
        const float new_N = (An * timestep + (1 - timestep / 2 * (An + Bn)) * N) / (timestep / 2 * (An + Bn) + 1);
        const float new_H = (Ah * timestep + (1 - timestep / 2 * (Ah + Bh)) * H) / (timestep / 2 * (Ah + Bh) + 1);

        const float Ar = p.Ar, Ad = p.Ad;
        const float local_T = local_num_in > 0 ? local_in / local_num_in : 0;
        const float new_local_Y = (Ar * local_T * timestep + (1 - timestep / 2 * (Ar * local_T + Ad)) * local_Y) /
                                  (timestep / 2 * (Ar * local_T + Ad) + 1);
        const float I_T = Inum_in > 0 ? Iin / Inum_in : 0;
        const float new_IY = (Ar * I_T * timestep + (1 - timestep / 2 * (Ar * I_T + Ad)) * IY) /
                             (timestep / 2 * (Ar * I_T + Ad) + 1);
        const float E_T = Enum_in > 0 ? Ein / Enum_in : 0;
        const float new_EY = (Ar * E_T * timestep + (1 - timestep / 2 * (Ar * E_T + Ad)) * EY) /
                             (timestep / 2 * (Ar * E_T + Ad) + 1);

        // G, E and the membrane update with every rounding explicit, in the
        // order and fusion the reference kernel has when nvcc builds it for
        // sm_103a (found by comparing the two kernels' outputs on the same
        // states: the reference forms E * dt inside a fused multiply-add on
        // top of the rounded (noise + I_app) * dt; left to the compiler, this
        // source fused the other product and differed by an ulp in 19 % of
        // the neurons).  The reference weights the local and excitatory
        // synapses by g_ampa and the inhibitory one by g_gaba; the whole-brain
        // variant sets them apart, hence g_local / g_exc.
        const float gna_m3h = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(p.gna, new_M), new_M), new_M), new_H);
        const float gk_n4 = __fmul_rn(p.gk, powf(new_N, 4));
        float G = __fadd_rn(__fadd_rn(gna_m3h, gk_n4), p.gl);
        G = __fadd_rn(G, __fmul_rn(p.g_local, new_local_Y));
        G = __fadd_rn(G, __fmul_rn(p.g_gaba, new_IY));
        G = __fadd_rn(G, __fmul_rn(p.g_exc, new_EY));
        float E = __fmaf_rn(gna_m3h, p.ena, __fmul_rn(gk_n4, p.ek));
        E = __fadd_rn(E, __fmul_rn(p.gl, p.el));
        E = __fadd_rn(E, __fmul_rn(__fmul_rn(p.g_local, new_local_Y), p.e_local));
        E = __fmaf_rn(__fmul_rn(p.g_gaba, new_IY), p.e_gaba, E);
        E = __fadd_rn(E, __fmul_rn(__fmul_rn(p.g_exc, new_EY), p.e_exc));

        const float white_noise = __fmaf_rn(p.noise_intensity, zi, p.noise_mean);
        const float half_dt = timestep / 2;
        float num = __fmaf_rn(E, timestep, __fmul_rn(__fadd_rn(white_noise, appcur), timestep));
        num = __fmaf_rn(__fmaf_rn(-half_dt, G, 1.0f), V, num);
        const float nV = __fdiv_rn(num, __fmaf_rn(half_dt, G, 1.0f));
        s.v[NN_HH_V][i] = nV;
        s.v[NN_HH_M][i] = new_M;
        s.v[NN_HH_N][i] = new_N;
        s.v[NN_HH_H][i] = new_H;
        s.v[NN_HH_LOCAL_Y][i] = new_local_Y;
        s.v[NN_HH_IY][i] = new_IY;
        s.v[NN_HH_EY][i] = new_EY;
        const float out = (float)(p.Tmax / (1.0 + expf(-(nV - p.Vt) / p.Kp)));
        s.v[NN_HH_LOCAL_OUTPUT][i] = out;
        s.v[NN_HH_IOUTPUT][i] = out;
        s.v[NN_HH_EOUTPUT][i] = out;
    }
}

// A thread steps the neuron pair (2k, 2k + 1), which shares one draw of the
// counter-based noise stream (the pair's two Box-Muller outputs).
template <bool EXT_Z>
__global__ void __launch_bounds__(256) k_leapfrog(LFVars s, int n, float timestep, nn_leapfrog_params p,
                                                  uint64_t seed, uint64_t step, const float* __restrict__ z)
{
    const int pairs = (n + 1) >> 1;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < pairs; k += gridDim.x * blockDim.x) {
        const int i0 = 2 * k;
        const bool two = i0 + 1 < n;
        float z0, z1;
        if (EXT_Z) {
            z0 = z[i0];
            z1 = two ? z[i0 + 1] : 0.0f;
        } else {
            nn_normal_pair(seed, (uint32_t)k, step, z0, z1);
        }
        lf_neuron(s, i0, timestep, p, z0);
        if (two) lf_neuron(s, i0 + 1, timestep, p, z1);
    }
}

nn_status leapfrog_launch(nn_ctx* ctx, float* const* vars, int n, float dt, const nn_leapfrog_params* p,
                          uint64_t seed, uint64_t step, const float* d_z, const char* what)
{
    if (!ctx || !vars || !p || n < 0) return nn_fail(ctx, NN_ERR_INVALID_ARG, "%s: bad argument", what);
    if (n == 0) return NN_OK;
    LFVars s;
    for (int q = 0; q < NN_HH_NUM_VARS; ++q) {
        if (!vars[q]) return nn_fail(ctx, NN_ERR_INVALID_ARG, "%s: sim_vars[%d] is NULL", what, q);
        s.v[q] = vars[q];
    }
    const int grid = nn_grid_for(ctx, ((int64_t)n + 1) / 2, 256, 64);
    if (d_z) k_leapfrog<true><<<grid, 256, 0, ctx->stream>>>(s, n, dt, *p, seed, step, d_z);
    else k_leapfrog<false><<<grid, 256, 0, ctx->stream>>>(s, n, dt, *p, seed, step, nullptr);
    NN_CHECK_LAUNCH(ctx, "k_leapfrog");
    return NN_OK;
}
}  // namespace

extern "C" nn_status nn_hh_leapfrog_step(nn_ctx* ctx, float* const* vars, int n, float dt,
                                         const nn_leapfrog_params* p, uint64_t seed, uint64_t step)
{
    return leapfrog_launch(ctx, vars, n, dt, p, seed, step, nullptr, "nn_hh_leapfrog_step");
}

extern "C" nn_status nn_hh_leapfrog_step_z(nn_ctx* ctx, float* const* vars, int n, float dt,
                                           const nn_leapfrog_params* p, const float* d_z)
{
    if (!d_z) return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_hh_leapfrog_step_z: d_z is NULL");
    return leapfrog_launch(ctx, vars, n, dt, p, 0, 0, d_z, "nn_hh_leapfrog_step_z");
}

// =============================================================== coupling ==

struct nn_coupling {
    nn_ctx* ctx = nullptr;
    int n = 0;
    int* firing = nullptr;       // n entries; first count ascending
    int* count = nullptr;        // device int
    int64_t* block_counts = nullptr;
    int nblocks = 0;
};

namespace {
constexpr int CMP_THREADS = 256;
constexpr int CMP_ITEMS = 8;
constexpr int CMP_TILE = CMP_THREADS * CMP_ITEMS;

// CheckFiringOperator (src/coupling.cu:103-109)
__device__ __forceinline__ int fires(float out) { return out > 0.1f ? 1 : 0; }

__global__ void __launch_bounds__(CMP_THREADS) k_cmp_count(const float* out, int n, int64_t* block_counts)
{
    const int base = blockIdx.x * CMP_TILE + threadIdx.x * CMP_ITEMS;
    int c = 0;
#pragma unroll
    for (int q = 0; q < CMP_ITEMS; ++q)
        if (base + q < n) c += fires(out[base + q]);
    __shared__ int tot;
    if (threadIdx.x == 0) tot = 0;
    __syncthreads();
    c = __reduce_add_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(&tot, c);
    __syncthreads();
    if (threadIdx.x == 0) block_counts[blockIdx.x] = tot;
}

// single block: exclusive scan of the block counts, total -> *count
__global__ void __launch_bounds__(1024) k_cmp_scan(int64_t* bc, int nb, int* count)
{
    __shared__ int64_t carry_s;
    __shared__ int64_t warp_tot[32];
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    for (int off = 0; off < nb; off += 1024) {
        const int i = off + threadIdx.x;
        int64_t v = i < nb ? bc[i] : 0;
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        int64_t inc = v;
        for (int o = 1; o < 32; o <<= 1) {
            int64_t t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) warp_tot[w] = inc;
        __syncthreads();
        if (w == 0) {
            int64_t t = warp_tot[lane];
            for (int o = 1; o < 32; o <<= 1) {
                int64_t u = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += u;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        const int64_t ex = carry_s + (w ? warp_tot[w - 1] : 0) + inc - v;
        if (i < nb) bc[i] = ex;
        __syncthreads();
        if (threadIdx.x == 0) carry_s += warp_tot[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) *count = (int)carry_s;
}

__global__ void __launch_bounds__(CMP_THREADS) k_cmp_write(const float* out, int n, const int64_t* block_off,
                                                           int* list)
{
    const int base = blockIdx.x * CMP_TILE + threadIdx.x * CMP_ITEMS;
    int f[CMP_ITEMS];
    int c = 0;
#pragma unroll
    for (int q = 0; q < CMP_ITEMS; ++q) {
        f[q] = base + q < n ? fires(out[base + q]) : 0;
        c += f[q];
    }
    // block exclusive scan of c
    __shared__ int wt[CMP_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int inc = c;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) wt[w] = inc;
    __syncthreads();
    int wbase = 0;
    for (int q = 0; q < w; ++q) wbase += wt[q];
    int pos = (int)block_off[blockIdx.x] + wbase + inc - c;
#pragma unroll
    for (int q = 0; q < CMP_ITEMS; ++q)
        if (f[q]) list[pos++] = base + q;
}

// Threshold count of each tile, with the tile's inputs zeroed (the first of
// the two launches of nn_coupling_run).
__global__ void __launch_bounds__(CMP_THREADS) k_cmp_count_zero(const float* out, int n, int64_t* block_counts,
                                                                float* inputs)
{
    const int base = blockIdx.x * CMP_TILE + threadIdx.x * CMP_ITEMS;
    int c = 0;
#pragma unroll
    for (int q = 0; q < CMP_ITEMS; ++q)
        if (base + q < n) {
            c += fires(out[base + q]);
            inputs[base + q] = 0.0f;
        }
    __shared__ int tot;
    if (threadIdx.x == 0) tot = 0;
    __syncthreads();
    c = __reduce_add_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(&tot, c);
    __syncthreads();
    if (threadIdx.x == 0) block_counts[blockIdx.x] = tot;
}

// The second launch: each tile's offset in the ascending firing list (the sum
// of the earlier tiles' counts), its entries written, the total stored by the
// last tile, and the tile's firing neurons scattered (signal_spikes_kernel),
// a warp per firing neuron with four targets per lane loaded before their
// reductions.
__global__ void __launch_bounds__(CMP_THREADS) k_cmp_write_push(const float* out, int n, const int64_t* block_counts,
                                                                int nblocks, int* list, int* count,
                                                                const int* indices, const int* offsets, float* inputs,
                                                                int signal_mode)
{
    __shared__ int64_t red[CMP_THREADS / 32];
    __shared__ int s_list[CMP_TILE];
    __shared__ int s_n;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t acc = 0;
    for (int b = threadIdx.x; b < (int)blockIdx.x; b += CMP_THREADS) acc += block_counts[b];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) red[w] = acc;
    __syncthreads();
    int64_t boff = 0;
    for (int q = 0; q < CMP_THREADS / 32; ++q) boff += red[q];
    if (blockIdx.x == nblocks - 1 && threadIdx.x == 0) *count = (int)(boff + block_counts[blockIdx.x]);
    const int base = blockIdx.x * CMP_TILE + threadIdx.x * CMP_ITEMS;
    int f[CMP_ITEMS];
    int c = 0;
#pragma unroll
    for (int q = 0; q < CMP_ITEMS; ++q) {
        f[q] = base + q < n ? fires(out[base + q]) : 0;
        c += f[q];
    }
    __shared__ int wt[CMP_THREADS / 32];
    int inc = c;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) wt[w] = inc;
    __syncthreads();
    int wbase = 0;
    for (int q = 0; q < w; ++q) wbase += wt[q];
    int pos = wbase + inc - c;
#pragma unroll
    for (int q = 0; q < CMP_ITEMS; ++q)
        if (f[q]) {
            list[boff + pos] = base + q;
            s_list[pos++] = base + q;
        }
    if (threadIdx.x == CMP_THREADS - 1) s_n = wbase + inc;
    __syncthreads();
    const int nf = s_n;
    for (int k = w; k < nf; k += CMP_THREADS / 32) {
        const int pre = s_list[k];
        const float sig = signal_mode ? out[pre] : 1.0f;
        const int beg = offsets[pre], end = offsets[pre + 1];
        for (int e0 = beg + lane; e0 < end; e0 += 128) {
            int post[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) post[u] = e0 + 32 * u < end ? indices[e0 + 32 * u] : -1;
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if ((unsigned)post[u] < (unsigned)n) atomicAdd(inputs + post[u], sig);
        }
    }
}

// signal_spikes_kernel (src/coupling.cu:34-48; src_wholebrain/coupling.cu:12-33),
// a warp per firing presynaptic neuron with the lanes over its targets.
__global__ void __launch_bounds__(256) k_push_ref(const int* list, const int* count, const int* indices,
                                                  const int* offsets, float* inputs, const float* outputs,
                                                  int signal_mode, int n, int target_base)
{
    const int lane = threadIdx.x & 31;
    const int nf = *count;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int f = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); f < nf; f += warps) {
        const int pre = list[f];
        const float sig = signal_mode ? outputs[pre] : 1.0f;
        const int beg = offsets[pre], end = offsets[pre + 1];
        for (int e = beg + lane; e < end; e += 32) {
            const int post = target_base + indices[e];
            if ((unsigned)post < (unsigned)n) atomicAdd(inputs + post, sig);
        }
    }
}
}  // namespace

extern "C" nn_status nn_coupling_create(nn_ctx* ctx, int n, nn_coupling** out)
{
    if (!ctx || !out || n < 0) return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_coupling_create: bad argument");
    nn_coupling* c = new nn_coupling();
    c->ctx = ctx;
    nn_ctx_retain(ctx);
    c->n = n;
    c->nblocks = (n + CMP_TILE - 1) / CMP_TILE;
    if (c->nblocks < 1) c->nblocks = 1;
    nn_status st = nn_alloc(ctx, &c->firing, (size_t)(n > 0 ? n : 1));
    if (st == NN_OK) st = nn_alloc(ctx, &c->count, 1);
    if (st == NN_OK) st = nn_alloc(ctx, &c->block_counts, (size_t)c->nblocks);
    if (st != NN_OK) {
        nn_coupling_destroy(c);
        return st;
    }
    // firing_neurons(N_, 0) (src/coupling.cu:5-8 of the coupling constructor)
    cudaMemsetAsync(c->firing, 0, sizeof(int) * (size_t)(n > 0 ? n : 1), ctx->stream);
    cudaMemsetAsync(c->count, 0, sizeof(int), ctx->stream);
    *out = c;
    return nn_cuda_check(ctx, cudaGetLastError(), "nn_coupling_create");
}

extern "C" nn_status nn_coupling_destroy(nn_coupling* c)
{
    if (!c) return NN_OK;
    if (c->ctx) cudaStreamSynchronize(c->ctx->stream);
    nn_release(c->firing);
    nn_release(c->count);
    nn_release(c->block_counts);
    nn_ctx* ctx = c->ctx;
    delete c;
    nn_ctx_release(ctx);
    return NN_OK;
}

extern "C" const int* nn_coupling_firing_list(const nn_coupling* c) { return c ? c->firing : nullptr; }
extern "C" const int* nn_coupling_firing_count(const nn_coupling* c) { return c ? c->count : nullptr; }

static nn_status coupling_compact(nn_coupling* c, float* d_inputs, const float* d_outputs)
{
    nn_ctx* ctx = c->ctx;
    NN_CUDA(ctx, cudaMemsetAsync(d_inputs, 0, sizeof(float) * (size_t)c->n, ctx->stream));
    k_cmp_count<<<c->nblocks, CMP_THREADS, 0, ctx->stream>>>(d_outputs, c->n, c->block_counts);
    NN_CHECK_LAUNCH(ctx, "k_cmp_count");
    k_cmp_scan<<<1, 1024, 0, ctx->stream>>>(c->block_counts, c->nblocks, c->count);
    NN_CHECK_LAUNCH(ctx, "k_cmp_scan");
    k_cmp_write<<<c->nblocks, CMP_THREADS, 0, ctx->stream>>>(d_outputs, c->n, c->block_counts, c->firing);
    NN_CHECK_LAUNCH(ctx, "k_cmp_write");
    return NN_OK;
}

static nn_status coupling_readback(nn_coupling* c, int* num_firing)
{
    if (!num_firing) return NN_OK;
    NN_CUDA(c->ctx, cudaMemcpyAsync(num_firing, c->count, sizeof(int), cudaMemcpyDeviceToHost, c->ctx->stream));
    NN_CUDA(c->ctx, cudaStreamSynchronize(c->ctx->stream));
    return NN_OK;
}

extern "C" nn_status nn_coupling_run(nn_coupling* c, const int* d_indices, const int* d_offsets, float* d_inputs,
                                     const float* d_outputs, int signal_mode, int* num_firing)
{
    if (!c || !d_offsets || !d_inputs || !d_outputs) return nn_fail(c ? c->ctx : nullptr, NN_ERR_INVALID_ARG, "nn_coupling_run: bad argument");
    if (c->n == 0) { if (num_firing) *num_firing = 0; return NN_OK; }
    nn_ctx* ctx = c->ctx;
    // two launches: threshold counts with the inputs zeroed, then the ordered
    // list, the count and the scatter
    k_cmp_count_zero<<<c->nblocks, CMP_THREADS, 0, ctx->stream>>>(d_outputs, c->n, c->block_counts, d_inputs);
    NN_CHECK_LAUNCH(ctx, "k_cmp_count_zero");
    k_cmp_write_push<<<c->nblocks, CMP_THREADS, 0, ctx->stream>>>(d_outputs, c->n, c->block_counts, c->nblocks,
                                                                  c->firing, c->count, d_indices, d_offsets, d_inputs,
                                                                  signal_mode);
    NN_CHECK_LAUNCH(ctx, "k_cmp_write_push");
    return coupling_readback(c, num_firing);
}

extern "C" nn_status nn_coupling_run_chunked(nn_coupling* c, int nchunks, int n_per_chunk,
                                             const int* const* d_chunk_indices, const int* const* d_chunk_offsets,
                                             float* d_inputs, const float* d_outputs, int* num_firing)
{
    if (!c || nchunks <= 0 || n_per_chunk <= 0 || !d_chunk_indices || !d_chunk_offsets || !d_inputs || !d_outputs)
        return nn_fail(c ? c->ctx : nullptr, NN_ERR_INVALID_ARG, "nn_coupling_run_chunked: bad argument");
    if (c->n == 0) { if (num_firing) *num_firing = 0; return NN_OK; }
    nn_ctx* ctx = c->ctx;
    NN_TRY(coupling_compact(c, d_inputs, d_outputs));
    for (int ch = 0; ch < nchunks; ++ch) {
        k_push_ref<<<nn_grid_for(ctx, (int64_t)c->n * 32, 256, 4), 256, 0, ctx->stream>>>(
            c->firing, c->count, d_chunk_indices[ch], d_chunk_offsets[ch], d_inputs, d_outputs, NN_SIGNAL_COUNT, c->n,
            ch * n_per_chunk);
        NN_CHECK_LAUNCH(ctx, "k_push_ref(chunk)");
    }
    return coupling_readback(c, num_firing);
}

// ======================================================== network factory ==

namespace {
uint32_t minstd_next(uint32_t& s)
{
    s = (uint32_t)(((uint64_t)s * 16807u) % 2147483647u);
    return s;
}

// libstdc++ uniform_int_distribution<int>(a, b) over minstd_rand0 ([1, 2^31-2]):
// downscaling by rejection (scaling = range / (b - a + 1)).
int uniform_int(uint32_t& s, int a, int b)
{
    const uint64_t urngrange = 2147483646u - 1u;
    const uint64_t urange = (uint64_t)((int64_t)b - (int64_t)a);
    uint64_t ret;
    if (urngrange > urange) {
        const uint64_t uerange = urange + 1, scaling = urngrange / uerange, past = uerange * scaling;
        do ret = (uint64_t)minstd_next(s) - 1u;
        while (ret >= past);
        ret /= scaling;
    } else {
        ret = (uint64_t)minstd_next(s) - 1u;
    }
    return (int)(ret + (uint64_t)(int64_t)a);
}
}  // namespace

extern "C" nn_status nn_net_uniform_random(int n, int ncouple, uint32_t* engine_state, int* h_indices, int* h_offsets)
{
    // UniformRandomNetwork::Generate (src/network_factory.cu:96-131).  The
    // reference loops forever when ncouple > n; that is rejected here.
    if (n <= 0 || ncouple < 0 || ncouple > n || !engine_state || !h_offsets || (ncouple && !h_indices))
        return NN_ERR_INVALID_ARG;
    std::vector<char> used((size_t)n, 0);
    for (int i = 0; i < n; ++i) {
        int* row = h_indices + (int64_t)i * ncouple;
        for (int j = 0; j < ncouple; ++j) {
            int d;
            do d = uniform_int(*engine_state, 0, n - 1);
            while (used[(size_t)d]);
            row[j] = d;
            used[(size_t)d] = 1;
        }
        for (int j = 0; j < ncouple; ++j) used[(size_t)row[j]] = 0;
        h_offsets[i] = i * ncouple;
    }
    h_offsets[n] = n * ncouple;
    return NN_OK;
}

namespace {
__global__ void k_tcount(const int* idx, int64_t nnz, int n, float* tcount)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x) {
        const int t = idx[e];
        if ((unsigned)t < (unsigned)n) atomicAdd(tcount + t, 1.0f);
    }
}

constexpr int MAX_CHUNKS = 64;
struct ChunkPtrs { int* p[MAX_CHUNKS]; };

// per row and chunk: number of targets in the chunk; written at [c][i + 1]
__global__ void k_chunk_count(const int* idx, const int* off, int n, int nchunks, int npc, int64_t* cnt)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        for (int c = 0; c < nchunks; ++c) cnt[(int64_t)c * (n + 1) + i] = 0;
        for (int e = off[i]; e < off[i + 1]; ++e) {
            const int c = idx[e] / npc;
            if (c >= 0 && c < nchunks) cnt[(int64_t)c * (n + 1) + i] += 1;
        }
    }
}

__global__ void k_chunk_fill(const int* idx, const int* off, int n, int nchunks, int npc, const int64_t* pos,
                             ChunkPtrs out_idx, ChunkPtrs out_off)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x) {
        int64_t cur[MAX_CHUNKS];
        for (int c = 0; c < nchunks; ++c) {
            cur[c] = pos[(int64_t)c * (n + 1) + i];
            out_off.p[c][i] = (int)cur[c];
        }
        if (i == n) continue;
        for (int e = off[i]; e < off[i + 1]; ++e) {
            const int t = idx[e];
            const int c = t / npc;
            if (c >= 0 && c < nchunks) out_idx.p[c][cur[c]++] = t % npc;
        }
    }
}
}  // namespace

extern "C" nn_status nn_net_tcount(nn_ctx* ctx, const int* d_indices, int64_t nnz, int n, float* d_tcount)
{
    // Tcount loop of Network::ToAdjacencyList (src/network_factory.cu:19-22)
    if (!ctx || n < 0 || nnz < 0 || (nnz && !d_indices) || (n && !d_tcount))
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_net_tcount: bad argument");
    if (n == 0) return NN_OK;
    NN_CUDA(ctx, cudaMemsetAsync(d_tcount, 0, sizeof(float) * (size_t)n, ctx->stream));
    if (nnz > 0) {
        k_tcount<<<nn_grid_for(ctx, nnz, 256, 16), 256, 0, ctx->stream>>>(d_indices, nnz, n, d_tcount);
        NN_CHECK_LAUNCH(ctx, "k_tcount");
    }
    return NN_OK;
}

extern "C" nn_status nn_net_to_chunked(nn_ctx* ctx, const int* d_indices, const int* d_offsets, int n, int nchunks,
                                       int n_per_chunk, int* const* d_chunk_indices, int* const* d_chunk_offsets,
                                       int64_t* chunk_nnz)
{
    // Network::ToChunkedAdjacencyList (src/network_factory.cu:29-85)
    if (!ctx || n <= 0 || nchunks <= 0 || nchunks > MAX_CHUNKS || n_per_chunk <= 0 || !d_offsets ||
        !d_chunk_indices || !d_chunk_offsets || !chunk_nnz)
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_net_to_chunked: bad argument");
    int64_t* cnt = nullptr;
    int64_t* pos = nullptr;
    const size_t stride = (size_t)n + 1;
    NN_TRY(nn_alloc(ctx, &cnt, stride * nchunks));
    NN_TRY(nn_alloc(ctx, &pos, stride * nchunks));
    k_chunk_count<<<nn_grid_for(ctx, n, 256, 16), 256, 0, ctx->stream>>>(d_indices, d_offsets, n, nchunks, n_per_chunk,
                                                                          cnt);
    NN_CHECK_LAUNCH(ctx, "k_chunk_count");
    for (int c = 0; c < nchunks; ++c) {
        NN_CUDA(ctx, cudaMemsetAsync(cnt + c * stride + n, 0, sizeof(int64_t), ctx->stream));
        NN_TRY(nn_scan_exclusive_i64(ctx, cnt + c * stride, pos + c * stride, (int64_t)stride));
    }
    ChunkPtrs oi, oo;
    for (int c = 0; c < nchunks; ++c) {
        oi.p[c] = d_chunk_indices[c];
        oo.p[c] = d_chunk_offsets[c];
    }
    k_chunk_fill<<<nn_grid_for(ctx, (int64_t)n + 1, 128, 16), 128, 0, ctx->stream>>>(d_indices, d_offsets, n, nchunks,
                                                                                     n_per_chunk, pos, oi, oo);
    NN_CHECK_LAUNCH(ctx, "k_chunk_fill");
    for (int c = 0; c < nchunks; ++c)
        NN_CUDA(ctx, cudaMemcpyAsync(&chunk_nnz[c], pos + c * stride + n, sizeof(int64_t), cudaMemcpyDeviceToHost,
                                     ctx->stream));
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFree(cnt);
    cudaFree(pos);
    return NN_OK;
}

// ============================================================== paracrine ==

struct nn_paracrine {
    nn_ctx* ctx = nullptr;
    nn_paracrine_ref_params p{};
    int n = 0;
    int64_t G = 0;
    int* idx8 = nullptr;
    float* w8 = nullptr;
    float* u = nullptr;          // density
    float* Ax = nullptr;         // scatter accumulator
    float *lap = nullptr, *x = nullptr, *b = nullptr, *r = nullptr, *pv = nullptr, *Ap = nullptr;
    float* at_neurons = nullptr;    // density_at_neurons
    float* generated = nullptr;     // density_generated_at_neurons
    float* g_out = nullptr;         // d_g_paracrine (caller's)
    double* scal = nullptr;         // [0]=rr [1]=pAp [2]=rr_new
    double* partials = nullptr;
    unsigned int* ticket = nullptr;
    int* done = nullptr;            // convergence flag
    int nparts = 0;
};

extern "C" void nn_paracrine_ref_params_default(nn_paracrine_ref_params* p)
{
    if (!p) return;
    // the SCN run of diekman_benchmark (src/main.cu:525) with its 32^3 grid
    p->nx = p->ny = p->nz = 32;
    p->h = 1.0f;
    p->D = 2e-5f;
    p->decay = 3e-4f;
    p->par_dt = 100.0f * 0.4f;
    p->coup_strength = 0.5f;
    p->max_iter = 20;
    p->abs_tol = 1e-6f;
    p->quirk_rhs = 1;
    p->quirk_firing_list = 1;
}

namespace {
struct Stencil27 { float k[27]; };

// Trilinear weights (src/paracrine.cu:136-270), written per neuron in the
// reference's corner order (:189-195) with the same float arithmetic.
__global__ void k_trilinear(int n, const float* x, const float* y, const float* z, int nx, int ny, int nz, float h,
                            int* idx8, float* w8)
{
    const float Lx = __fmul_rn((float)(nx - 1), h), Ly = __fmul_rn((float)(ny - 1), h), Lz = __fmul_rn((float)(nz - 1), h);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float xr = __fadd_rn(__fdiv_rn(x[i], Lx), 0.5f);
        const float yr = __fadd_rn(__fdiv_rn(y[i], Ly), 0.5f);
        const float zr = __fadd_rn(__fdiv_rn(z[i], Lz), 0.5f);
        const float sx = __fmul_rn((float)(nx - 1), xr), sy = __fmul_rn((float)(ny - 1), yr), sz = __fmul_rn((float)(nz - 1), zr);
        const int m = (int)sx, q = (int)sy, pz = (int)sz;
        const float fx = __fsub_rn(sx, (float)m), fy = __fsub_rn(sy, (float)q), fz = __fsub_rn(sz, (float)pz);
        const int base = m + q * nx + pz * nx * ny;
        const float kx0 = __fsub_rn(1.0f, fx), ky0 = __fsub_rn(1.0f, fy), kz0 = __fsub_rn(1.0f, fz);
        const float kx1 = __fsub_rn(1.0f, kx0), ky1 = __fsub_rn(1.0f, ky0), kz1 = __fsub_rn(1.0f, kz0);
        const float xy[4] = {__fmul_rn(kx0, ky0), __fmul_rn(kx1, ky0), __fmul_rn(kx0, ky1), __fmul_rn(kx1, ky1)};
        const int off[8] = {0, 1, nx, nx + 1, nx * ny, nx * ny + 1, nx * ny + nx, nx * ny + nx + 1};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            w8[8 * (int64_t)i + c] = __fmul_rn(xy[c], kz0);
            w8[8 * (int64_t)i + c + 4] = __fmul_rn(xy[c], kz1);
        }
#pragma unroll
        for (int c = 0; c < 8; ++c) idx8[8 * (int64_t)i + c] = base + off[c];
    }
}

// scatter_to_grid (src/paracrine.cu:276-287): grid += G^T s
__global__ void k_scatter(int n, const int* idx8, const float* w8, const float* s, float* grid, int64_t G)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float v = s[i];
        if (v == 0.0f) continue;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int g = idx8[8 * (int64_t)i + c];
            if ((uint64_t)g < (uint64_t)G) atomicAdd(grid + g, w8[8 * (int64_t)i + c] * v);
        }
    }
}

// interpolate_at_location (src/paracrine.cu:288-296)
__global__ void k_interp(int n, const int* idx8, const float* w8, const float* grid, int64_t G, float* out, float* out2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float acc = 0.0f;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int g = idx8[8 * (int64_t)i + c];
            if ((uint64_t)g < (uint64_t)G) acc += w8[8 * (int64_t)i + c] * grid[g];
        }
        out[i] = acc;
        if (out2) out2[i] = acc;
    }
}

// update_on_fine_timescale (src/paracrine.cuh:246-253)
__global__ void k_fine(int n, const int* list, const int* count, float* gen, float coup, int quirk)
{
    if (quirk) {
        // transform_if with the compacted index buffer as the stencil
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            if (list[i] != 0) gen[i] += coup;
    } else {
        const int nf = *count;
        for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) gen[list[f]] += coup;
    }
}

// zero-padded 3x3x3 correlation (af::convolve3 with AF_CONV_DEFAULT), x fastest
__global__ void k_conv27(const float* in, float* out, int nx, int ny, int nz, Stencil27 K, const int* done)
{
    if (done && *done) return;
    const int64_t G = (int64_t)nx * ny * nz;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < G; c += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % nx);
        const int j = (int)((c / nx) % ny);
        const int k = (int)(c / ((int64_t)nx * ny));
        float acc = 0.0f;
#pragma unroll
        for (int dz = -1; dz <= 1; ++dz) {
            const int kk = k + dz;
            if (kk < 0 || kk >= nz) continue;
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy) {
                const int jj = j + dy;
                if (jj < 0 || jj >= ny) continue;
#pragma unroll
                for (int dx = -1; dx <= 1; ++dx) {
                    const int ii = i + dx;
                    if (ii < 0 || ii >= nx) continue;
                    acc += K.k[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)] * in[ii + (int64_t)nx * (jj + (int64_t)ny * kk)];
                }
            }
        }
        out[c] = acc;
    }
}

__global__ void k_add(float* u, const float* a, int64_t G)
{
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < G; q += (int64_t)gridDim.x * blockDim.x)
        u[q] += a[q];
}

// x = a*u + b*lap ; y = c*u + d*lap
__global__ void k_cn_init(const float* u, const float* lap, float* x, float* b, int64_t G, float a, float bb, float c,
                          float d)
{
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < G; q += (int64_t)gridDim.x * blockDim.x) {
        x[q] = a * u[q] + bb * lap[q];
        b[q] = c * u[q] + d * lap[q];
    }
}

// Finish a grid-wide FP64 sum: block partial -> last block reduces in a fixed order.
__device__ bool last_block_reduce(double v, double* partials, unsigned int* ticket, double* result)
{
    __shared__ double ws[32];
    __shared__ bool is_last;
    v = nn_warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) ws[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += ws[q];
        partials[blockIdx.x] = s;
        __threadfence();
        is_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!is_last) return false;
    // the last block sums the partials with all its threads (fixed order)
    __threadfence();
    double s = 0.0;
    for (unsigned q = threadIdx.x; q < gridDim.x; q += blockDim.x) s += ((volatile double*)partials)[q];
    s = nn_warp_sum(s);
    __syncthreads();
    if (lane == 0) ws[w] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += ws[q];
        *result = t;
        *ticket = 0;
    }
    __syncthreads();
    return true;
}

// r = b - Ax ; p = r ; rr = (r, r); done = rr < tol
__global__ void k_cn_residual(const float* b, const float* Ax, float* r, float* p, int64_t G, double* partials,
                              unsigned int* ticket, double* scal, int* done, float tol)
{
    double acc = 0.0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < G; q += (int64_t)gridDim.x * blockDim.x) {
        const float rv = b[q] - Ax[q];
        r[q] = rv;
        p[q] = rv;
        acc += (double)rv * rv;
    }
    if (last_block_reduce(acc, partials, ticket, &scal[0]) && threadIdx.x == 0) *done = scal[0] < (double)tol ? 2 : 0;
}

// pAp = (p, Ap)
__global__ void k_cn_pap(const float* p, const float* Ap, int64_t G, double* partials, unsigned int* ticket,
                         double* scal, const int* done)
{
    if (*done) return;
    double acc = 0.0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < G; q += (int64_t)gridDim.x * blockDim.x)
        acc += (double)p[q] * Ap[q];
    last_block_reduce(acc, partials, ticket, &scal[1]);
}

// x += a p ; r -= a Ap ; rr_new = (r, r); converged -> done; else p = r + beta p (next kernel)
__global__ void k_cn_update(float* x, float* r, const float* p, const float* Ap, int64_t G, double* partials,
                            unsigned int* ticket, double* scal, int* done, float tol, int* iters)
{
    if (*done) return;
    const float alpha = (float)(scal[0] / scal[1]);
    double acc = 0.0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < G; q += (int64_t)gridDim.x * blockDim.x) {
        x[q] += alpha * p[q];
        const float rv = r[q] - alpha * Ap[q];
        r[q] = rv;
        acc += (double)rv * rv;
    }
    if (last_block_reduce(acc, partials, ticket, &scal[2]) && threadIdx.x == 0) {
        *iters += 1;
        if (scal[2] < (double)tol) *done = 1;
    }
}

__global__ void k_cn_direction(float* p, const float* r, int64_t G, double* scal, const int* done)
{
    if (*done) return;
    const float beta = (float)(scal[2] / scal[0]);
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < G; q += (int64_t)gridDim.x * blockDim.x)
        p[q] = r[q] + beta * p[q];
}

__global__ void k_cn_roll(double* scal, const int* done)
{
    if (*done) return;
    scal[0] = scal[2];
}

// data = x unless the initial residual already met the tolerance (src/paracrine.cu:114-116)
__global__ void k_cn_commit(float* u, const float* x, int64_t G, const int* done)
{
    if (*done == 2) return;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < G; q += (int64_t)gridDim.x * blockDim.x)
        u[q] = x[q];
}
}  // namespace

extern "C" nn_status nn_paracrine_ref_create(nn_ctx* ctx, const nn_paracrine_ref_params* p, int n, const float* d_x,
                                             const float* d_y, const float* d_z, float* d_g_paracrine,
                                             nn_paracrine** out)
{
    if (!ctx || !p || !out || n < 0 || p->nx < 2 || p->ny < 2 || p->nz < 2 || (n && (!d_x || !d_y || !d_z)))
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_paracrine_ref_create: bad argument");
    nn_paracrine* pm = new nn_paracrine();
    pm->ctx = ctx;
    nn_ctx_retain(ctx);
    pm->p = *p;
    pm->n = n;
    pm->G = (int64_t)p->nx * p->ny * p->nz;
    pm->g_out = d_g_paracrine;
    const size_t G = (size_t)pm->G, N = (size_t)(n > 0 ? n : 1);
    pm->nparts = nn_grid_for(ctx, pm->G, 256, 4);
    nn_status st = NN_OK;
#define PM_ALLOC(ptr, cnt) if (st == NN_OK) st = nn_alloc(ctx, &pm->ptr, cnt)
    PM_ALLOC(idx8, 8 * N); PM_ALLOC(w8, 8 * N);
    PM_ALLOC(u, G); PM_ALLOC(Ax, G); PM_ALLOC(lap, G); PM_ALLOC(x, G); PM_ALLOC(b, G);
    PM_ALLOC(r, G); PM_ALLOC(pv, G); PM_ALLOC(Ap, G);
    PM_ALLOC(at_neurons, N); PM_ALLOC(generated, N);
    PM_ALLOC(scal, 4); PM_ALLOC(partials, (size_t)pm->nparts); PM_ALLOC(ticket, 1); PM_ALLOC(done, 2);
#undef PM_ALLOC
    if (st != NN_OK) {
        nn_paracrine_destroy(pm);
        return st;
    }
    cudaStream_t s = ctx->stream;
    cudaMemsetAsync(pm->u, 0, sizeof(float) * G, s);
    cudaMemsetAsync(pm->generated, 0, sizeof(float) * N, s);
    cudaMemsetAsync(pm->at_neurons, 0, sizeof(float) * N, s);
    cudaMemsetAsync(pm->ticket, 0, sizeof(unsigned int), s);
    if (n > 0) {
        k_trilinear<<<nn_grid_for(ctx, n, 256, 16), 256, 0, s>>>(n, d_x, d_y, d_z, p->nx, p->ny, p->nz, p->h, pm->idx8,
                                                                  pm->w8);
        ctx->launches++;
        // constructor: interpolate the (zero) density and copy it out (src/paracrine.cuh:238-242)
        k_interp<<<nn_grid_for(ctx, n, 256, 16), 256, 0, s>>>(n, pm->idx8, pm->w8, pm->u, pm->G, pm->at_neurons,
                                                               pm->g_out);
        ctx->launches++;
    }
    st = nn_cuda_check(ctx, cudaGetLastError(), "nn_paracrine_ref_create");
    if (st != NN_OK) {
        nn_paracrine_destroy(pm);
        return st;
    }
    *out = pm;
    return NN_OK;
}

extern "C" nn_status nn_paracrine_destroy(nn_paracrine* pm)
{
    if (!pm) return NN_OK;
    if (pm->ctx) cudaStreamSynchronize(pm->ctx->stream);
    nn_release(pm->idx8); nn_release(pm->w8); nn_release(pm->u); nn_release(pm->Ax); nn_release(pm->lap);
    nn_release(pm->x); nn_release(pm->b); nn_release(pm->r); nn_release(pm->pv); nn_release(pm->Ap);
    nn_release(pm->at_neurons); nn_release(pm->generated); nn_release(pm->scal); nn_release(pm->partials);
    nn_release(pm->ticket); nn_release(pm->done);
    nn_ctx* ctx = pm->ctx;
    delete pm;
    nn_ctx_release(ctx);
    return NN_OK;
}

extern "C" float* nn_paracrine_density(nn_paracrine* pm) { return pm ? pm->u : nullptr; }
extern "C" float* nn_paracrine_sources(nn_paracrine* pm) { return pm ? pm->generated : nullptr; }

extern "C" nn_status nn_paracrine_ref_fine(nn_paracrine* pm, const nn_coupling* c)
{
    if (!pm || !c || c->n != pm->n) return nn_fail(pm ? pm->ctx : nullptr, NN_ERR_INVALID_ARG, "nn_paracrine_ref_fine: bad argument");
    if (pm->n == 0) return NN_OK;
    nn_ctx* ctx = pm->ctx;
    k_fine<<<nn_grid_for(ctx, pm->n, 256, 16), 256, 0, ctx->stream>>>(pm->n, c->firing, c->count, pm->generated,
                                                                       pm->p.coup_strength, pm->p.quirk_firing_list);
    NN_CHECK_LAUNCH(ctx, "k_fine");
    return NN_OK;
}

extern "C" nn_status nn_paracrine_ref_own(nn_paracrine* pm, int* iters, float* final_rr)
{
    if (!pm) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = pm->ctx;
    cudaStream_t s = ctx->stream;
    const auto& p = pm->p;
    const int64_t G = pm->G;
    const int gb = pm->nparts;
    const int nb = nn_grid_for(ctx, pm->n, 256, 16);
    // scatter_to_grid: Ax = G^T generated; density += Ax (src/paracrine.cu:276-287)
    NN_CUDA(ctx, cudaMemsetAsync(pm->Ax, 0, sizeof(float) * (size_t)G, s));
    if (pm->n > 0) {
        k_scatter<<<nb, 256, 0, s>>>(pm->n, pm->idx8, pm->w8, pm->generated, pm->Ax, G);
        NN_CHECK_LAUNCH(ctx, "k_scatter");
    }
    // update_density (src/paracrine.cu:63-134)
    const double h = p.h, dt = p.par_dt;
    Stencil27 L, A;
    static const float st[27] = {1, 3, 1, 3, 14, 3, 1, 3, 1, 3, 14, 3, 14, -128, 14, 3, 14, 3,
                                 1, 3, 1, 3, 14, 3, 1, 3, 1};
    for (int q = 0; q < 27; ++q) {
        const double lq = st[q] * (1.0 / (h * h * 30.0));
        L.k[q] = (float)lq;
        A.k[q] = (float)(-0.5 * p.D * dt * lq);
    }
    A.k[13] = (float)((double)A.k[13] + 1.0 + 0.5 * dt * p.decay);
    k_add<<<gb, 256, 0, s>>>(pm->u, pm->Ax, G);  // density += Ax
    NN_CHECK_LAUNCH(ctx, "k_add");
    k_conv27<<<gb, 256, 0, s>>>(pm->u, pm->lap, p.nx, p.ny, p.nz, L, nullptr);
    NN_CHECK_LAUNCH(ctx, "k_conv27(L)");
    const double c = p.quirk_rhs ? h : dt;
    k_cn_init<<<gb, 256, 0, s>>>(pm->u, pm->lap, pm->x, pm->b, G, (float)(1.0 - dt * p.decay), (float)(dt * p.D),
                                 (float)(1.0 - c * p.decay / 2.0), (float)(c * p.D / 2.0));
    NN_CHECK_LAUNCH(ctx, "k_cn_init");
    k_conv27<<<gb, 256, 0, s>>>(pm->x, pm->Ap, p.nx, p.ny, p.nz, A, nullptr);
    NN_CHECK_LAUNCH(ctx, "k_conv27(A x0)");
    NN_CUDA(ctx, cudaMemsetAsync(pm->done, 0, 2 * sizeof(int), s));
    k_cn_residual<<<gb, 256, 0, s>>>(pm->b, pm->Ap, pm->r, pm->pv, G, pm->partials, pm->ticket, pm->scal, pm->done,
                                     p.abs_tol);
    NN_CHECK_LAUNCH(ctx, "k_cn_residual");
    for (int it = 0; it < p.max_iter; ++it) {
        k_conv27<<<gb, 256, 0, s>>>(pm->pv, pm->Ap, p.nx, p.ny, p.nz, A, pm->done);
        NN_CHECK_LAUNCH(ctx, "k_conv27(A p)");
        k_cn_pap<<<gb, 256, 0, s>>>(pm->pv, pm->Ap, G, pm->partials, pm->ticket, pm->scal, pm->done);
        NN_CHECK_LAUNCH(ctx, "k_cn_pap");
        k_cn_update<<<gb, 256, 0, s>>>(pm->x, pm->r, pm->pv, pm->Ap, G, pm->partials, pm->ticket, pm->scal, pm->done,
                                       p.abs_tol, pm->done + 1);
        NN_CHECK_LAUNCH(ctx, "k_cn_update");
        k_cn_direction<<<gb, 256, 0, s>>>(pm->pv, pm->r, G, pm->scal, pm->done);
        NN_CHECK_LAUNCH(ctx, "k_cn_direction");
        k_cn_roll<<<1, 1, 0, s>>>(pm->scal, pm->done);
        NN_CHECK_LAUNCH(ctx, "k_cn_roll");
    }
    k_cn_commit<<<gb, 256, 0, s>>>(pm->u, pm->x, G, pm->done);
    NN_CHECK_LAUNCH(ctx, "k_cn_commit");
    // interpolate, reset sources, copy out (src/paracrine.cuh:259-264)
    if (pm->n > 0) {
        k_interp<<<nb, 256, 0, s>>>(pm->n, pm->idx8, pm->w8, pm->u, G, pm->at_neurons, pm->g_out);
        NN_CHECK_LAUNCH(ctx, "k_interp");
        NN_CUDA(ctx, cudaMemsetAsync(pm->generated, 0, sizeof(float) * (size_t)pm->n, s));
    }
    if (std::getenv("NN_DEBUG_PARACRINE")) {
        int h_done[2];
        double h_scal[3];
        std::vector<float> hu((size_t)G), hx((size_t)G), hax((size_t)G);
        cudaMemcpyAsync(h_done, pm->done, sizeof h_done, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(h_scal, pm->scal, sizeof h_scal, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hu.data(), pm->u, sizeof(float) * (size_t)G, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hx.data(), pm->x, sizeof(float) * (size_t)G, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hax.data(), pm->Ax, sizeof(float) * (size_t)G, cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        double su = 0, sx = 0, sa = 0;
        for (int64_t q = 0; q < G; ++q) { su += hu[(size_t)q]; sx += hx[(size_t)q]; sa += hax[(size_t)q]; }
        fprintf(stderr, "[paracrine] done=%d iters=%d rr0=%g pAp=%g rr=%g sum(u)=%.9g sum(x)=%.9g sum(Ax)=%.9g\n",
                h_done[0], h_done[1], h_scal[0], h_scal[1], h_scal[2], su, sx, sa);
    }
    if (iters || final_rr) {
        int h_done[2];
        double h_scal[3];
        NN_CUDA(ctx, cudaMemcpyAsync(h_done, pm->done, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
        NN_CUDA(ctx, cudaMemcpyAsync(h_scal, pm->scal, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
        NN_CUDA(ctx, cudaStreamSynchronize(s));
        if (iters) *iters = h_done[1];
        if (final_rr) *final_rr = (float)(h_done[1] == 0 ? h_scal[0] : (h_done[0] == 1 ? h_scal[2] : h_scal[0]));
    }
    return NN_OK;
}
