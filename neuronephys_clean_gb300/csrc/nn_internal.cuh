// Internal declarations shared by the translation units of libneuronephys.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "neuronephys.h"

// ----------------------------------------------------------------- context --
struct nn_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    int64_t launches = 0;  // kernels launched on behalf of the caller
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // nn_ctx_time_begin/end
    // Objects created on a context hold a reference, so destroying the context
    // before them (in any order) never leaves them with a dangling pointer.
    int refs = 1;
};

// Take / drop a reference; the last release frees the context.
void nn_ctx_retain(nn_ctx* ctx);
void nn_ctx_release(nn_ctx* ctx);

nn_status nn_fail(nn_ctx* ctx, nn_status st, const char* fmt, ...);
nn_status nn_cuda_check(nn_ctx* ctx, cudaError_t e, const char* what);

#define NN_CUDA(ctx, expr)                                                   \
    do {                                                                     \
        cudaError_t e_ = (expr);                                             \
        if (e_ != cudaSuccess) return nn_cuda_check((ctx), e_, #expr);       \
    } while (0)

#define NN_CHECK_LAUNCH(ctx, what)                                           \
    do {                                                                     \
        cudaError_t e_ = cudaGetLastError();                                 \
        if (e_ != cudaSuccess) return nn_cuda_check((ctx), e_, what);        \
        (ctx)->launches++;                                                   \
    } while (0)

#define NN_TRY(expr)                                                         \
    do {                                                                     \
        nn_status s_ = (expr);                                               \
        if (s_ != NN_OK) return s_;                                          \
    } while (0)

template <class T>
nn_status nn_alloc(nn_ctx* ctx, T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) return NN_OK;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return nn_fail(ctx, e == cudaErrorMemoryAllocation ? NN_ERR_OOM : NN_ERR_CUDA,
                       "cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
    }
    return NN_OK;
}

template <class T>
void nn_release(T*& p)
{
    if (p) cudaFree((void*)p);
    p = nullptr;
}

// The context stream is non-blocking: legacy-stream copies and memsets are
// not ordered with its kernels.  These go through the context stream.
inline cudaError_t nn_copy_sync(nn_ctx* ctx, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind)
{
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e;
}
inline cudaError_t nn_zero_async(nn_ctx* ctx, void* p, size_t bytes) { return cudaMemsetAsync(p, 0, bytes, ctx->stream); }

// Programmatic dependent launch: the kernel may begin while the kernel before
// it on the stream finishes (its launch and prologue overlap that kernel's
// tail).  Such a kernel calls nn_grid_dep_wait() before it touches any memory
// the kernels before it write or read; without a programmatic dependency the
// wait returns at once.
template <typename... KArgs, typename... Args>
inline cudaError_t nn_launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                 Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at;
    at.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at.val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = &at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}
__device__ __forceinline__ void nn_grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

inline int nn_grid_for(const nn_ctx* ctx, int64_t work, int threads, int per_sm = 8)
{
    int64_t b = (work + threads - 1) / threads;
    int64_t cap = (int64_t)ctx->num_sms * per_sm;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

// ---------------------------------------------------------- counter RNG --
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11).  Streams are addressed by (seed; a, b, c, purpose).
enum nn_rng_purpose : uint32_t {
    NN_P_NOISE = 1, NN_P_DRIVE = 2, NN_P_POS = 3, NN_P_ER = 4, NN_P_GAUSS = 5,
    NN_P_WEIGHT = 6, NN_P_TYPE = 7, NN_P_BLOCK = 8, NN_P_REGION = 9
};

struct nn_u4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ void nn_mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo)
{
#ifdef __CUDA_ARCH__
    hi = __umulhi(a, b);
    lo = a * b;
#else
    uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
#endif
}

__host__ __device__ __forceinline__ nn_u4 nn_philox(uint64_t seed, uint32_t a, uint32_t b, uint32_t c, uint32_t purpose)
{
    uint32_t c0 = a, c1 = b, c2 = c, c3 = purpose;
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        nn_mulhilo(0xD2511F53u, c0, hi0, lo0);
        nn_mulhilo(0xCD9E8D57u, c2, hi1, lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return nn_u4{c0, c1, c2, c3};
}

// Philox2x32-10 (same paper): the neuron-update noise stream, one draw per
// neuron pair and step.
__host__ __device__ __forceinline__ void nn_philox2(uint32_t key, uint32_t c0, uint32_t c1, uint32_t& o0, uint32_t& o1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi, lo;
        nn_mulhilo(0xD256D193u, c0, hi, lo);
        const uint32_t n0 = hi ^ key ^ c1;
        c1 = lo;
        c0 = n0;
        key += 0x9E3779B9u;
    }
    o0 = c0;
    o1 = c1;
}

// its key: both seed words and the high step word mixed into one word
__host__ __device__ __forceinline__ uint32_t nn_noise_key(uint64_t seed, uint64_t step)
{
    return (uint32_t)seed + 0x9E3779B9u * (uint32_t)(seed >> 32) + 0x85EBCA6Bu * (uint32_t)(step >> 32);
}

// uniform in [0,1) and (0,1] with 24 random bits (exact in float)
__host__ __device__ __forceinline__ float nn_u01f(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }
__host__ __device__ __forceinline__ float nn_u01f_open(uint32_t x) { return (float)((x >> 8) + 1u) * (1.0f / 16777216.0f); }
__host__ __device__ __forceinline__ double nn_u01d(uint32_t x) { return (double)(x >> 8) * (1.0 / 16777216.0); }
__host__ __device__ __forceinline__ double nn_u01d_open(uint32_t x) { return (double)((x >> 8) + 1u) * (1.0 / 16777216.0); }

// Lattice side of the jittered-lattice layout: smallest L with L^3 >= n.
__host__ __device__ inline int nn_lattice_side(int n)
{
    int L = 1;
    while ((int64_t)L * L * L < n) ++L;
    return L;
}

// ------------------------------------------------------ shared host helpers --
nn_status nn_scan_exclusive_i64(nn_ctx* ctx, const int64_t* d_in, int64_t* d_out, int64_t n);
nn_status nn_build_csc(nn_ctx* ctx, int n, int64_t nnz, const int64_t* d_row_ptr, const int32_t* d_col,
                       int64_t* d_col_ptr, uint32_t* d_edge_of);
struct nn_pcg;
nn_status nn_pcg_run_best(nn_pcg* pc, const float* d_b, float* d_x, double rtol, int max_iter, int* iters,
                          double* relres, int* converged);
// operator data of a PCG object: dims, 1/diag (per cell, or the constant
// when invd is null), the caller's cell field D (may be null)
void nn_pcg_info(const nn_pcg* pc, nn_ctx** ctx, int* nx, int* ny, int* nz, const float** invd, float* invd_const,
                 const float** D);
// The operator's coefficients: A = (1 + beta) I + alpha L_D.
void nn_pcg_coefficients(const nn_pcg* pc, double* alpha, double* beta);

// multigrid internals (nn_mg.cu) used by the learned coarse solver (nn_unet.cu)
struct nn_mg;
// replaces the treatment of one level: x = solve(b) on that level's grid,
// followed by the V-cycle's post-smoothing there; enqueued on the context
// stream, never synchronising (it may run inside a captured graph)
typedef nn_status (*nn_mg_level_fn)(void* user, const float* d_b, float* d_x);
// sees the right-hand side reaching one level in each V-cycle (enqueue only)
typedef nn_status (*nn_mg_record_fn)(void* user, const float* d_b);
nn_status nn_mg_set_level_solver(nn_mg* mg, int level, nn_mg_level_fn fn, void* user);  // fn null: classical
nn_status nn_mg_set_recorder(nn_mg* mg, int level, nn_mg_record_fn fn, void* user);    // fn null: off
nn_status nn_mg_set_level_sweeps(nn_mg* mg, int sweeps);  // smoothing sweeps after the level solver (default 2)
// dims and diagonal of level >= 1
nn_status nn_mg_level_dims(const nn_mg* mg, int level, int* nx, int* ny, int* nz, const float** diag);
// Jacobi-PCG on level >= 1 from x = 0 to rtol (synchronising; for training targets)
nn_status nn_mg_level_cg(nn_mg* mg, int level, const float* d_b, float* d_x, double rtol, int max_iter, int* iters);

// batched PCG (nn_bpcg.cu)
int64_t nn_bpcg_cells(const nn_bpcg* bp);
const int64_t* nn_bpcg_offsets(const nn_bpcg* bp);
void nn_bpcg_set_timing(nn_bpcg* bp, bool on);
void nn_bpcg_last_timing(const nn_bpcg* bp, float* ms, int* iters);
// asynchronous solve on a stream (no host read until finish)
nn_status nn_bpcg_async_begin(nn_bpcg* bp, const float* d_b, float* d_x, double rtol, int max_iter, int n,
                              cudaStream_t cs);
nn_status nn_bpcg_async_finish(nn_bpcg* bp, int* h_iters, int* max_iters, int* unconverged);
int nn_bpcg_cells_per_block(const nn_bpcg* bp);

struct nn_cg_plan;
nn_status nn_cg_plan_create(nn_ctx* ctx, int nx, int ny, int nz, double alpha, double beta, const float* D,
                            const float* invdv, nn_cg_plan** out);
void nn_cg_plan_destroy(nn_cg_plan* pl);
nn_status nn_cg_run(nn_cg_plan* pl, const float* d_b, float* d_x, double rtol, int max_iter, int* iters,
                    double* relres, int* converged);
void nn_cg_set_timing(nn_cg_plan* pl, bool on);
nn_status nn_cg_async_begin(nn_cg_plan* pl, const float* d_b, float* d_x, double rtol, int max_iter, int n,
                            cudaStream_t cs);
nn_status nn_cg_async_more(nn_cg_plan* pl, int n);
nn_status nn_cg_async_finish(nn_cg_plan* pl, int* iters, double* relres, int* converged);
nn_status nn_pcg_async_begin(nn_pcg* pc, const float* d_b, float* d_x, double rtol, int max_iter, int n,
                             cudaStream_t cs);
nn_status nn_pcg_async_finish(nn_pcg* pc, int* iters, double* relres, int* converged);
bool nn_pcg_async_supported(const nn_pcg* pc);
void nn_cg_last_timing(const nn_cg_plan* pl, float* ms, int* iters);
nn_status nn_cg_plan_autotune(nn_cg_plan* pl, const float* d_b, float* d_x, int iters, int* zc_out, float* ms_out);
int nn_cg_plan_tile_depth(const nn_cg_plan* pl);
void nn_cg_plan_set_tile_depth(nn_cg_plan* pl, int zc);
struct nn_pcg;
nn_status nn_pcg_autotune_tiles(nn_pcg* pc, int iters, int* tile_z, float* ms_per_iter);
int nn_pcg_tile_depth(const nn_pcg* pc);
void nn_pcg_set_tile_depth(nn_pcg* pc, int zc);
double nn_host_inv_phi(double p);
void nn_host_gauss_table(double sigma_sites, int16_t* table4096);

// Device warp helpers
__device__ __forceinline__ double nn_warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float nn_warp_sumf(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
