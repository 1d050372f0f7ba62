// Context, error reporting, memory helpers and device utilities (scan, CSC
// transpose) of libneuronephys.
#include <cmath>
#include <cstring>

#include "nn_internal.cuh"

// ------------------------------------------------------------ errors --------

nn_status nn_fail(nn_ctx* ctx, nn_status st, const char* fmt, ...)
{
    if (ctx) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return st;
}

nn_status nn_cuda_check(nn_ctx* ctx, cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return NN_OK;
    cudaGetLastError();  // clear a non-sticky error
    return nn_fail(ctx, e == cudaErrorMemoryAllocation ? NN_ERR_OOM : NN_ERR_CUDA, "%s: %s (%s)", what,
                   cudaGetErrorString(e), cudaGetErrorName(e));
}

extern "C" const char* nn_status_string(nn_status s)
{
    switch (s) {
        case NN_OK: return "ok";
        case NN_ERR_INVALID_ARG: return "invalid argument";
        case NN_ERR_OOM: return "out of device memory";
        case NN_ERR_CUDA: return "CUDA error";
        case NN_ERR_NOT_CONVERGED: return "solver did not converge";
        case NN_ERR_NUMERIC: return "non-finite neuron state";
        case NN_ERR_TIMEOUT: return "device-side wait timed out";
        case NN_ERR_UNSUPPORTED: return "unsupported";
        case NN_ERR_NO_DEVICE: return "no CUDA device";
    }
    return "unknown status";
}

extern "C" int nn_version(void) { return 100; }

// ------------------------------------------------------------ context -------

extern "C" nn_status nn_ctx_create(int device, nn_ctx** out)
{
    if (!out) return NN_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return NN_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) return NN_ERR_INVALID_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return NN_ERR_CUDA;
    nn_ctx* c = new nn_ctx();
    c->device = device;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return NN_ERR_CUDA;
    }
    *out = c;
    return NN_OK;
}

void nn_ctx_retain(nn_ctx* ctx)
{
    if (ctx) ++ctx->refs;
}

void nn_ctx_release(nn_ctx* ctx)
{
    if (!ctx || --ctx->refs > 0) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

// Drops the caller's reference; objects still alive on the context keep it
// (and its stream) until they are destroyed.
extern "C" nn_status nn_ctx_destroy(nn_ctx* ctx)
{
    if (!ctx) return NN_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    nn_ctx_release(ctx);
    return NN_OK;
}

extern "C" const char* nn_ctx_last_error(const nn_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

extern "C" nn_status nn_ctx_synchronize(nn_ctx* ctx)
{
    if (!ctx) return NN_ERR_INVALID_ARG;
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return NN_OK;
}

extern "C" int64_t nn_ctx_kernel_launches(const nn_ctx* ctx) { return ctx ? ctx->launches : 0; }

extern "C" int nn_ctx_num_sms(const nn_ctx* ctx) { return ctx ? ctx->num_sms : 0; }

extern "C" void* nn_ctx_stream(nn_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

extern "C" nn_status nn_ctx_time_begin(nn_ctx* ctx)
{
    if (!ctx) return NN_ERR_INVALID_ARG;
    if (!ctx->ev0) {
        NN_CUDA(ctx, cudaEventCreate(&ctx->ev0));
        NN_CUDA(ctx, cudaEventCreate(&ctx->ev1));
    }
    NN_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    return NN_OK;
}

extern "C" nn_status nn_ctx_time_end(nn_ctx* ctx, float* ms)
{
    if (!ctx || !ms || !ctx->ev0) return NN_ERR_INVALID_ARG;
    NN_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    NN_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
    NN_CUDA(ctx, cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
    return NN_OK;
}

extern "C" nn_status nn_host_alloc(size_t bytes, void** hptr)
{
    if (!hptr) return NN_ERR_INVALID_ARG;
    *hptr = nullptr;
    cudaError_t e = cudaMallocHost(hptr, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *hptr = nullptr;
        return e == cudaErrorMemoryAllocation ? NN_ERR_OOM : NN_ERR_CUDA;
    }
    return NN_OK;
}

extern "C" nn_status nn_host_free(void* hptr)
{
    if (hptr) cudaFreeHost(hptr);
    return NN_OK;
}

extern "C" nn_status nn_malloc(nn_ctx* ctx, size_t bytes, void** dptr)
{
    if (!ctx || !dptr) return NN_ERR_INVALID_ARG;
    char* p = nullptr;
    NN_TRY(nn_alloc(ctx, &p, bytes));
    *dptr = p;
    return NN_OK;
}

extern "C" nn_status nn_free(nn_ctx* ctx, void* dptr)
{
    if (!ctx) return NN_ERR_INVALID_ARG;
    if (!dptr) return NN_OK;
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    NN_CUDA(ctx, cudaFree(dptr));
    return NN_OK;
}

extern "C" nn_status nn_memcpy_h2d(nn_ctx* ctx, void* dst, const void* src, size_t bytes)
{
    if (!ctx || (bytes && (!dst || !src))) return NN_ERR_INVALID_ARG;
    if (!bytes) return NN_OK;
    NN_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return NN_OK;
}

extern "C" nn_status nn_memcpy_d2h(nn_ctx* ctx, void* dst, const void* src, size_t bytes)
{
    if (!ctx || (bytes && (!dst || !src))) return NN_ERR_INVALID_ARG;
    if (!bytes) return NN_OK;
    NN_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return NN_OK;
}

extern "C" nn_status nn_memset_d(nn_ctx* ctx, void* dst, int value, size_t bytes)
{
    if (!ctx || (bytes && !dst)) return NN_ERR_INVALID_ARG;
    if (!bytes) return NN_OK;
    NN_CUDA(ctx, cudaMemsetAsync(dst, value, bytes, ctx->stream));
    return NN_OK;
}

// ------------------------------------------------------------ scan ----------
// Exclusive prefix sum of int64 in three passes: block totals, a single-block
// scan of the totals, then the in-block scan plus the block offset.

namespace {
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ int64_t warp_incl_scan(int64_t v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ int64_t block_excl_scan(int64_t v, int64_t* excl)
{
    __shared__ int64_t warp_tot[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int64_t inc = warp_incl_scan(v);
    if (lane == 31) warp_tot[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int64_t t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
        t = warp_incl_scan(t);
        warp_tot[lane] = t;
    }
    __syncthreads();
    int64_t base = wid ? warp_tot[wid - 1] : 0;
    *excl = base + inc - v;
    int64_t total = warp_tot[(blockDim.x >> 5) - 1];
    __syncthreads();
    return total;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_totals(const int64_t* in, int64_t n, int64_t* totals)
{
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int64_t s = 0;
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS; ++q)
        if (base + q < n) s += in[base + q];
    int64_t dummy;
    int64_t tot = block_excl_scan(s, &dummy);
    if (threadIdx.x == 0) totals[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_single(int64_t* totals, int64_t nb)
{
    int64_t carry = 0;
    for (int64_t off = 0; off < nb; off += SCAN_THREADS) {
        int64_t i = off + threadIdx.x;
        int64_t v = i < nb ? totals[i] : 0;
        int64_t ex;
        int64_t tot = block_excl_scan(v, &ex);
        if (i < nb) totals[i] = carry + ex;
        carry += tot;
    }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const int64_t* in, int64_t* out, int64_t n,
                                                             const int64_t* offsets)
{
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int64_t v[SCAN_ITEMS];
    int64_t s = 0;
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS; ++q) {
        v[q] = base + q < n ? in[base + q] : 0;
        s += v[q];
    }
    int64_t ex;
    block_excl_scan(s, &ex);
    int64_t run = offsets[blockIdx.x] + ex;
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS; ++q) {
        if (base + q < n) out[base + q] = run;
        run += v[q];
    }
}
}  // namespace

nn_status nn_scan_exclusive_i64(nn_ctx* ctx, const int64_t* d_in, int64_t* d_out, int64_t n)
{
    if (n <= 0) return NN_OK;
    int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    int64_t* totals = nullptr;
    NN_TRY(nn_alloc(ctx, &totals, (size_t)nb));
    k_scan_totals<<<(unsigned)nb, SCAN_THREADS, 0, ctx->stream>>>(d_in, n, totals);
    NN_CHECK_LAUNCH(ctx, "k_scan_totals");
    k_scan_single<<<1, SCAN_THREADS, 0, ctx->stream>>>(totals, nb);
    NN_CHECK_LAUNCH(ctx, "k_scan_single");
    k_scan_apply<<<(unsigned)nb, SCAN_THREADS, 0, ctx->stream>>>(d_in, d_out, n, totals);
    NN_CHECK_LAUNCH(ctx, "k_scan_apply");
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFree(totals);
    return NN_OK;
}

// ------------------------------------------------------------ CSC -----------
// Deterministic CSR -> CSC: count in-degrees, scan, place edge ids with
// atomics, then sort each column's edge ids so entries appear in ascending CSR
// position (the order a stable counting sort gives).

namespace {
__global__ void k_count_cols(const int32_t* col, int64_t nnz, unsigned long long* cnt)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(cnt + col[e], 1ull);
}

__global__ void k_place(const int32_t* col, int64_t nnz, unsigned long long* cursor, uint32_t* edge_of)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x) {
        unsigned long long pos = atomicAdd(cursor + col[e], 1ull);
        edge_of[pos] = (uint32_t)e;
    }
}

constexpr int WARP_SORT_MAX = 1024;
constexpr int BLOCK_SORT_MAX = 16384;

// Bitonic sort of P (power of two) keys in shared memory by `nthreads`
// threads starting at thread index `tid`.
template <bool WARP>
__device__ void bitonic_sort(uint32_t* s, int P, int tid, int nthreads)
{
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < P; i += nthreads) {
                int p = i ^ j;
                if (p > i) {
                    uint32_t a = s[i], b = s[p];
                    bool up = (i & k) == 0;
                    if ((a > b) == up) { s[i] = b; s[p] = a; }
                }
            }
            if (WARP) __syncwarp(); else __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(256) k_sort_short(const int64_t* col_ptr, int n, uint32_t* edge_of,
                                                    int* long_list, int* long_count)
{
    __shared__ uint32_t sm[8][WARP_SORT_MAX];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t* s = sm[w];
    for (int c = blockIdx.x * 8 + w; c < n; c += gridDim.x * 8) {
        const int64_t beg = col_ptr[c];
        const int len = (int)(col_ptr[c + 1] - beg);
        if (len <= 1) continue;
        if (len > WARP_SORT_MAX) {
            if (lane == 0) long_list[atomicAdd(long_count, 1)] = c;
            continue;
        }
        int P = 1;
        while (P < len) P <<= 1;
        for (int i = lane; i < P; i += 32) s[i] = i < len ? edge_of[beg + i] : 0xffffffffu;
        __syncwarp();
        bitonic_sort<true>(s, P, lane, 32);
        for (int i = lane; i < len; i += 32) edge_of[beg + i] = s[i];
        __syncwarp();
    }
}

__global__ void __launch_bounds__(1024) k_sort_long(const int64_t* col_ptr, const int* list, int count,
                                                    uint32_t* edge_of, uint32_t* tmp)
{
    extern __shared__ uint32_t s[];
    for (int q = blockIdx.x; q < count; q += gridDim.x) {
        const int c = list[q];
        const int64_t beg = col_ptr[c];
        const int64_t len = col_ptr[c + 1] - beg;
        if (len <= BLOCK_SORT_MAX) {
            int P = 1;
            while (P < len) P <<= 1;
            for (int i = threadIdx.x; i < P; i += blockDim.x) s[i] = i < len ? edge_of[beg + i] : 0xffffffffu;
            __syncthreads();
            bitonic_sort<false>(s, P, threadIdx.x, blockDim.x);
            for (int i = threadIdx.x; i < len; i += blockDim.x) edge_of[beg + i] = s[i];
            __syncthreads();
        } else {
            // rank sort for very long columns (keys are distinct edge ids)
            for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
                const uint32_t key = edge_of[beg + i];
                int64_t rank = 0;
                for (int64_t j = 0; j < len; ++j) rank += edge_of[beg + j] < key;
                tmp[beg + rank] = key;
            }
            __syncthreads();
            for (int64_t i = threadIdx.x; i < len; i += blockDim.x) edge_of[beg + i] = tmp[beg + i];
            __syncthreads();
        }
    }
}
}  // namespace

nn_status nn_build_csc(nn_ctx* ctx, int n, int64_t nnz, const int64_t* d_row_ptr, const int32_t* d_col,
                       int64_t* d_col_ptr, uint32_t* d_edge_of)
{
    (void)d_row_ptr;
    if (nnz >= (int64_t)0xffffffffu) return nn_fail(ctx, NN_ERR_UNSUPPORTED, "CSC build supports < 2^32 synapses");
    unsigned long long* cnt = nullptr;
    NN_TRY(nn_alloc(ctx, &cnt, (size_t)n + 1));
    NN_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * ((size_t)n + 1), ctx->stream));
    if (nnz > 0) {
        k_count_cols<<<nn_grid_for(ctx, nnz, 256, 16), 256, 0, ctx->stream>>>(d_col, nnz, cnt);
        NN_CHECK_LAUNCH(ctx, "k_count_cols");
    }
    NN_TRY(nn_scan_exclusive_i64(ctx, (const int64_t*)cnt, d_col_ptr, (int64_t)n + 1));
    if (nnz > 0) {
        NN_CUDA(ctx, cudaMemcpyAsync(cnt, d_col_ptr, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyDeviceToDevice,
                                     ctx->stream));
        k_place<<<nn_grid_for(ctx, nnz, 256, 16), 256, 0, ctx->stream>>>(d_col, nnz, cnt, d_edge_of);
        NN_CHECK_LAUNCH(ctx, "k_place");
        int* long_list = nullptr;
        int* long_count = nullptr;
        NN_TRY(nn_alloc(ctx, &long_list, (size_t)n));
        NN_TRY(nn_alloc(ctx, &long_count, 1));
        NN_CUDA(ctx, cudaMemsetAsync(long_count, 0, sizeof(int), ctx->stream));
        k_sort_short<<<nn_grid_for(ctx, (int64_t)n * 32, 256, 8), 256, 0, ctx->stream>>>(d_col_ptr, n, d_edge_of,
                                                                                           long_list, long_count);
        NN_CHECK_LAUNCH(ctx, "k_sort_short");
        int h_long = 0;
        NN_CUDA(ctx, cudaMemcpyAsync(&h_long, long_count, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (h_long > 0) {
            uint32_t* tmp = nullptr;
            NN_TRY(nn_alloc(ctx, &tmp, (size_t)nnz));
            const size_t smem = BLOCK_SORT_MAX * sizeof(uint32_t);
            NN_CUDA(ctx, cudaFuncSetAttribute(k_sort_long, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k_sort_long<<<nn_grid_for(ctx, h_long, 1, 2), 1024, smem, ctx->stream>>>(d_col_ptr, long_list, h_long,
                                                                                     d_edge_of, tmp);
            NN_CHECK_LAUNCH(ctx, "k_sort_long");
            NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            cudaFree(tmp);
        }
        cudaFree(long_list);
        cudaFree(long_count);
    }
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFree(cnt);
    return NN_OK;
}

// ------------------------------------------------------------ tables --------

double nn_host_inv_phi(double pr)
{
    double lo = -40.0, hi = 40.0;
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        const double c = 0.5 * std::erfc(-mid / std::sqrt(2.0));
        if (c < pr) lo = mid; else hi = mid;
    }
    return 0.5 * (lo + hi);
}

void nn_host_gauss_table(double sigma_sites, int16_t* table)
{
    for (int m = 0; m < 4096; ++m) {
        const double z = nn_host_inv_phi(((double)m + 0.5) / 4096.0);
        table[m] = (int16_t)std::lround(sigma_sites * z);
    }
}
