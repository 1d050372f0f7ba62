// On-disk connectivity and positions, and the reference's sub-sampling of
// them (FileNetwork, src/network_factory.cu:154-211; FileMorphology,
// src/morphology.cpp:260-330).
//
// The reference reads HDF5 datasets /row_ptr, /col_idx (int32) and /x, /y,
// /z (float32).  No HDF5 library exists in this build, so the same datasets
// travel in a raw little-endian container:
//   connectivity: "NNCSR001" | int64 n_rows | int64 nnz | int32 row_ptr[n_rows + 1] | int32 col_idx[nnz]
//   positions:    "NNPOS001" | int64 n | float32 x[n] | float32 y[n] | float32 z[n]
// Sub-sampling N of n_rows neurons keeps every sparsity-th row (sparsity =
// n_rows / N) and, within it, the targets divisible by sparsity (renumbered
// target / sparsity): a device count pass, a scan and a fill that keeps the
// file's target order.  Positions take every stride-th point (stride = n / N)
// and map the bounding box of all n points onto [-1, 1] with the reference's
// FP32 operation order (translate by -min, scale by 2 / (max - min),
// translate by -1), without contraction so the result is bit-identical.
#include <cstdio>
#include <cstring>
#include <vector>

#include "nn_internal.cuh"

namespace {
const char CSR_MAGIC[8] = {'N', 'N', 'C', 'S', 'R', '0', '0', '1'};
const char POS_MAGIC[8] = {'N', 'N', 'P', 'O', 'S', '0', '0', '1'};

struct File {
    FILE* f = nullptr;
    explicit File(const char* path, const char* mode) { f = std::fopen(path, mode); }
    ~File() { if (f) std::fclose(f); }
};

bool read_exact(FILE* f, void* p, size_t bytes) { return std::fread(p, 1, bytes, f) == bytes; }
bool write_exact(FILE* f, const void* p, size_t bytes) { return std::fwrite(p, 1, bytes, f) == bytes; }

__global__ void k_sub_count(const int32_t* row_ptr, const int32_t* col, int N, int sparsity, int64_t* cnt)
{
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = gw; i < N; i += nw) {
        const int64_t r = (int64_t)i * sparsity;
        int c = 0;
        for (int e = row_ptr[r] + lane; e < row_ptr[r + 1]; e += 32) c += (col[e] % sparsity) == 0;
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if (lane == 0) cnt[i] = c;
    }
}

// kept targets of row i in file order: warp ballot + prefix per 32-entry chunk
__global__ void k_sub_fill(const int32_t* row_ptr, const int32_t* col, int N, int sparsity, const int64_t* out_ptr,
                           int32_t* out_col)
{
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = gw; i < N; i += nw) {
        const int64_t r = (int64_t)i * sparsity;
        int64_t pos = out_ptr[i];
        const int beg = row_ptr[r], end = row_ptr[r + 1];
        for (int e0 = beg; e0 < end; e0 += 32) {
            const int e = e0 + lane;
            const bool keep = e < end && (col[e] % sparsity) == 0;
            const unsigned m = __ballot_sync(0xffffffffu, keep);
            if (keep) out_col[pos + __popc(m & ((1u << lane) - 1u))] = col[e] / sparsity;
            pos += __popc(m);
        }
    }
}

__global__ void k_minmax(const float* v, int64_t n, float* out)  // out[0] min, out[1] max (one block)
{
    __shared__ float smin[32], smax[32];
    float lo = INFINITY, hi = -INFINITY;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        lo = fminf(lo, v[i]);
        hi = fmaxf(hi, v[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        smin[threadIdx.x >> 5] = lo;
        smax[threadIdx.x >> 5] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            lo = fminf(lo, smin[w]);
            hi = fmaxf(hi, smax[w]);
        }
        out[0] = fminf(lo, smin[0]);
        out[1] = fmaxf(hi, smax[0]);
    }
}

__global__ void k_pos_sample(const float* x, const float* y, const float* z, const float* mm, int N, int64_t stride,
                             float* ox, float* oy, float* oz)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const int64_t j = stride * i;
        const float* src[3] = {x, y, z};
        float* dst[3] = {ox, oy, oz};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float lo = mm[2 * a], hi = mm[2 * a + 1];
            const float scale = __fdiv_rn(2.0f, __fsub_rn(hi, lo));
            const float t = __fadd_rn(src[a][j], -lo);
            dst[a][i] = __fadd_rn(__fmul_rn(t, scale), -1.0f);
        }
    }
}
}  // namespace

extern "C" nn_status nn_net_file_write(const char* path, int64_t n_rows, int64_t nnz, const int32_t* h_row_ptr,
                                       const int32_t* h_col)
{
    if (!path || n_rows < 1 || nnz < 0 || !h_row_ptr || (nnz > 0 && !h_col)) return NN_ERR_INVALID_ARG;
    File f(path, "wb");
    if (!f.f) return NN_ERR_INVALID_ARG;
    const bool ok = write_exact(f.f, CSR_MAGIC, 8) && write_exact(f.f, &n_rows, 8) && write_exact(f.f, &nnz, 8) &&
                    write_exact(f.f, h_row_ptr, sizeof(int32_t) * (n_rows + 1)) &&
                    write_exact(f.f, h_col, sizeof(int32_t) * nnz);
    return ok ? NN_OK : NN_ERR_INVALID_ARG;
}

// Two calls: with NULL arrays returns the sizes; then fills the arrays.
extern "C" nn_status nn_net_file_read(const char* path, int64_t* n_rows, int64_t* nnz, int32_t* h_row_ptr,
                                      int32_t* h_col)
{
    if (!path || !n_rows || !nnz) return NN_ERR_INVALID_ARG;
    File f(path, "rb");
    if (!f.f) return NN_ERR_INVALID_ARG;
    char magic[8];
    int64_t nr = 0, nz = 0;
    if (!read_exact(f.f, magic, 8) || std::memcmp(magic, CSR_MAGIC, 8) || !read_exact(f.f, &nr, 8) ||
        !read_exact(f.f, &nz, 8) || nr < 1 || nz < 0)
        return NN_ERR_INVALID_ARG;
    *n_rows = nr;
    *nnz = nz;
    if (!h_row_ptr) return NN_OK;
    if (!read_exact(f.f, h_row_ptr, sizeof(int32_t) * (nr + 1))) return NN_ERR_INVALID_ARG;
    if (h_col && !read_exact(f.f, h_col, sizeof(int32_t) * nz)) return NN_ERR_INVALID_ARG;
    return NN_OK;
}

// Sub-sample N neurons of an n_rows-row CSR already on the device.  Outputs:
// d_out_row_ptr[N + 1] (int64) and d_out_col (capacity: the input nnz); the
// kept synapse count to *out_nnz.
extern "C" nn_status nn_net_subsample(nn_ctx* ctx, const int32_t* d_row_ptr, const int32_t* d_col, int64_t n_rows,
                                      int N, int64_t* d_out_row_ptr, int32_t* d_out_col, int64_t* out_nnz)
{
    if (!ctx || !d_row_ptr || !d_col || !d_out_row_ptr || !d_out_col || !out_nnz || N < 1) return NN_ERR_INVALID_ARG;
    if (N > n_rows)
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "not enough points in the file: N = %d, %lld available", N,
                       (long long)n_rows);
    const int sparsity = (int)(n_rows / N);
    int64_t* cnt = nullptr;
    NN_TRY(nn_alloc(ctx, &cnt, (size_t)N + 1));
    cudaStream_t cs = ctx->stream;
    const int blocks = nn_grid_for(ctx, (int64_t)N * 32, 256, 8);
    nn_status st = nn_cuda_check(ctx, cudaMemsetAsync(cnt + N, 0, sizeof(int64_t), cs), "memset");
    k_sub_count<<<blocks, 256, 0, cs>>>(d_row_ptr, d_col, N, sparsity, cnt);
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaGetLastError(), "k_sub_count");
    ctx->launches++;
    if (st == NN_OK) st = nn_scan_exclusive_i64(ctx, cnt, d_out_row_ptr, (int64_t)N + 1);
    if (st == NN_OK) {
        k_sub_fill<<<blocks, 256, 0, cs>>>(d_row_ptr, d_col, N, sparsity, d_out_row_ptr, d_out_col);
        st = nn_cuda_check(ctx, cudaGetLastError(), "k_sub_fill");
        ctx->launches++;
    }
    if (st == NN_OK)
        st = nn_cuda_check(ctx, cudaMemcpyAsync(out_nnz, d_out_row_ptr + N, sizeof(int64_t), cudaMemcpyDeviceToHost, cs),
                           "copy");
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaStreamSynchronize(cs), "nn_net_subsample");
    nn_release(cnt);
    return st;
}

extern "C" nn_status nn_positions_file_write(const char* path, int64_t n, const float* h_x, const float* h_y,
                                             const float* h_z)
{
    if (!path || n < 1 || !h_x || !h_y || !h_z) return NN_ERR_INVALID_ARG;
    File f(path, "wb");
    if (!f.f) return NN_ERR_INVALID_ARG;
    const bool ok = write_exact(f.f, POS_MAGIC, 8) && write_exact(f.f, &n, 8) && write_exact(f.f, h_x, 4 * n) &&
                    write_exact(f.f, h_y, 4 * n) && write_exact(f.f, h_z, 4 * n);
    return ok ? NN_OK : NN_ERR_INVALID_ARG;
}

extern "C" nn_status nn_positions_file_read(const char* path, int64_t* n, float* h_x, float* h_y, float* h_z)
{
    if (!path || !n) return NN_ERR_INVALID_ARG;
    File f(path, "rb");
    if (!f.f) return NN_ERR_INVALID_ARG;
    char magic[8];
    int64_t m = 0;
    if (!read_exact(f.f, magic, 8) || std::memcmp(magic, POS_MAGIC, 8) || !read_exact(f.f, &m, 8) || m < 1)
        return NN_ERR_INVALID_ARG;
    *n = m;
    if (!h_x) return NN_OK;
    if (!h_y || !h_z || !read_exact(f.f, h_x, 4 * m) || !read_exact(f.f, h_y, 4 * m) || !read_exact(f.f, h_z, 4 * m))
        return NN_ERR_INVALID_ARG;
    return NN_OK;
}

// N positions from n (device arrays), scaled to [-1, 1] by the bounding box of all n.
extern "C" nn_status nn_positions_subsample(nn_ctx* ctx, const float* d_x, const float* d_y, const float* d_z,
                                            int64_t n, int N, float* d_ox, float* d_oy, float* d_oz)
{
    if (!ctx || !d_x || !d_y || !d_z || !d_ox || !d_oy || !d_oz || N < 1) return NN_ERR_INVALID_ARG;
    if (N > n) return nn_fail(ctx, NN_ERR_INVALID_ARG, "not enough points: N = %d, %lld available", N, (long long)n);
    float* mm = nullptr;
    NN_TRY(nn_alloc(ctx, &mm, 6));
    cudaStream_t cs = ctx->stream;
    const float* src[3] = {d_x, d_y, d_z};
    nn_status st = NN_OK;
    for (int a = 0; a < 3 && st == NN_OK; ++a) {
        k_minmax<<<1, 1024, 0, cs>>>(src[a], n, mm + 2 * a);
        st = nn_cuda_check(ctx, cudaGetLastError(), "k_minmax");
        ctx->launches++;
    }
    if (st == NN_OK) {
        k_pos_sample<<<nn_grid_for(ctx, N, 256, 4), 256, 0, cs>>>(d_x, d_y, d_z, mm, N, n / N, d_ox, d_oy, d_oz);
        st = nn_cuda_check(ctx, cudaGetLastError(), "k_pos_sample");
        ctx->launches++;
    }
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaStreamSynchronize(cs), "nn_positions_subsample");
    nn_release(mm);
    return st;
}
