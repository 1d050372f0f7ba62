// Local Gaussian-ball connectivity of the whole-brain model (NormalNetwork,
// src_wholebrain/network_factory.cu:95-138), built on the GPU with a uniform
// grid hash instead of the reference's kd-tree ball query.
//
// Rule (the reference's): neuron i connects to every other neuron j within
// n_stddevs * stddev with probability exp(-|x_i - x_j|^2 / (2 stddev^2)).
// Draws: one counter-based uniform per ordered pair (Philox keyed by seed, i,
// j), so the result does not depend on the visiting order; the reference
// draws from its unseeded default engine in kd-tree order, so individual
// edges differ while the distribution is the same.
//
// Build: cells of side n_stddevs * stddev over the positions' bounding box;
// a count / scan / fill pass places neurons by cell, each cell's list sorted
// ascending; then a warp per neuron visits the 27 neighbouring cells
// (dz, dy, dx in -1..1 order, neurons ascending within a cell), tests the
// radius in FP32 (no contraction) and the probability in FP64.  Two passes
// (count, fill) over the same decisions give a CSR with rows in that order.
#include <cmath>
#include <vector>

#include "nn_internal.cuh"

namespace {
constexpr uint32_t NN_P_LOCAL = 10;
constexpr int CT = 256;

struct Hash {
    float x0, y0, z0, inv_h;
    int gx, gy, gz;
};

__device__ __forceinline__ int cell_of(const Hash& H, float x, float y, float z, int& cx, int& cy, int& cz)
{
    cx = min(max((int)(__fsub_rn(x, H.x0) * H.inv_h), 0), H.gx - 1);
    cy = min(max((int)(__fsub_rn(y, H.y0) * H.inv_h), 0), H.gy - 1);
    cz = min(max((int)(__fsub_rn(z, H.z0) * H.inv_h), 0), H.gz - 1);
    return cx + H.gx * (cy + H.gy * cz);
}

__global__ void k_cell_count(int n, const float* x, const float* y, const float* z, Hash H, int* cell, int64_t* cnt)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int cx, cy, cz;
        const int c = cell_of(H, x[i], y[i], z[i], cx, cy, cz);
        cell[i] = c;
        atomicAdd((unsigned long long*)&cnt[c], 1ull);
    }
}

__global__ void k_cell_fill(int n, const int* cell, const int64_t* start, int* fill, int* members)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int c = cell[i];
        members[start[c] + atomicAdd(&fill[c], 1)] = i;
    }
}

// ascending members per cell (cells hold few neurons: insertion sort)
__global__ void k_cell_sort(int ncells, const int64_t* start, int* members)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x) {
        const int64_t b = start[c], e = start[c + 1];
        for (int64_t p = b + 1; p < e; ++p) {
            const int v = members[p];
            int64_t q = p - 1;
            while (q >= b && members[q] > v) {
                members[q + 1] = members[q];
                --q;
            }
            members[q + 1] = v;
        }
    }
}

struct Rule {
    float r2;          // (n_stddevs * stddev)^2
    double inv_2var;   // 1 / (2 stddev^2)
    uint64_t seed;
};

__device__ __forceinline__ bool accept(const Rule& R, int i, int j, float xi, float yi, float zi, float xj, float yj,
                                       float zj)
{
    const float dx = __fsub_rn(xi, xj), dy = __fsub_rn(yi, yj), dz = __fsub_rn(zi, zj);
    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    if (!(d2 <= R.r2)) return false;
    const nn_u4 r = nn_philox(R.seed, (uint32_t)i, (uint32_t)j, 0u, NN_P_LOCAL);
    const double u = ((double)(r.x >> 5) * 67108864.0 + (double)(r.y >> 6)) * (1.0 / 9007199254740992.0);
    return u < exp(-(double)d2 * R.inv_2var);
}

// warp per neuron; lanes stride each neighbouring cell's member list;
// fill == nullptr: count only
__global__ void __launch_bounds__(CT) k_local_rows(int n, const float* x, const float* y, const float* z, Hash H,
                                                   const int64_t* start, const int* members, Rule R,
                                                   const int* row_off, int* cnt, int* out)
{
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * CT + threadIdx.x) >> 5;
    const int nw = (gridDim.x * CT) >> 5;
    for (int i = gw; i < n; i += nw) {
        const float xi = x[i], yi = y[i], zi = z[i];
        int cx, cy, cz;
        cell_of(H, xi, yi, zi, cx, cy, cz);
        int pos = out ? row_off[i] : 0;
        int total = 0;
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int ax = cx + dx, ay = cy + dy, az = cz + dz;
                    if (ax < 0 || ay < 0 || az < 0 || ax >= H.gx || ay >= H.gy || az >= H.gz) continue;
                    const int c = ax + H.gx * (ay + H.gy * az);
                    const int64_t b = start[c], e = start[c + 1];
                    for (int64_t p0 = b; p0 < e; p0 += 32) {
                        const int64_t p = p0 + lane;
                        bool ok = false;
                        int j = -1;
                        if (p < e) {
                            j = members[p];
                            ok = j != i && accept(R, i, j, xi, yi, zi, x[j], y[j], z[j]);
                        }
                        const unsigned m = __ballot_sync(0xffffffffu, ok);
                        if (out && ok) out[pos + __popc(m & ((1u << lane) - 1u))] = j;
                        pos += __popc(m);
                        total += __popc(m);
                    }
                }
        if (!out && lane == 0) cnt[i] = total;
    }
}
}  // namespace

// NormalNetwork::Generate(N) on the device.  d_offsets (n + 1 ints) always
// receives the row offsets; d_indices (nullable) receives the targets when
// capacity >= the edge count, which *nnz returns.
extern "C" nn_status nn_net_local_gaussian(nn_ctx* ctx, int n, const float* d_x, const float* d_y, const float* d_z,
                                           float stddev, int n_stddevs, uint64_t seed, int* d_offsets, int* d_indices,
                                           int64_t capacity, int64_t* nnz)
{
    if (!ctx || n < 1 || !d_x || !d_y || !d_z || !(stddev > 0.0f) || n_stddevs < 1 || !d_offsets || !nnz)
        return NN_ERR_INVALID_ARG;
    cudaStream_t cs = ctx->stream;
    // bounding box on the host (positions are small: n floats per axis)
    std::vector<float> hx((size_t)n), hy((size_t)n), hz((size_t)n);
    NN_CUDA(ctx, cudaMemcpyAsync(hx.data(), d_x, sizeof(float) * n, cudaMemcpyDeviceToHost, cs));
    NN_CUDA(ctx, cudaMemcpyAsync(hy.data(), d_y, sizeof(float) * n, cudaMemcpyDeviceToHost, cs));
    NN_CUDA(ctx, cudaMemcpyAsync(hz.data(), d_z, sizeof(float) * n, cudaMemcpyDeviceToHost, cs));
    NN_CUDA(ctx, cudaStreamSynchronize(cs));
    float lo[3] = {hx[0], hy[0], hz[0]}, hi[3] = {hx[0], hy[0], hz[0]};
    for (int i = 0; i < n; ++i) {
        const float v[3] = {hx[(size_t)i], hy[(size_t)i], hz[(size_t)i]};
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], v[a]);
            hi[a] = std::max(hi[a], v[a]);
        }
    }
    const float h = stddev * (float)n_stddevs;
    Hash H;
    H.x0 = lo[0]; H.y0 = lo[1]; H.z0 = lo[2];
    H.inv_h = 1.0f / h;
    H.gx = std::max(1, (int)std::ceil((hi[0] - lo[0]) / h));
    H.gy = std::max(1, (int)std::ceil((hi[1] - lo[1]) / h));
    H.gz = std::max(1, (int)std::ceil((hi[2] - lo[2]) / h));
    const int64_t ncells = (int64_t)H.gx * H.gy * H.gz;
    if (ncells > (int64_t)1 << 28) return nn_fail(ctx, NN_ERR_INVALID_ARG, "local network: stddev too small for the extent");
    int *cell = nullptr, *fill = nullptr, *members = nullptr, *cnt = nullptr;
    int64_t *ccount = nullptr, *cstart = nullptr;
    nn_status st = nn_alloc(ctx, &cell, (size_t)n);
    if (st == NN_OK) st = nn_alloc(ctx, &members, (size_t)n);
    if (st == NN_OK) st = nn_alloc(ctx, &fill, (size_t)ncells);
    if (st == NN_OK) st = nn_alloc(ctx, &ccount, (size_t)ncells + 1);
    if (st == NN_OK) st = nn_alloc(ctx, &cstart, (size_t)ncells + 1);
    if (st == NN_OK) st = nn_alloc(ctx, &cnt, (size_t)n + 1);
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaMemsetAsync(ccount, 0, sizeof(int64_t) * (ncells + 1), cs), "memset");
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaMemsetAsync(fill, 0, sizeof(int) * ncells, cs), "memset");
    if (st == NN_OK) {
        k_cell_count<<<nn_grid_for(ctx, n, 256, 8), 256, 0, cs>>>(n, d_x, d_y, d_z, H, cell, ccount);
        st = nn_cuda_check(ctx, cudaGetLastError(), "k_cell_count");
        ctx->launches++;
    }
    if (st == NN_OK) st = nn_scan_exclusive_i64(ctx, ccount, cstart, ncells + 1);
    if (st == NN_OK) {
        k_cell_fill<<<nn_grid_for(ctx, n, 256, 8), 256, 0, cs>>>(n, cell, cstart, fill, members);
        k_cell_sort<<<nn_grid_for(ctx, ncells, 256, 8), 256, 0, cs>>>((int)ncells, cstart, members);
        st = nn_cuda_check(ctx, cudaGetLastError(), "k_cell_fill");
        ctx->launches += 2;
    }
    Rule R;
    R.r2 = h * h;
    R.inv_2var = 1.0 / (2.0 * (double)stddev * (double)stddev);
    R.seed = seed;
    if (st == NN_OK) {
        k_local_rows<<<nn_grid_for(ctx, (int64_t)n * 32, CT, 8), CT, 0, cs>>>(n, d_x, d_y, d_z, H, cstart, members, R,
                                                                               nullptr, cnt, nullptr);
        st = nn_cuda_check(ctx, cudaGetLastError(), "k_local_rows");
        ctx->launches++;
    }
    // offsets (int, as the reference's AdjacencyList)
    std::vector<int> hcnt((size_t)n), hoff((size_t)n + 1, 0);
    if (st == NN_OK) st = nn_cuda_check(ctx, nn_copy_sync(ctx, hcnt.data(), cnt, sizeof(int) * n, cudaMemcpyDeviceToHost), "copy");
    int64_t total = 0;
    for (int i = 0; i < n && st == NN_OK; ++i) {
        total += hcnt[(size_t)i];
        if (total > INT32_MAX) st = nn_fail(ctx, NN_ERR_INVALID_ARG, "local network exceeds 2^31 edges");
        hoff[(size_t)i + 1] = (int)total;
    }
    if (st == NN_OK)
        st = nn_cuda_check(ctx, nn_copy_sync(ctx, d_offsets, hoff.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice), "copy");
    *nnz = total;
    if (st == NN_OK && d_indices) {
        if (capacity < total) {
            st = nn_fail(ctx, NN_ERR_INVALID_ARG, "local network: capacity %lld < %lld edges", (long long)capacity,
                         (long long)total);
        } else {
            k_local_rows<<<nn_grid_for(ctx, (int64_t)n * 32, CT, 8), CT, 0, cs>>>(n, d_x, d_y, d_z, H, cstart,
                                                                                   members, R, d_offsets, nullptr,
                                                                                   d_indices);
            st = nn_cuda_check(ctx, cudaGetLastError(), "k_local_rows");
            ctx->launches++;
        }
    }
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaStreamSynchronize(cs), "nn_net_local_gaussian");
    nn_release(cell); nn_release(members); nn_release(fill); nn_release(ccount); nn_release(cstart); nn_release(cnt);
    return st;
}
