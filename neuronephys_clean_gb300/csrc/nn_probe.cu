// Consumers of the simulation step: electrode sampling, synchrony measures
// and the Hebbian weight rule (the reference's ElectrodeNet, SynchronyNet and
// Hebbian classes).
//
// Electrodes (src/electrode_net.cu:3-49, src_wholebrain/electrode_net.cu:3-54):
// per region, the mean membrane potential over its index list and the number
// of its neurons flagged as firing.  The reference runs one thread per
// region over the whole list; here a warp takes a region and its lanes stride
// the list (coalesced index loads, gathered V), reduced in a fixed order.
//
// Synchrony (src_wholebrain/electrode_net.cu:56-124): running FP64 sums of
// V_i^2 and V_i for each listed neuron, and of <V>_sub and <V>_sub^2 for
// nested sub-populations (the first Nsub listed neurons); the measure
// chi_sub = Nsub sigma^2(<V>_sub) / sum_j sigma^2(V_j) is formed on the host
// exactly as GetSynchronyMeasures does.
//
// Hebbian (src_wholebrain/hebbian.cu:3-69): per synapse a timer; a firing
// presynaptic neuron sets the timers of all its synapses to the window; each
// update then visits every synapse with a running timer: decrement; at zero,
// w -= inc * exp(-|w - 1|); else if the target fires, w += inc * exp(-|w - 1|)
// and the timer stops.  The reference sweeps all synapses every update; only
// the rows of neurons that fired within the last `window` updates can hold a
// running timer, so here a row countdown selects those rows (a compaction)
// and a warp per active row applies the rule: the same result at a cost
// proportional to the recently active synapses.
#include <cmath>
#include <vector>

#include "nn_internal.cuh"

namespace {
constexpr int PT = 256;

__global__ void __launch_bounds__(PT) k_electrodes(int n_regions, const int* idx, const int* off, const float* V,
                                                   const int* is_firing, float* avg, int* nfiring)
{
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * (PT / 32) + (threadIdx.x >> 5);
    const int nw = gridDim.x * (PT / 32);
    for (int r = gw; r < n_regions; r += nw) {
        const int beg = off[r], end = off[r + 1];
        float s = 0.0f;
        int f = 0;
        for (int q = beg + lane; q < end; q += 32) {
            const int i = idx[q];
            s += V[i];
            if (is_firing) f += is_firing[i];
        }
        s = nn_warp_sumf(s);
        for (int o = 16; o > 0; o >>= 1) f += __shfl_xor_sync(0xffffffffu, f, o);
        if (lane == 0) {
            avg[r] = s / (float)(end - beg);
            if (is_firing) nfiring[r] = f;
        }
    }
}

// sum of V over n entries (FP32 per thread, fixed-order tree) -> out (FP32)
__global__ void __launch_bounds__(PT) k_sum_f(const float* V, const int* idx, int n, float* out)
{
    __shared__ float ws[PT / 32];
    float s = 0.0f;
    for (int q = threadIdx.x; q < n; q += PT) s += V[idx ? idx[q] : q];
    s = nn_warp_sumf(s);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int w = 0; w < PT / 32; ++w) t += ws[w];
        *out = t;
    }
}

__global__ void k_variance(int n, const int* idx, const float* V, double* vi2, double* vi)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const float v = V[idx[q]];
        vi2[q] += (double)(v * v);
        vi[q] += (double)v;
    }
}

// Hebbian: start the row countdown and the synapse timers of firing neurons
__global__ void k_heb_set(int num_firing, const int* firing, const int* off, int window, int* timers, int* row_left)
{
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * (PT / 32) + (threadIdx.x >> 5);
    const int nw = gridDim.x * (PT / 32);
    for (int q = gw; q < num_firing; q += nw) {
        const int pre = firing[q];
        if (lane == 0) row_left[pre] = window;
        for (int s = off[pre] + lane; s < off[pre + 1]; s += 32) timers[s] = window;
    }
}

// rows with a running countdown -> list (order irrelevant: rows are disjoint)
__global__ void k_heb_rows(int n, int* row_left, int* rows, int* nrows)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int left = row_left[i];
        if (left > 0) {
            rows[atomicAdd(nrows, 1)] = i;
            row_left[i] = left - 1;
        }
    }
}

__global__ void __launch_bounds__(PT) k_heb_rule(const int* rows, const int* nrows, const int* off, const int* col,
                                                 const int* is_firing, int* timers, float* w, float inc)
{
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * (PT / 32) + (threadIdx.x >> 5);
    const int nw = gridDim.x * (PT / 32);
    const int nr = *nrows;
    for (int q = gw; q < nr; q += nw) {
        const int pre = rows[q];
        for (int s = off[pre] + lane; s < off[pre + 1]; s += 32) {
            int t = timers[s];
            if (t == 0) continue;
            t -= 1;
            const float wv = w[s];
            const float a = expf(-fabsf(wv - 1.0f));
            if (t == 0) {
                w[s] = wv - inc * a;
            } else if (is_firing[col[s]]) {
                w[s] = wv + inc * a;
                t = 0;
            }
            timers[s] = t;
        }
    }
}
}  // namespace

// ------------------------------------------------------------ electrodes --

struct nn_electrodes {
    nn_ctx* ctx = nullptr;
    int n_regions = 0;
    int *idx = nullptr, *off = nullptr;
    float* avg = nullptr;
    int* nfiring = nullptr;
};

extern "C" nn_status nn_electrodes_create(nn_ctx* ctx, const int* h_indices, const int* h_offsets, int n_regions,
                                          nn_electrodes** out)
{
    if (!ctx || !h_offsets || !out || n_regions < 1) return NN_ERR_INVALID_ARG;
    *out = nullptr;
    const int nidx = h_offsets[n_regions];
    if (h_offsets[0] != 0 || nidx < 0 || (nidx > 0 && !h_indices)) return NN_ERR_INVALID_ARG;
    for (int r = 0; r < n_regions; ++r)
        if (h_offsets[r + 1] <= h_offsets[r])
            return nn_fail(ctx, NN_ERR_INVALID_ARG, "electrode region %d is empty or offsets decrease", r);
    nn_electrodes* e = new nn_electrodes();
    e->ctx = ctx;
    nn_ctx_retain(ctx);
    e->n_regions = n_regions;
    nn_status st = nn_alloc(ctx, &e->idx, (size_t)nidx);
    if (st == NN_OK) st = nn_alloc(ctx, &e->off, (size_t)n_regions + 1);
    if (st == NN_OK) st = nn_alloc(ctx, &e->avg, (size_t)n_regions);
    if (st == NN_OK) st = nn_alloc(ctx, &e->nfiring, (size_t)n_regions);
    if (st == NN_OK)
        st = nn_cuda_check(ctx, nn_copy_sync(ctx, e->idx, h_indices, sizeof(int) * nidx, cudaMemcpyHostToDevice), "copy");
    if (st == NN_OK)
        st = nn_cuda_check(ctx, nn_copy_sync(ctx, e->off, h_offsets, sizeof(int) * (n_regions + 1), cudaMemcpyHostToDevice),
                           "copy");
    if (st == NN_OK) st = nn_cuda_check(ctx, nn_zero_async(ctx, e->nfiring, sizeof(int) * n_regions), "memset");
    if (st != NN_OK) {
        nn_electrodes_destroy(e);
        return st;
    }
    *out = e;
    return NN_OK;
}

extern "C" nn_status nn_electrodes_destroy(nn_electrodes* e)
{
    if (!e) return NN_OK;
    if (e->ctx) cudaStreamSynchronize(e->ctx->stream);
    nn_release(e->idx);
    nn_release(e->off);
    nn_release(e->avg);
    nn_release(e->nfiring);
    nn_ctx* ctx = e->ctx;
    delete e;
    nn_ctx_release(ctx);
    return NN_OK;
}

extern "C" nn_status nn_electrodes_measure(nn_electrodes* e, const float* d_V, const int* d_is_firing, float* h_avg,
                                           int* h_firing)
{
    if (!e || !d_V) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = e->ctx;
    k_electrodes<<<nn_grid_for(ctx, (int64_t)e->n_regions * 32, PT, 8), PT, 0, ctx->stream>>>(
        e->n_regions, e->idx, e->off, d_V, d_is_firing, e->avg, e->nfiring);
    NN_CHECK_LAUNCH(ctx, "k_electrodes");
    if (h_avg)
        NN_CUDA(ctx, cudaMemcpyAsync(h_avg, e->avg, sizeof(float) * e->n_regions, cudaMemcpyDeviceToHost, ctx->stream));
    if (h_firing)
        NN_CUDA(ctx, cudaMemcpyAsync(h_firing, e->nfiring, sizeof(int) * e->n_regions, cudaMemcpyDeviceToHost,
                                     ctx->stream));
    if (h_avg || h_firing) NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return NN_OK;
}

extern "C" nn_status nn_measure_average(nn_ctx* ctx, const float* d_V, int n, float* out)
{
    if (!ctx || !d_V || n < 1 || !out) return NN_ERR_INVALID_ARG;
    float* d = nullptr;
    NN_TRY(nn_alloc(ctx, &d, 1));
    k_sum_f<<<1, PT, 0, ctx->stream>>>(d_V, nullptr, n, d);
    nn_status st = nn_cuda_check(ctx, cudaGetLastError(), "k_sum_f");
    ctx->launches++;
    float s = 0.0f;
    if (st == NN_OK)
        st = nn_cuda_check(ctx, cudaMemcpyAsync(&s, d, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream), "copy");
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    nn_release(d);
    *out = s / (float)n;
    return st;
}

// ------------------------------------------------------------- synchrony --

struct nn_synchrony {
    nn_ctx* ctx = nullptr;
    int n = 0;
    int* idx = nullptr;
    double *vi2 = nullptr, *vi = nullptr;
    float* sub_sum = nullptr;
    std::vector<int> sub;
    std::vector<double> avg2, avg;
    int steps = 0;
};

extern "C" nn_status nn_synchrony_create(nn_ctx* ctx, const int* h_region_inds, int n_inds, const int* h_sub_counts,
                                         int n_sub, nn_synchrony** out)
{
    if (!ctx || !h_region_inds || n_inds < 1 || !h_sub_counts || n_sub < 1 || !out) return NN_ERR_INVALID_ARG;
    *out = nullptr;
    for (int q = 0; q < n_sub; ++q)
        if (h_sub_counts[q] < 1 || h_sub_counts[q] > n_inds)
            return nn_fail(ctx, NN_ERR_INVALID_ARG, "sub-population %d size outside [1, %d]", q, n_inds);
    nn_synchrony* s = new nn_synchrony();
    s->ctx = ctx;
    nn_ctx_retain(ctx);
    s->n = n_inds;
    s->sub.assign(h_sub_counts, h_sub_counts + n_sub);
    s->avg2.assign(n_sub, 0.0);
    s->avg.assign(n_sub, 0.0);
    nn_status st = nn_alloc(ctx, &s->idx, (size_t)n_inds);
    if (st == NN_OK) st = nn_alloc(ctx, &s->vi2, (size_t)n_inds);
    if (st == NN_OK) st = nn_alloc(ctx, &s->vi, (size_t)n_inds);
    if (st == NN_OK) st = nn_alloc(ctx, &s->sub_sum, (size_t)n_sub);
    if (st == NN_OK)
        st = nn_cuda_check(ctx, nn_copy_sync(ctx, s->idx, h_region_inds, sizeof(int) * n_inds, cudaMemcpyHostToDevice), "copy");
    if (st == NN_OK) st = nn_cuda_check(ctx, nn_zero_async(ctx, s->vi2, sizeof(double) * n_inds), "memset");
    if (st == NN_OK) st = nn_cuda_check(ctx, nn_zero_async(ctx, s->vi, sizeof(double) * n_inds), "memset");
    if (st != NN_OK) {
        nn_synchrony_destroy(s);
        return st;
    }
    *out = s;
    return NN_OK;
}

extern "C" nn_status nn_synchrony_destroy(nn_synchrony* s)
{
    if (!s) return NN_OK;
    if (s->ctx) cudaStreamSynchronize(s->ctx->stream);
    nn_release(s->idx);
    nn_release(s->vi2);
    nn_release(s->vi);
    nn_release(s->sub_sum);
    nn_ctx* ctx = s->ctx;
    delete s;
    nn_ctx_release(ctx);
    return NN_OK;
}

extern "C" nn_status nn_synchrony_measure(nn_synchrony* s, const float* d_V)
{
    if (!s || !d_V) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    k_variance<<<nn_grid_for(ctx, s->n, PT, 8), PT, 0, ctx->stream>>>(s->n, s->idx, d_V, s->vi2, s->vi);
    NN_CHECK_LAUNCH(ctx, "k_variance");
    const int ns = (int)s->sub.size();
    for (int q = 0; q < ns; ++q) {
        k_sum_f<<<1, PT, 0, ctx->stream>>>(d_V, s->idx, s->sub[q], s->sub_sum + q);
        NN_CHECK_LAUNCH(ctx, "k_sum_f");
    }
    std::vector<float> sums(ns);
    NN_CUDA(ctx, cudaMemcpyAsync(sums.data(), s->sub_sum, sizeof(float) * ns, cudaMemcpyDeviceToHost, ctx->stream));
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int q = 0; q < ns; ++q) {
        const double a = sums[q] / s->sub[q];
        s->avg[q] += a;
        s->avg2[q] += a * a;
    }
    s->steps += 1;
    return NN_OK;
}

// chi for every sub-population (GetSynchronyMeasures)
extern "C" nn_status nn_synchrony_get(nn_synchrony* s, double* h_chi)
{
    if (!s || !h_chi) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    std::vector<double> vi2(s->n), vi(s->n);
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    NN_CUDA(ctx, nn_copy_sync(ctx, vi2.data(), s->vi2, sizeof(double) * s->n, cudaMemcpyDeviceToHost));
    NN_CUDA(ctx, nn_copy_sync(ctx, vi.data(), s->vi, sizeof(double) * s->n, cudaMemcpyDeviceToHost));
    const double T = s->steps;
    if (T > 0)
        for (int i = 0; i < s->n; ++i) {
            vi2[i] /= T;
            vi[i] /= T;
        }
    for (size_t q = 0; q < s->sub.size(); ++q) {
        const int ns = s->sub[q];
        double denom = 0.0;
        for (int j = 0; j < ns; ++j) denom += vi2[j] - vi[j] * vi[j];
        const double var = T > 0 ? (s->avg2[q] - s->avg[q] * s->avg[q] / T) / T : 0.0;
        h_chi[q] = ns * var / denom;
    }
    return NN_OK;
}

// -------------------------------------------------------------- Hebbian --

struct nn_hebbian {
    nn_ctx* ctx = nullptr;
    int64_t nconns = 0;
    int n = 0;
    int window = 0;
    float inc = 0.0f;
    int* timers = nullptr;
    int* row_left = nullptr;
    int* rows = nullptr;
    int* nrows = nullptr;
};

extern "C" nn_status nn_hebbian_create(nn_ctx* ctx, int window, float inc, int64_t nconns, int n_neurons,
                                       nn_hebbian** out)
{
    if (!ctx || !out || window < 1 || nconns < 0 || n_neurons < 1 || nconns > INT32_MAX) return NN_ERR_INVALID_ARG;
    *out = nullptr;
    nn_hebbian* h = new nn_hebbian();
    h->ctx = ctx;
    nn_ctx_retain(ctx);
    h->nconns = nconns;
    h->n = n_neurons;
    h->window = window;
    h->inc = inc;
    nn_status st = nn_alloc(ctx, &h->timers, (size_t)std::max<int64_t>(nconns, 1));
    if (st == NN_OK) st = nn_alloc(ctx, &h->row_left, (size_t)n_neurons);
    if (st == NN_OK) st = nn_alloc(ctx, &h->rows, (size_t)n_neurons);
    if (st == NN_OK) st = nn_alloc(ctx, &h->nrows, 1);
    if (st == NN_OK) st = nn_cuda_check(ctx, nn_zero_async(ctx, h->timers, sizeof(int) * std::max<int64_t>(nconns, 1)), "memset");
    if (st == NN_OK) st = nn_cuda_check(ctx, nn_zero_async(ctx, h->row_left, sizeof(int) * n_neurons), "memset");
    if (st != NN_OK) {
        nn_hebbian_destroy(h);
        return st;
    }
    *out = h;
    return NN_OK;
}

extern "C" nn_status nn_hebbian_destroy(nn_hebbian* h)
{
    if (!h) return NN_OK;
    if (h->ctx) cudaStreamSynchronize(h->ctx->stream);
    nn_release(h->timers);
    nn_release(h->row_left);
    nn_release(h->rows);
    nn_release(h->nrows);
    nn_ctx* ctx = h->ctx;
    delete h;
    nn_ctx_release(ctx);
    return NN_OK;
}

// UpdateWeights(connectivity, is_firing, firing_inds): d_indices / d_offsets
// the CSR (row = presynaptic), is_firing per neuron, firing_inds the list of
// num_firing presynaptic neurons whose timers are set.  Asynchronous.
extern "C" nn_status nn_hebbian_update(nn_hebbian* h, const int* d_indices, const int* d_offsets,
                                       const int* d_is_firing, const int* d_firing_inds, int num_firing,
                                       float* d_weights)
{
    if (!h || !d_indices || !d_offsets || !d_is_firing || !d_weights || num_firing < 0 ||
        (num_firing > 0 && !d_firing_inds))
        return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = h->ctx;
    cudaStream_t cs = ctx->stream;
    if (num_firing > 0) {
        k_heb_set<<<nn_grid_for(ctx, (int64_t)num_firing * 32, PT, 8), PT, 0, cs>>>(
            num_firing, d_firing_inds, d_offsets, h->window, h->timers, h->row_left);
        NN_CHECK_LAUNCH(ctx, "k_heb_set");
    }
    NN_CUDA(ctx, cudaMemsetAsync(h->nrows, 0, sizeof(int), cs));
    k_heb_rows<<<nn_grid_for(ctx, h->n, PT, 8), PT, 0, cs>>>(h->n, h->row_left, h->rows, h->nrows);
    NN_CHECK_LAUNCH(ctx, "k_heb_rows");
    k_heb_rule<<<nn_grid_for(ctx, (int64_t)h->n * 32, PT, 8), PT, 0, cs>>>(h->rows, h->nrows, d_offsets, d_indices,
                                                                         d_is_firing, h->timers, d_weights, h->inc);
    NN_CHECK_LAUNCH(ctx, "k_heb_rule");
    return NN_OK;
}

extern "C" nn_status nn_hebbian_timers(nn_hebbian* h, int* h_timers)
{
    if (!h || !h_timers) return NN_ERR_INVALID_ARG;
    NN_CUDA(h->ctx, cudaStreamSynchronize(h->ctx->stream));
    NN_CUDA(h->ctx, nn_copy_sync(h->ctx, h_timers, h->timers, sizeof(int) * h->nconns, cudaMemcpyDeviceToHost));
    return NN_OK;
}
