// Batched Jacobi-PCG: many independent cubic 7-point backward-Euler systems
// (one per network instance of a batch, each with its own side g_b and
// alpha_b = dt D g_b^2) solved together, each to its own relative residual.
//
// The instances' cells are concatenated (instance b at cell offset off_b,
// x fastest).  A thread block covers CPB = 256 VPT consecutive cells of one
// instance (VPT per thread, strided by the block size; VPT = 8 unless the
// autotuner, nn_bpcg_autotune, chose 2, 4 or 16),
// so every reduction is per instance: a block writes its FP64 partials, and
// the last block of an instance to arrive (a per-instance ticket) sums them in
// fixed order and forms that instance's scalars.  Per iteration two kernels
// run (the structure of the two-kernel PCG: direction + operator, then
// update), and blocks of converged instances return at once, so the batch
// iterates until its slowest instance converges while the others stop
// costing work.  The host reads the counter of unconverged instances and
// their flags once per chunk of iterations; once instances have converged,
// the chunk's kernels are launched over the blocks of the running instances
// only (a list of block ids), since even a block that returns at once costs
// its launch.
#include <algorithm>
#include <cmath>
#include <vector>

#include "nn_internal.cuh"

namespace {
constexpr int BT = 256;
constexpr int VPT_MIN = 2;        // cells per thread: 2, 4, 8 or 16

struct Batch {
    int n_inst;
    const int* side;         // [n_inst]
    const int64_t* off;      // [n_inst + 1] cell offsets
    const float* alpha;      // [n_inst]
    const float* invd;       // [n_inst] 1 / (1 + beta + 6 alpha)
    float onepb;             // 1 + beta
    const int* blk_inst;     // block -> instance
    const int* blk_first;    // [n_inst + 1] first block of each instance
    double* scal;            // [n_inst][S_COUNT]
    double* partials;        // [3][nblocks]
    unsigned int* ticket;    // [n_inst]
    int* flags;              // [n_inst] 0 running, 1 converged, 2 stopped (non-finite)
    int* iters;              // [n_inst]
    int* running;            // [1] unconverged instances
    const int* work;         // launched block -> block id (null: the identity)
    int nblocks;             // all blocks (the partials' stride)
    double rtol2;
};

// The block this CTA stands for.
__device__ __forceinline__ int block_id(const Batch& B) { return B.work ? B.work[blockIdx.x] : (int)blockIdx.x; }

enum { S_RZ = 0, S_PAP, S_RR, S_BB, S_ALPHA, S_BETA, S_COUNT };

// n / g and n % g for 0 <= n < 2^24, g >= 1: the FP32 quotient is exact or
// one off, and one correction step fixes it
__device__ __forceinline__ int divmod_small(int n, int g, float invg, int& rem)
{
    int q = __float2int_rz((float)n * invg);
    int r = n - q * g;
    if (r < 0) {
        --q;
        r += g;
    } else if (r >= g) {
        ++q;
        r -= g;
    }
    rem = r;
    return q;
}

// (i, j, k) of cell c of a g^3 cube (g^3 < 2^24: the instance sides are at
// most 256)
__device__ __forceinline__ void coords(int64_t c, int g, int& i, int& j, int& k)
{
    const float invg = 1.0f / (float)g;
    const int t = divmod_small((int)c, g, invg, i);
    k = divmod_small(t, g, invg, j);
}

// (A v)_c on the instance's cube (zero outside)
template <class V>
__device__ __forceinline__ float apply_cell(float onepb, float al, int g, int64_t c, V v)
{
    int i, j, k;
    coords(c, g, i, j, k);
    const int64_t sy = g, sz = (int64_t)g * g;
    float nb = 0.0f;
    nb += i > 0 ? v(c - 1) : 0.0f;
    nb += i < g - 1 ? v(c + 1) : 0.0f;
    nb += j > 0 ? v(c - sy) : 0.0f;
    nb += j < g - 1 ? v(c + sy) : 0.0f;
    nb += k > 0 ? v(c - sz) : 0.0f;
    nb += k < g - 1 ? v(c + sz) : 0.0f;
    return (onepb + 6.0f * al) * v(c) - al * nb;
}

// block partial sums (FP32 within a warp, FP64 across warps); the last block
// of instance b to arrive sums the instance's partials in block order
__device__ bool instance_reduce(const Batch& B, int blk, int b, int nsum, const float* v, double* out)
{
    __shared__ double ws[3][BT / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nblocks = B.nblocks;
    for (int q = 0; q < nsum; ++q) {
        float s = v[q];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) ws[q][w] = (double)s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 0; q < nsum; ++q) {
            double s = 0.0;
            for (int u = 0; u < BT / 32; ++u) s += ws[q][u];
            B.partials[(size_t)q * nblocks + blk] = s;
        }
        __threadfence();
        const unsigned nb = (unsigned)(B.blk_first[b + 1] - B.blk_first[b]);
        last = atomicAdd(&B.ticket[b], 1u) == nb - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    const int f0 = B.blk_first[b], f1 = B.blk_first[b + 1];
    for (int q = 0; q < nsum; ++q) {
        const volatile double* pp = B.partials + (size_t)q * nblocks;
        double s = 0.0;
        for (int k = f0 + threadIdx.x; k < f1; k += BT) s += pp[k];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        __syncthreads();
        if (lane == 0) ws[q][w] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int u = 0; u < BT / 32; ++u) t += ws[q][u];
            out[q] = t;
        }
    }
    if (threadIdx.x == 0) B.ticket[b] = 0;
    __syncthreads();
    return true;
}

// r = b - A x, p = z = M r; partials (r, z), (b, b), (r, r)
template <int VPT>
__global__ void __launch_bounds__(BT) k_bpcg_init(Batch B, const float* rhs, const float* x, float* r, float* p)
{
    const int blk = block_id(B);
    const int b = B.blk_inst[blk];
    const int g = B.side[b];
    const int64_t base = B.off[b], cells = B.off[b + 1] - base;
    const int64_t c0 = (int64_t)(blk - B.blk_first[b]) * (BT * VPT) + threadIdx.x;
    float rz = 0.0f, bb = 0.0f, rr = 0.0f;
#pragma unroll
    for (int v = 0; v < VPT; ++v) {
        const int64_t c = c0 + v * BT;
        if (c >= cells) break;
        const float* xb = x + base;
        const float ax = apply_cell(B.onepb, B.alpha[b], g, c, [&](int64_t q) { return xb[q]; });
        const float bv = rhs[base + c];
        const float rv = bv - ax;
        const float zv = B.invd[b] * rv;
        r[base + c] = rv;
        p[base + c] = zv;
        rz += rv * zv;
        bb += bv * bv;
        rr += rv * rv;
    }
    float v[3] = {rz, bb, rr};
    double out[3];
    if (instance_reduce(B, blk, b, 3, v, out) && threadIdx.x == 0) {
        double* s = B.scal + (size_t)b * S_COUNT;
        s[S_RZ] = out[0];
        s[S_BB] = out[1];
        s[S_RR] = out[2];
        s[S_BETA] = 0.0;
        B.iters[b] = 0;
        const bool done = out[2] <= B.rtol2 * out[1];
        B.flags[b] = done ? 1 : 0;
        if (!done) atomicAdd(B.running, 1);
    }
}

// p = z + beta p_old (z = M r; the first iteration has beta = 0 and p_old = z),
// Ap = A p; partial (p, Ap) -> alpha = rz / pAp
template <int VPT>
__global__ void __launch_bounds__(BT) k_bpcg_dir_apply(Batch B, const float* r, const float* p_old, float* p_new,
                                                       float* Ap)
{
    const int blk = block_id(B);
    const int b = B.blk_inst[blk];
    if (B.flags[b]) return;
    const int g = B.side[b];
    const int64_t base = B.off[b], cells = B.off[b + 1] - base;
    const int64_t c0 = (int64_t)(blk - B.blk_first[b]) * (BT * VPT) + threadIdx.x;
    const double* s = B.scal + (size_t)b * S_COUNT;
    const float beta = (float)s[S_BETA], md = B.invd[b];
    float pap = 0.0f;
    const float* rb = r + base;
    const float* pb = p_old + base;
    auto pv = [&](int64_t q) { return md * rb[q] + beta * pb[q]; };
#pragma unroll
    for (int v = 0; v < VPT; ++v) {
        const int64_t c = c0 + v * BT;
        if (c >= cells) break;
        const float pc = pv(c);
        p_new[base + c] = pc;
        const float ap = apply_cell(B.onepb, B.alpha[b], g, c, pv);
        Ap[base + c] = ap;
        pap += pc * ap;
    }
    float v[1] = {pap};
    double out[1];
    if (instance_reduce(B, blk, b, 1, v, out) && threadIdx.x == 0) {
        double* sw = B.scal + (size_t)b * S_COUNT;
        sw[S_PAP] = out[0];
        sw[S_ALPHA] = out[0] != 0.0 ? sw[S_RZ] / out[0] : 0.0;
    }
}

// x += alpha p, r -= alpha Ap; partials (r, z), (r, r) -> beta, convergence
template <int VPT>
__global__ void __launch_bounds__(BT) k_bpcg_update(Batch B, float* x, float* r, const float* p, const float* Ap,
                                                    int max_iter)
{
    const int blk = block_id(B);
    const int b = B.blk_inst[blk];
    if (B.flags[b]) return;
    const int64_t base = B.off[b], cells = B.off[b + 1] - base;
    const int64_t c0 = (int64_t)(blk - B.blk_first[b]) * (BT * VPT) + threadIdx.x;
    const double* s = B.scal + (size_t)b * S_COUNT;
    const float alpha = (float)s[S_ALPHA];
    float rz = 0.0f, rr = 0.0f;
#pragma unroll
    for (int v = 0; v < VPT; ++v) {
        const int64_t c = c0 + v * BT;
        if (c >= cells) break;
        const int64_t q = base + c;
        x[q] += alpha * p[q];
        const float rv = r[q] - alpha * Ap[q];
        r[q] = rv;
        rz += rv * (B.invd[b] * rv);
        rr += rv * rv;
    }
    float v[2] = {rz, rr};
    double out[2];
    if (instance_reduce(B, blk, b, 2, v, out) && threadIdx.x == 0) {
        double* sw = B.scal + (size_t)b * S_COUNT;
        const int it = B.iters[b] + 1;
        B.iters[b] = it;
        sw[S_BETA] = sw[S_RZ] != 0.0 ? out[0] / sw[S_RZ] : 0.0;
        sw[S_RZ] = out[0];
        sw[S_RR] = out[1];
        int f = 0;
        if (out[1] <= B.rtol2 * sw[S_BB]) f = 1;
        else if (!std::isfinite(out[1])) f = 2;
        else if (it >= max_iter) f = 3;
        if (f) {
            B.flags[b] = f;
            atomicSub(B.running, 1);
        }
    }
}
}  // namespace

struct nn_bpcg {
    nn_ctx* ctx = nullptr;
    int n_inst = 0;
    int64_t G = 0;
    int nblocks = 0;
    int vpt = 8;                   // cells per thread of the current block layout
    int max_blocks = 0;            // blocks at VPT_MIN (the layout arrays' size)
    std::vector<int> h_side;
    std::vector<int64_t> h_off;
    int *side = nullptr, *blk_inst = nullptr, *blk_first = nullptr, *flags = nullptr, *iters = nullptr,
        *running = nullptr;
    int64_t* off = nullptr;
    float *alpha = nullptr, *invd = nullptr;
    float onepb = 1.0f;
    double* scal = nullptr;
    double* partials = nullptr;
    unsigned int* ticket = nullptr;
    float *r = nullptr, *p0 = nullptr, *p1 = nullptr, *Ap = nullptr;
    // blocks of the running instances (host list, device copy)
    std::vector<int> h_first;
    std::vector<int> h_work, h_flags;
    int* work = nullptr;
    // asynchronous solve in progress (nn_bpcg_async_*)
    bool as_active = false;
    float* as_x = nullptr;
    double as_rtol = 0.0;
    int as_max_iter = 0, as_it = 0;
    cudaStream_t as_cs = nullptr;
    // timing of the last solve (events around the iteration chunks)
    bool timing = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float last_ms = 0.0f;
    int last_iters = 0;
};

extern "C" nn_status nn_bpcg_destroy(nn_bpcg* bp)
{
    if (!bp) return NN_OK;
    if (bp->ctx) cudaStreamSynchronize(bp->ctx->stream);
    for (void* q : {(void*)bp->side, (void*)bp->blk_inst, (void*)bp->blk_first, (void*)bp->flags, (void*)bp->iters,
                    (void*)bp->running, (void*)bp->off, (void*)bp->alpha, (void*)bp->invd, (void*)bp->scal,
                    (void*)bp->partials, (void*)bp->ticket, (void*)bp->r, (void*)bp->p0, (void*)bp->p1, (void*)bp->Ap,
                    (void*)bp->work})
        if (q) cudaFree(q);
    if (bp->ev0) cudaEventDestroy(bp->ev0);
    if (bp->ev1) cudaEventDestroy(bp->ev1);
    nn_ctx* ctx = bp->ctx;
    delete bp;
    if (ctx) nn_ctx_release(ctx);
    return NN_OK;
}

// Block layout for vpt cells per thread: blocks of each instance, block ->
// instance table, first block of each instance.
static nn_status set_layout(nn_bpcg* bp, int vpt)
{
    nn_ctx* ctx = bp->ctx;
    const int64_t cpb = (int64_t)BT * vpt;
    std::vector<int> first((size_t)bp->n_inst + 1, 0), binst;
    for (int b = 0; b < bp->n_inst; ++b) {
        const int64_t cells = bp->h_off[(size_t)b + 1] - bp->h_off[(size_t)b];
        const int nb = (int)((cells + cpb - 1) / cpb);
        first[(size_t)b + 1] = first[(size_t)b] + nb;
        for (int q = 0; q < nb; ++q) binst.push_back(b);
    }
    NN_CUDA(ctx, nn_copy_sync(ctx, bp->blk_inst, binst.data(), sizeof(int) * binst.size(), cudaMemcpyHostToDevice));
    NN_CUDA(ctx, nn_copy_sync(ctx, bp->blk_first, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice));
    bp->vpt = vpt;
    bp->nblocks = first.back();
    bp->h_first = first;
    return NN_OK;
}

// sides[b] >= 1; alpha_b = alpha_unit * side_b^2 (alpha_unit = dt D on the unit cube)
extern "C" nn_status nn_bpcg_create(nn_ctx* ctx, int n_inst, const int* h_sides, double alpha_unit, double beta,
                                    nn_bpcg** out)
{
    if (!ctx || !h_sides || !out) return NN_ERR_INVALID_ARG;
    *out = nullptr;
    if (n_inst < 1) return nn_fail(ctx, NN_ERR_INVALID_ARG, "batched PCG: no instances");
    nn_bpcg* bp = new nn_bpcg();
    bp->ctx = ctx;
    nn_ctx_retain(ctx);
    bp->n_inst = n_inst;
    bp->h_side.assign(h_sides, h_sides + n_inst);
    bp->h_off.assign((size_t)n_inst + 1, 0);
    std::vector<float> al(n_inst), iv(n_inst);
    for (int b = 0; b < n_inst; ++b) {
        const int g = h_sides[b];
        if (g < 1 || g > 255) {
            nn_bpcg_destroy(bp);
            return nn_fail(ctx, NN_ERR_INVALID_ARG, "batched PCG: instance %d has side %d (1 .. 255)", b, g);
        }
        const int64_t cells = (int64_t)g * g * g;
        bp->h_off[(size_t)b + 1] = bp->h_off[(size_t)b] + cells;
        al[b] = (float)(alpha_unit * g * g);
        iv[b] = (float)(1.0 / (1.0 + beta + 6.0 * alpha_unit * g * g));
        bp->max_blocks += (int)((cells + BT * VPT_MIN - 1) / (BT * VPT_MIN));
    }
    bp->G = bp->h_off.back();
    bp->onepb = (float)(1.0 + beta);
    nn_status st = NN_OK;
    const size_t G = (size_t)bp->G;
    if (st == NN_OK) st = nn_alloc(ctx, &bp->side, (size_t)n_inst);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->off, (size_t)n_inst + 1);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->alpha, (size_t)n_inst);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->invd, (size_t)n_inst);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->blk_inst, (size_t)bp->max_blocks);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->blk_first, (size_t)n_inst + 1);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->work, (size_t)bp->max_blocks);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->flags, (size_t)n_inst);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->iters, (size_t)n_inst);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->running, 1);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->scal, (size_t)n_inst * S_COUNT);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->partials, (size_t)3 * bp->max_blocks);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->ticket, (size_t)n_inst);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->r, G);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->p0, G);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->p1, G);
    if (st == NN_OK) st = nn_alloc(ctx, &bp->Ap, G);
    if (st == NN_OK) st = nn_cuda_check(ctx, nn_copy_sync(ctx, bp->side, h_sides, sizeof(int) * n_inst, cudaMemcpyHostToDevice), "copy");
    if (st == NN_OK)
        st = nn_cuda_check(ctx, nn_copy_sync(ctx, bp->off, bp->h_off.data(), sizeof(int64_t) * (n_inst + 1), cudaMemcpyHostToDevice), "copy");
    if (st == NN_OK) st = nn_cuda_check(ctx, nn_copy_sync(ctx, bp->alpha, al.data(), sizeof(float) * n_inst, cudaMemcpyHostToDevice), "copy");
    if (st == NN_OK) st = nn_cuda_check(ctx, nn_copy_sync(ctx, bp->invd, iv.data(), sizeof(float) * n_inst, cudaMemcpyHostToDevice), "copy");
    if (st == NN_OK) st = set_layout(bp, 8);
    if (st == NN_OK) st = nn_cuda_check(ctx, nn_zero_async(ctx, bp->ticket, sizeof(unsigned int) * n_inst), "memset");
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventCreate(&bp->ev0), "event");
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventCreate(&bp->ev1), "event");
    if (st != NN_OK) {
        nn_bpcg_destroy(bp);
        return st;
    }
    *out = bp;
    return NN_OK;
}

int64_t nn_bpcg_cells(const nn_bpcg* bp) { return bp->G; }
const int64_t* nn_bpcg_offsets(const nn_bpcg* bp) { return bp->h_off.data(); }
void nn_bpcg_set_timing(nn_bpcg* bp, bool on) { bp->timing = on; }
void nn_bpcg_last_timing(const nn_bpcg* bp, float* ms, int* iters)
{
    *ms = bp->last_ms;
    *iters = bp->last_iters;
}

static Batch batch_args(nn_bpcg* bp, double rtol)
{
    Batch B;
    B.n_inst = bp->n_inst;
    B.side = bp->side;
    B.off = bp->off;
    B.alpha = bp->alpha;
    B.invd = bp->invd;
    B.onepb = bp->onepb;
    B.blk_inst = bp->blk_inst;
    B.blk_first = bp->blk_first;
    B.scal = bp->scal;
    B.partials = bp->partials;
    B.ticket = bp->ticket;
    B.flags = bp->flags;
    B.iters = bp->iters;
    B.running = bp->running;
    B.work = nullptr;
    B.nblocks = bp->nblocks;
    B.rtol2 = rtol * rtol;
    return B;
}

namespace {

// r0, z0 and the instances' initial scalars on stream cs
nn_status enqueue_init(nn_bpcg* bp, const Batch& B, const float* d_b, const float* d_x, cudaStream_t cs)
{
    nn_ctx* ctx = bp->ctx;
    NN_CUDA(ctx, cudaMemsetAsync(bp->running, 0, sizeof(int), cs));
    NN_CUDA(ctx, cudaMemsetAsync(bp->ticket, 0, sizeof(unsigned int) * bp->n_inst, cs));
    if (bp->timing) NN_CUDA(ctx, cudaEventRecord(bp->ev0, cs));
    switch (bp->vpt) {
        case 2: k_bpcg_init<2><<<bp->nblocks, BT, 0, cs>>>(B, d_b, d_x, bp->r, bp->p0); break;
        case 4: k_bpcg_init<4><<<bp->nblocks, BT, 0, cs>>>(B, d_b, d_x, bp->r, bp->p0); break;
        case 16: k_bpcg_init<16><<<bp->nblocks, BT, 0, cs>>>(B, d_b, d_x, bp->r, bp->p0); break;
        default: k_bpcg_init<8><<<bp->nblocks, BT, 0, cs>>>(B, d_b, d_x, bp->r, bp->p0); break;
    }
    NN_CHECK_LAUNCH(ctx, "k_bpcg_init");
    return NN_OK;
}

// iterations it .. it + n - 1 over `grid` launched blocks (B.work: their ids)
nn_status enqueue_iters(nn_bpcg* bp, const Batch& B, float* d_x, int it, int n, int grid, int max_iter,
                        cudaStream_t cs)
{
    nn_ctx* ctx = bp->ctx;
    for (int q = 0; q < n; ++q, ++it) {
        // p0 holds z = M r at the start (beta = 0), then the directions alternate
        const float* p_old = (it & 1) ? bp->p1 : bp->p0;
        float* p_new = (it & 1) ? bp->p0 : bp->p1;
        switch (bp->vpt) {
            case 2: k_bpcg_dir_apply<2><<<grid, BT, 0, cs>>>(B, bp->r, p_old, p_new, bp->Ap); break;
            case 4: k_bpcg_dir_apply<4><<<grid, BT, 0, cs>>>(B, bp->r, p_old, p_new, bp->Ap); break;
            case 16: k_bpcg_dir_apply<16><<<grid, BT, 0, cs>>>(B, bp->r, p_old, p_new, bp->Ap); break;
            default: k_bpcg_dir_apply<8><<<grid, BT, 0, cs>>>(B, bp->r, p_old, p_new, bp->Ap); break;
        }
        NN_CHECK_LAUNCH(ctx, "k_bpcg_dir_apply");
        switch (bp->vpt) {
            case 2: k_bpcg_update<2><<<grid, BT, 0, cs>>>(B, d_x, bp->r, p_new, bp->Ap, max_iter); break;
            case 4: k_bpcg_update<4><<<grid, BT, 0, cs>>>(B, d_x, bp->r, p_new, bp->Ap, max_iter); break;
            case 16: k_bpcg_update<16><<<grid, BT, 0, cs>>>(B, d_x, bp->r, p_new, bp->Ap, max_iter); break;
            default: k_bpcg_update<8><<<grid, BT, 0, cs>>>(B, d_x, bp->r, p_new, bp->Ap, max_iter); break;
        }
        NN_CHECK_LAUNCH(ctx, "k_bpcg_update");
    }
    return NN_OK;
}

// Iterate from iteration *it until no instance runs, reading the counter and
// the flags once per chunk; once instances have stopped, only the blocks of
// the running ones are launched.
nn_status iterate(nn_bpcg* bp, Batch B, float* d_x, int* it, int max_iter, cudaStream_t cs)
{
    nn_ctx* ctx = bp->ctx;
    const int chunk = 16;
    int running = 0;
    bp->h_flags.assign((size_t)bp->n_inst, 0);
    while (true) {
        NN_CUDA(ctx, cudaMemcpyAsync(&running, bp->running, sizeof(int), cudaMemcpyDeviceToHost, cs));
        NN_CUDA(ctx, cudaMemcpyAsync(bp->h_flags.data(), bp->flags, sizeof(int) * bp->n_inst,
                                     cudaMemcpyDeviceToHost, cs));
        NN_CUDA(ctx, cudaStreamSynchronize(cs));
        if (running == 0 || *it >= max_iter) break;
        // the blocks of the instances still running (all blocks while none has stopped)
        int grid = bp->nblocks;
        B.work = nullptr;
        if (running < bp->n_inst) {
            bp->h_work.clear();
            for (int b = 0; b < bp->n_inst; ++b)
                if (bp->h_flags[(size_t)b] == 0)
                    for (int k = bp->h_first[(size_t)b]; k < bp->h_first[(size_t)b + 1]; ++k) bp->h_work.push_back(k);
            grid = (int)bp->h_work.size();
            if (grid == 0) break;
            NN_CUDA(ctx, cudaMemcpyAsync(bp->work, bp->h_work.data(), sizeof(int) * bp->h_work.size(),
                                         cudaMemcpyHostToDevice, cs));
            B.work = bp->work;
        }
        const int n = std::min(chunk, max_iter - *it);
        NN_TRY(enqueue_iters(bp, B, d_x, *it, n, grid, max_iter, cs));
        *it += n;
    }
    return NN_OK;
}

// Per-instance iteration counts and convergence of the finished solve.
nn_status collect(nn_bpcg* bp, cudaStream_t cs, int* h_iters, int* max_iters, int* unconverged)
{
    nn_ctx* ctx = bp->ctx;
    if (bp->timing) {
        NN_CUDA(ctx, cudaEventRecord(bp->ev1, cs));
        NN_CUDA(ctx, cudaEventSynchronize(bp->ev1));
        NN_CUDA(ctx, cudaEventElapsedTime(&bp->last_ms, bp->ev0, bp->ev1));
    }
    std::vector<int> its(bp->n_inst), fl(bp->n_inst);
    NN_CUDA(ctx, cudaMemcpyAsync(its.data(), bp->iters, sizeof(int) * bp->n_inst, cudaMemcpyDeviceToHost, cs));
    NN_CUDA(ctx, cudaMemcpyAsync(fl.data(), bp->flags, sizeof(int) * bp->n_inst, cudaMemcpyDeviceToHost, cs));
    NN_CUDA(ctx, cudaStreamSynchronize(cs));
    int mx = 0, bad = 0;
    for (int b = 0; b < bp->n_inst; ++b) {
        mx = std::max(mx, its[(size_t)b]);
        bad += fl[(size_t)b] != 1;
    }
    if (h_iters) std::copy(its.begin(), its.end(), h_iters);
    if (max_iters) *max_iters = mx;
    if (unconverged) *unconverged = bad;
    bp->last_iters = mx;
    return NN_OK;
}

}  // namespace

// Solve every instance (x holds the initial guesses).  *unconverged: the
// instances that stopped before reaching rtol (0 on success); iters
// (nullable, n_inst entries): per-instance iteration counts; *max_iters: the
// batch's iteration count.
extern "C" nn_status nn_bpcg_solve(nn_bpcg* bp, const float* d_b, float* d_x, double rtol, int max_iter,
                                   int* h_iters, int* max_iters, int* unconverged)
{
    if (!bp || !d_b || !d_x || !(rtol > 0.0) || max_iter < 0) return NN_ERR_INVALID_ARG;
    cudaStream_t cs = bp->ctx->stream;
    const Batch B = batch_args(bp, rtol);
    NN_TRY(enqueue_init(bp, B, d_b, d_x, cs));
    int it = 0;
    NN_TRY(iterate(bp, B, d_x, &it, max_iter, cs));
    return collect(bp, cs, h_iters, max_iters, unconverged);
}

// Asynchronous solve on stream cs: the init and n iterations over all blocks
// (blocks of converged instances return at once) are enqueued with no host
// read; nn_bpcg_async_finish waits for the stream, completes the solve if n
// was not enough and reports as nn_bpcg_solve does.  The arithmetic of every
// instance is that of nn_bpcg_solve.
nn_status nn_bpcg_async_begin(nn_bpcg* bp, const float* d_b, float* d_x, double rtol, int max_iter, int n,
                              cudaStream_t cs)
{
    if (!bp || !d_b || !d_x || !(rtol > 0.0) || max_iter < 0) return NN_ERR_INVALID_ARG;
    const Batch B = batch_args(bp, rtol);
    NN_TRY(enqueue_init(bp, B, d_b, d_x, cs));
    const int m = std::max(0, std::min(n, max_iter));
    NN_TRY(enqueue_iters(bp, B, d_x, 0, m, bp->nblocks, max_iter, cs));
    bp->as_active = true;
    bp->as_x = d_x;
    bp->as_rtol = rtol;
    bp->as_max_iter = max_iter;
    bp->as_it = m;
    bp->as_cs = cs;
    return NN_OK;
}

nn_status nn_bpcg_async_finish(nn_bpcg* bp, int* h_iters, int* max_iters, int* unconverged)
{
    if (!bp || !bp->as_active) return NN_ERR_INVALID_ARG;
    bp->as_active = false;
    int it = bp->as_it;
    NN_TRY(iterate(bp, batch_args(bp, bp->as_rtol), bp->as_x, &it, bp->as_max_iter, bp->as_cs));
    return collect(bp, bp->as_cs, h_iters, max_iters, unconverged);
}

// Block-size autotuner: time `iters` iterations over all blocks (after two
// untimed ones) for 2, 4, 8 and 16 cells per thread on the batch's own
// operators -- right-hand side d_b, d_x as scratch (overwritten), a residual
// target no instance reaches -- and keep the fastest layout.
extern "C" nn_status nn_bpcg_autotune(nn_bpcg* bp, const float* d_b, float* d_x, int iters, int* cells_per_block,
                                      float* ms_per_iter)
{
    if (!bp || !d_b || !d_x || iters < 1) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = bp->ctx;
    if (bp->as_active) return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_bpcg_autotune: a solve is pending");
    cudaStream_t cs = ctx->stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    NN_CUDA(ctx, cudaEventCreate(&e0));
    NN_CUDA(ctx, cudaEventCreate(&e1));
    const int vpt0 = bp->vpt;
    const bool timing0 = bp->timing;
    bp->timing = false;
    int best_vpt = vpt0;
    float best = 1e30f;
    nn_status st = NN_OK;
    const int max_iter = 1 << 30;
    for (int vpt : {2, 4, 8, 16}) {
        if (st != NN_OK) break;
        st = set_layout(bp, vpt);
        const Batch B = batch_args(bp, 1e-30);
        if (st == NN_OK) st = nn_cuda_check(ctx, cudaMemsetAsync(d_x, 0, sizeof(float) * (size_t)bp->G, cs), "memset");
        if (st == NN_OK) st = enqueue_init(bp, B, d_b, d_x, cs);
        if (st == NN_OK) st = enqueue_iters(bp, B, d_x, 0, 2, bp->nblocks, max_iter, cs);
        if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventRecord(e0, cs), "event");
        if (st == NN_OK) st = enqueue_iters(bp, B, d_x, 2, iters, bp->nblocks, max_iter, cs);
        if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventRecord(e1, cs), "event");
        int running = 0;
        if (st == NN_OK)
            st = nn_cuda_check(ctx, cudaMemcpyAsync(&running, bp->running, sizeof(int), cudaMemcpyDeviceToHost, cs),
                               "copy");
        if (st == NN_OK) st = nn_cuda_check(ctx, cudaStreamSynchronize(cs), "nn_bpcg_autotune");
        float ms = 0.0f;
        if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventElapsedTime(&ms, e0, e1), "event");
        // a layout under which instances stopped early did less work: no timing
        if (st == NN_OK && running == bp->n_inst && ms / iters < best) {
            best = ms / iters;
            best_vpt = vpt;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    bp->timing = timing0;
    const nn_status st2 = set_layout(bp, st == NN_OK ? best_vpt : vpt0);
    if (st == NN_OK) st = st2;
    if (cells_per_block) *cells_per_block = BT * bp->vpt;
    if (ms_per_iter) *ms_per_iter = best < 1e30f ? best : 0.0f;
    return st;
}

int nn_bpcg_cells_per_block(const nn_bpcg* bp) { return BT * bp->vpt; }

extern "C" nn_status nn_bpcg_set_cells_per_block(nn_bpcg* bp, int cells_per_block)
{
    if (!bp) return NN_ERR_INVALID_ARG;
    const int vpt = cells_per_block / BT;
    if (cells_per_block != BT * vpt || (vpt != 2 && vpt != 4 && vpt != 8 && vpt != 16))
        return nn_fail(bp->ctx, NN_ERR_INVALID_ARG, "nn_bpcg_set_cells_per_block: 512, 1024, 2048 or 4096");
    if (bp->as_active) return nn_fail(bp->ctx, NN_ERR_INVALID_ARG, "nn_bpcg_set_cells_per_block: a solve is pending");
    return set_layout(bp, vpt);
}
