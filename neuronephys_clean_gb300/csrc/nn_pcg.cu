// 7-point backward-Euler diffusion operator and Jacobi-preconditioned CG.
//
// A = (1 + beta) I + alpha L_D on an nx*ny*nz grid (x fastest), where
// (L_D x)_c = sum over the 6 faces f of c_f (x_c - x_nb), c_f the harmonic
// mean of the cell field D on the two sides (D_c at the domain boundary, whose
// ghost values are zero: homogeneous Dirichlet).  With D == NULL every c_f = 1.
//
// Per iteration two kernels run, each finishing its grid-wide FP64 reduction
// in the last block to arrive (no host round trip):
//   k_pcg_dir_apply : p = z + b p_old (z = r / diag, recomputed at the 6
//                     neighbours), Ap = A p, partial (p, Ap)  -> a = rz / pAp
//   k_pcg_update    : x += a p, r -= a Ap, partials (r, z), (r, r)
//                     -> b = rz_new / rz, convergence flag
// p is double-buffered because the direction update reads neighbours.
// Products are accumulated in FP32 within a thread's strip of cells and in
// FP64 from the warp level up.
#include <algorithm>
#include <cmath>
#include <mutex>

#include "nn_internal.cuh"

struct nn_pcg {
    nn_ctx* ctx = nullptr;
    int nx = 0, ny = 0, nz = 0;
    int64_t G = 0;
    double alpha = 0, beta = 0;
    const float* Dcell = nullptr;  // caller's cell field (may be NULL)
    float* invd = nullptr;         // 1/diag (heterogeneous case)
    float inv_diag_const = 0.0f;
    float *r = nullptr, *p0 = nullptr, *p1 = nullptr, *Ap = nullptr;
    double* scal = nullptr;        // see enum below
    double* partials = nullptr;
    unsigned int* ticket = nullptr;
    int* flags = nullptr;          // [0] done, [1] iterations
    int nblocks = 0;
    // optional timing of the iteration kernels (events around each chunk)
    bool timing = false;
    std::vector<cudaEvent_t> ev_a, ev_b;
    float last_ms = 0.0f;
    int last_iters = 0;
    // single-kernel TMA iteration (nx % 4 == 0, aligned D); null: two-kernel path
    nn_cg_plan* fast = nullptr;
};

void nn_pcg_set_timing(nn_pcg* pc, bool on)
{
    pc->timing = on;
    if (pc->fast) nn_cg_set_timing(pc->fast, on);
}
void nn_pcg_last_timing(const nn_pcg* pc, float* ms, int* iters)
{
    if (pc->fast) {
        nn_cg_last_timing(pc->fast, ms, iters);
        return;
    }
    *ms = pc->last_ms;
    *iters = pc->last_iters;
}

enum { S_RZ = 0, S_PAP, S_RZNEW, S_RR, S_BB, S_BETA, S_ALPHA, S_COUNT };

namespace {
constexpr int PCG_THREADS = 256;

struct Op {
    int nx, ny, nz;
    float alpha, onepb;  // alpha, 1 + beta
    const float* D;      // may be null
    const float* invd;   // may be null (constant)
    float invd_c;
};

__device__ __forceinline__ float face(const float* D, float dc, int64_t nb, bool inside)
{
    if (!D) return 1.0f;
    if (!inside) return dc;
    const float dn = D[nb];
    return __fdividef(2.0f * dc * dn, dc + dn);
}

__device__ __forceinline__ void cell_coords(const Op& o, int64_t c, int& i, int& j, int& k)
{
    i = (int)(c % o.nx);
    const int64_t t = c / o.nx;
    j = (int)(t % o.ny);
    k = (int)(t / o.ny);
}

// (A v)_c given v at the cell and its 6 neighbours (zero outside).
__device__ __forceinline__ float apply_cell(const Op& o, int64_t c, int i, int j, int k, float vc, const float vn[6])
{
    const int64_t sy = o.nx, sz = (int64_t)o.nx * o.ny;
    const bool in[6] = {i > 0, i < o.nx - 1, j > 0, j < o.ny - 1, k > 0, k < o.nz - 1};
    const int64_t nb[6] = {c - 1, c + 1, c - sy, c + sy, c - sz, c + sz};
    const float dc = o.D ? o.D[c] : 1.0f;
    float acc = 0.0f;
#pragma unroll
    for (int f = 0; f < 6; ++f) acc += face(o.D, dc, nb[f], in[f]) * (vc - vn[f]);
    return o.onepb * vc + o.alpha * acc;
}

__device__ bool last_block_sum(int nsum, const double* v, double* partials, unsigned int* ticket, double* out)
{
    __shared__ double ws[3][PCG_THREADS / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = 0; q < nsum; ++q) {
        double s = nn_warp_sum(v[q]);
        if (lane == 0) ws[q][w] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 0; q < nsum; ++q) {
            double s = 0.0;
            for (int u = 0; u < PCG_THREADS / 32; ++u) s += ws[q][u];
            partials[(size_t)q * gridDim.x + blockIdx.x] = s;
        }
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    // the last block sums the partials with all its threads (fixed order)
    __threadfence();
    for (int q = 0; q < nsum; ++q) {
        const volatile double* pp = partials + (size_t)q * gridDim.x;
        double s = 0.0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += PCG_THREADS) s += pp[b];
        s = nn_warp_sum(s);
        __syncthreads();
        if (lane == 0) ws[q][w] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int u = 0; u < PCG_THREADS / 32; ++u) t += ws[q][u];
            out[q] = t;
        }
    }
    if (threadIdx.x == 0) *ticket = 0;
    __syncthreads();
    return true;
}

__global__ void __launch_bounds__(PCG_THREADS) k_pcg_apply(Op o, const float* x, float* y)
{
    const int64_t G = (int64_t)o.nx * o.ny * o.nz;
    const int64_t sy = o.nx, sz = (int64_t)o.nx * o.ny;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < G; c += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_coords(o, c, i, j, k);
        float vn[6];
        vn[0] = i > 0 ? x[c - 1] : 0.0f;
        vn[1] = i < o.nx - 1 ? x[c + 1] : 0.0f;
        vn[2] = j > 0 ? x[c - sy] : 0.0f;
        vn[3] = j < o.ny - 1 ? x[c + sy] : 0.0f;
        vn[4] = k > 0 ? x[c - sz] : 0.0f;
        vn[5] = k < o.nz - 1 ? x[c + sz] : 0.0f;
        y[c] = apply_cell(o, c, i, j, k, x[c], vn);
    }
}

__global__ void k_pcg_invdiag(Op o, float* invd)
{
    const int64_t G = (int64_t)o.nx * o.ny * o.nz;
    const int64_t sy = o.nx, sz = (int64_t)o.nx * o.ny;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < G; c += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_coords(o, c, i, j, k);
        const float dc = o.D[c];
        float s = 0.0f;
        s += face(o.D, dc, c - 1, i > 0);
        s += face(o.D, dc, c + 1, i < o.nx - 1);
        s += face(o.D, dc, c - sy, j > 0);
        s += face(o.D, dc, c + sy, j < o.ny - 1);
        s += face(o.D, dc, c - sz, k > 0);
        s += face(o.D, dc, c + sz, k < o.nz - 1);
        invd[c] = 1.0f / (o.onepb + o.alpha * s);
    }
}

__device__ __forceinline__ float invd_at(const Op& o, int64_t c) { return o.invd ? o.invd[c] : o.invd_c; }

// r = b - A x; rz = (r, z); rr = (r, r); bb = (b, b); beta = 0
__global__ void __launch_bounds__(PCG_THREADS) k_pcg_init(Op o, const float* b, const float* x, float* r, double* scal,
                                                          double* partials, unsigned int* ticket, int* flags,
                                                          double rtol2)
{
    const int64_t G = (int64_t)o.nx * o.ny * o.nz;
    const int64_t sy = o.nx, sz = (int64_t)o.nx * o.ny;
    float a_rz = 0.0f, a_rr = 0.0f, a_bb = 0.0f;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < G; c += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_coords(o, c, i, j, k);
        float vn[6];
        vn[0] = i > 0 ? x[c - 1] : 0.0f;
        vn[1] = i < o.nx - 1 ? x[c + 1] : 0.0f;
        vn[2] = j > 0 ? x[c - sy] : 0.0f;
        vn[3] = j < o.ny - 1 ? x[c + sy] : 0.0f;
        vn[4] = k > 0 ? x[c - sz] : 0.0f;
        vn[5] = k < o.nz - 1 ? x[c + sz] : 0.0f;
        const float bv = b[c];
        const float rv = bv - apply_cell(o, c, i, j, k, x[c], vn);
        r[c] = rv;
        a_rz += rv * rv * invd_at(o, c);
        a_rr += rv * rv;
        a_bb += bv * bv;
    }
    double v[3] = {a_rz, a_rr, a_bb};
    double out[3];
    if (last_block_sum(3, v, partials, ticket, out) && threadIdx.x == 0) {
        scal[S_RZ] = out[0];
        scal[S_RR] = out[1];
        scal[S_BB] = out[2];
        scal[S_BETA] = 0.0;
        flags[1] = 0;
        flags[0] = (out[1] <= rtol2 * out[2]) ? 1 : 0;
    }
}

// p = z + beta p_old (z = r / diag), Ap = A p, (p, Ap) -> alpha
__global__ void __launch_bounds__(PCG_THREADS) k_pcg_dir_apply(Op o, const float* r, const float* p_old, float* p_new,
                                                               float* Ap, double* scal, double* partials,
                                                               unsigned int* ticket, const int* flags)
{
    if (flags[0]) return;
    const int64_t G = (int64_t)o.nx * o.ny * o.nz;
    const int64_t sy = o.nx, sz = (int64_t)o.nx * o.ny;
    const float bt = (float)scal[S_BETA];
    float a_pap = 0.0f;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < G; c += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_coords(o, c, i, j, k);
        const bool in[6] = {i > 0, i < o.nx - 1, j > 0, j < o.ny - 1, k > 0, k < o.nz - 1};
        const int64_t nb[6] = {c - 1, c + 1, c - sy, c + sy, c - sz, c + sz};
        float vn[6];
#pragma unroll
        for (int f = 0; f < 6; ++f)
            vn[f] = in[f] ? r[nb[f]] * invd_at(o, nb[f]) + bt * p_old[nb[f]] : 0.0f;
        const float pc = r[c] * invd_at(o, c) + bt * p_old[c];
        p_new[c] = pc;
        const float ap = apply_cell(o, c, i, j, k, pc, vn);
        Ap[c] = ap;
        a_pap += pc * ap;
    }
    double v[1] = {a_pap};
    double out[1];
    if (last_block_sum(1, v, partials, ticket, out) && threadIdx.x == 0) {
        scal[S_PAP] = out[0];
        scal[S_ALPHA] = scal[S_RZ] / out[0];
    }
}

// x += alpha p, r -= alpha Ap, (r, z), (r, r) -> beta, convergence
__global__ void __launch_bounds__(PCG_THREADS) k_pcg_update(Op o, float* x, float* r, const float* p, const float* Ap,
                                                            double* scal, double* partials, unsigned int* ticket,
                                                            int* flags, double rtol2, int max_iter)
{
    if (flags[0]) return;
    const int64_t G = (int64_t)o.nx * o.ny * o.nz;
    const float a = (float)scal[S_ALPHA];
    float a_rz = 0.0f, a_rr = 0.0f;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < G; c += (int64_t)gridDim.x * blockDim.x) {
        x[c] += a * p[c];
        const float rv = r[c] - a * Ap[c];
        r[c] = rv;
        a_rz += rv * rv * invd_at(o, c);
        a_rr += rv * rv;
    }
    double v[2] = {a_rz, a_rr};
    double out[2];
    if (last_block_sum(2, v, partials, ticket, out) && threadIdx.x == 0) {
        scal[S_BETA] = out[0] / scal[S_RZ];
        scal[S_RZ] = out[0];
        scal[S_RR] = out[1];
        const int it = flags[1] + 1;
        flags[1] = it;
        if (out[1] <= rtol2 * scal[S_BB]) flags[0] = 1;
        else if (it >= max_iter) flags[0] = 2;
    }
}

Op make_op(const nn_pcg* pc)
{
    Op o;
    o.nx = pc->nx; o.ny = pc->ny; o.nz = pc->nz;
    o.alpha = (float)pc->alpha;
    o.onepb = (float)(1.0 + pc->beta);
    o.D = pc->Dcell;
    o.invd = pc->invd;
    o.invd_c = pc->inv_diag_const;
    return o;
}
}  // namespace

extern "C" nn_status nn_pcg_create(nn_ctx* ctx, int nx, int ny, int nz, double alpha, double beta,
                                   const float* d_Dcell, nn_pcg** out)
{
    if (!ctx || !out || nx < 1 || ny < 1 || nz < 1 || !(alpha >= 0.0) || !(beta > -1.0))
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_pcg_create: bad argument");
    nn_pcg* pc = new nn_pcg();
    pc->ctx = ctx;
    nn_ctx_retain(ctx);
    pc->nx = nx; pc->ny = ny; pc->nz = nz;
    pc->G = (int64_t)nx * ny * nz;
    pc->alpha = alpha;
    pc->beta = beta;
    pc->Dcell = d_Dcell;
    pc->inv_diag_const = (float)(1.0 / (1.0 + beta + 6.0 * alpha));
    pc->nblocks = nn_grid_for(ctx, pc->G, PCG_THREADS, 8);
    const size_t G = (size_t)pc->G;
    nn_status st = nn_alloc(ctx, &pc->r, G);
    if (st == NN_OK) st = nn_alloc(ctx, &pc->p0, G);
    if (st == NN_OK) st = nn_alloc(ctx, &pc->p1, G);
    if (st == NN_OK) st = nn_alloc(ctx, &pc->Ap, G);
    if (st == NN_OK) st = nn_alloc(ctx, &pc->scal, S_COUNT);
    if (st == NN_OK) st = nn_alloc(ctx, &pc->partials, (size_t)3 * pc->nblocks);
    if (st == NN_OK) st = nn_alloc(ctx, &pc->ticket, 1);
    if (st == NN_OK) st = nn_alloc(ctx, &pc->flags, 2);
    if (st == NN_OK && d_Dcell) st = nn_alloc(ctx, &pc->invd, G);
    if (st != NN_OK) {
        nn_pcg_destroy(pc);
        return st;
    }
    cudaMemsetAsync(pc->ticket, 0, sizeof(unsigned int), ctx->stream);
    cudaMemsetAsync(pc->p0, 0, sizeof(float) * G, ctx->stream);
    cudaMemsetAsync(pc->p1, 0, sizeof(float) * G, ctx->stream);
    if (d_Dcell) {
        Op o = make_op(pc);
        k_pcg_invdiag<<<pc->nblocks, PCG_THREADS, 0, ctx->stream>>>(o, pc->invd);
        ctx->launches++;
    }
    st = nn_cuda_check(ctx, cudaGetLastError(), "nn_pcg_create");
    if (st == NN_OK && !std::getenv("NN_PCG_TWO_KERNEL")) {
        // the single-kernel TMA iteration where supported
        nn_status fs = nn_cg_plan_create(ctx, nx, ny, nz, alpha, beta, d_Dcell, pc->invd, &pc->fast);
        if (fs != NN_OK && fs != NN_ERR_UNSUPPORTED) st = fs;
        ctx->last_error.clear();
    }
    if (st != NN_OK) {
        nn_pcg_destroy(pc);
        return st;
    }
    *out = pc;
    return NN_OK;
}

extern "C" nn_status nn_pcg_destroy(nn_pcg* pc)
{
    if (!pc) return NN_OK;
    if (pc->ctx) cudaStreamSynchronize(pc->ctx->stream);
    nn_release(pc->r); nn_release(pc->p0); nn_release(pc->p1); nn_release(pc->Ap); nn_release(pc->scal);
    nn_release(pc->partials); nn_release(pc->ticket); nn_release(pc->flags); nn_release(pc->invd);
    if (pc->fast) nn_cg_plan_destroy(pc->fast);
    for (auto e : pc->ev_a) cudaEventDestroy(e);
    for (auto e : pc->ev_b) cudaEventDestroy(e);
    nn_ctx* ctx = pc->ctx;
    delete pc;
    nn_ctx_release(ctx);
    return NN_OK;
}

extern "C" nn_status nn_pcg_apply(nn_pcg* pc, const float* d_x, float* d_y)
{
    if (!pc || !d_x || !d_y) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = pc->ctx;
    Op o = make_op(pc);
    k_pcg_apply<<<pc->nblocks, PCG_THREADS, 0, ctx->stream>>>(o, d_x, d_y);
    NN_CHECK_LAUNCH(ctx, "k_pcg_apply");
    return NN_OK;
}

// Enqueue the whole solve without host synchronisation: init + max_iter
// iteration pairs, each a no-op once the device flag says converged.  Used
// inside captured simulation periods.
nn_status nn_pcg_enqueue(nn_pcg* pc, const float* d_b, float* d_x, double rtol, int max_iter)
{
    nn_ctx* ctx = pc->ctx;
    cudaStream_t s = ctx->stream;
    Op o = make_op(pc);
    const double rtol2 = rtol * rtol;
    k_pcg_init<<<pc->nblocks, PCG_THREADS, 0, s>>>(o, d_b, d_x, pc->r, pc->scal, pc->partials, pc->ticket, pc->flags,
                                                    rtol2);
    NN_CHECK_LAUNCH(ctx, "k_pcg_init");
    for (int it = 0; it < max_iter; ++it) {
        float* p_old = (it & 1) ? pc->p1 : pc->p0;
        float* p_new = (it & 1) ? pc->p0 : pc->p1;
        k_pcg_dir_apply<<<pc->nblocks, PCG_THREADS, 0, s>>>(o, pc->r, p_old, p_new, pc->Ap, pc->scal, pc->partials,
                                                             pc->ticket, pc->flags);
        NN_CHECK_LAUNCH(ctx, "k_pcg_dir_apply");
        k_pcg_update<<<pc->nblocks, PCG_THREADS, 0, s>>>(o, d_x, pc->r, p_new, pc->Ap, pc->scal, pc->partials,
                                                          pc->ticket, pc->flags, rtol2, max_iter);
        NN_CHECK_LAUNCH(ctx, "k_pcg_update");
    }
    return NN_OK;
}

// Host-driven solve: enqueue iterations in chunks and stop at convergence.
nn_status nn_pcg_run(nn_pcg* pc, const float* d_b, float* d_x, double rtol, int max_iter, int* iters, double* relres,
                     int* converged)
{
    nn_ctx* ctx = pc->ctx;
    cudaStream_t s = ctx->stream;
    Op o = make_op(pc);
    const double rtol2 = rtol * rtol;
    k_pcg_init<<<pc->nblocks, PCG_THREADS, 0, s>>>(o, d_b, d_x, pc->r, pc->scal, pc->partials, pc->ticket, pc->flags,
                                                    rtol2);
    NN_CHECK_LAUNCH(ctx, "k_pcg_init");
    int h_flags[2] = {0, 0};
    int it = 0;
    const int chunk = 16;
    int nchunks = 0;
    while (true) {
        NN_CUDA(ctx, cudaMemcpyAsync(h_flags, pc->flags, sizeof h_flags, cudaMemcpyDeviceToHost, s));
        NN_CUDA(ctx, cudaStreamSynchronize(s));
        if (h_flags[0] || it >= max_iter) break;
        if (pc->timing) {
            if ((int)pc->ev_a.size() <= nchunks) {
                cudaEvent_t a, b;
                NN_CUDA(ctx, cudaEventCreate(&a));
                NN_CUDA(ctx, cudaEventCreate(&b));
                pc->ev_a.push_back(a);
                pc->ev_b.push_back(b);
            }
            NN_CUDA(ctx, cudaEventRecord(pc->ev_a[nchunks], s));
        }
        for (int q = 0; q < chunk && it < max_iter; ++q, ++it) {
            float* p_old = (it & 1) ? pc->p1 : pc->p0;
            float* p_new = (it & 1) ? pc->p0 : pc->p1;
            k_pcg_dir_apply<<<pc->nblocks, PCG_THREADS, 0, s>>>(o, pc->r, p_old, p_new, pc->Ap, pc->scal, pc->partials,
                                                                 pc->ticket, pc->flags);
            NN_CHECK_LAUNCH(ctx, "k_pcg_dir_apply");
            k_pcg_update<<<pc->nblocks, PCG_THREADS, 0, s>>>(o, d_x, pc->r, p_new, pc->Ap, pc->scal, pc->partials,
                                                              pc->ticket, pc->flags, rtol2, max_iter);
            NN_CHECK_LAUNCH(ctx, "k_pcg_update");
        }
        if (pc->timing) NN_CUDA(ctx, cudaEventRecord(pc->ev_b[nchunks], s));
        ++nchunks;
    }
    double h_scal[S_COUNT];
    NN_CUDA(ctx, cudaMemcpyAsync(h_scal, pc->scal, sizeof h_scal, cudaMemcpyDeviceToHost, s));
    NN_CUDA(ctx, cudaStreamSynchronize(s));
    if (pc->timing) {
        float tot = 0.0f;
        for (int c = 0; c < nchunks; ++c) {
            float ms = 0.0f;
            NN_CUDA(ctx, cudaEventElapsedTime(&ms, pc->ev_a[c], pc->ev_b[c]));
            tot += ms;
        }
        pc->last_ms = tot;
        pc->last_iters = h_flags[1];
    }
    if (iters) *iters = h_flags[1];
    if (relres) *relres = h_scal[S_BB] > 0 ? std::sqrt(h_scal[S_RR] / h_scal[S_BB]) : 0.0;
    if (converged) *converged = h_flags[0] == 1;
    return NN_OK;
}

nn_status nn_pcg_stats(nn_pcg* pc, int* iters, double* relres, int* converged)
{
    nn_ctx* ctx = pc->ctx;
    int h_flags[2];
    double h_scal[S_COUNT];
    NN_CUDA(ctx, cudaMemcpyAsync(h_flags, pc->flags, sizeof h_flags, cudaMemcpyDeviceToHost, ctx->stream));
    NN_CUDA(ctx, cudaMemcpyAsync(h_scal, pc->scal, sizeof h_scal, cudaMemcpyDeviceToHost, ctx->stream));
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (iters) *iters = h_flags[1];
    if (relres) *relres = h_scal[S_BB] > 0 ? std::sqrt(h_scal[S_RR] / h_scal[S_BB]) : 0.0;
    if (converged) *converged = h_flags[0] == 1;
    return NN_OK;
}

extern "C" nn_status nn_pcg_solve(nn_pcg* pc, const float* d_b, float* d_x, double rtol, int max_iter, int* iters,
                                  double* relres)
{
    if (!pc || !d_b || !d_x || !(rtol > 0.0) || max_iter < 0) return NN_ERR_INVALID_ARG;
    int conv = 0;
    NN_TRY(nn_pcg_run_best(pc, d_b, d_x, rtol, max_iter, iters, relres, &conv));
    if (!conv) return nn_fail(pc->ctx, NN_ERR_NOT_CONVERGED, "PCG did not reach rtol %g in %d iterations", rtol, max_iter);
    return NN_OK;
}

void nn_pcg_info(const nn_pcg* pc, nn_ctx** ctx, int* nx, int* ny, int* nz, const float** invd, float* invd_const,
                 const float** D)
{
    *ctx = pc->ctx;
    *nx = pc->nx;
    *ny = pc->ny;
    *nz = pc->nz;
    *invd = pc->invd;
    *invd_const = pc->inv_diag_const;
    *D = pc->Dcell;
}

void nn_pcg_coefficients(const nn_pcg* pc, double* alpha, double* beta)
{
    *alpha = pc->alpha;
    *beta = pc->beta;
}

extern "C" nn_status nn_pcg_set_kernel_timing(nn_pcg* pc, int enable)
{
    if (!pc) return NN_ERR_INVALID_ARG;
    nn_pcg_set_timing(pc, enable != 0);
    return NN_OK;
}

extern "C" nn_status nn_pcg_kernel_time(nn_pcg* pc, float* ms, int* iters)
{
    if (!pc || !ms || !iters) return NN_ERR_INVALID_ARG;
    nn_pcg_last_timing(pc, ms, iters);
    return NN_OK;
}

// Asynchronous solve on a stream (single-kernel path only; UNSUPPORTED
// otherwise): n iterations enqueued now, the rest and the outcome at finish.
nn_status nn_pcg_async_begin(nn_pcg* pc, const float* d_b, float* d_x, double rtol, int max_iter, int n,
                             cudaStream_t cs)
{
    if (!pc->fast) return NN_ERR_UNSUPPORTED;
    return nn_cg_async_begin(pc->fast, d_b, d_x, rtol, max_iter, n, cs);
}

nn_status nn_pcg_async_finish(nn_pcg* pc, int* iters, double* relres, int* converged)
{
    if (!pc->fast) return NN_ERR_UNSUPPORTED;
    return nn_cg_async_finish(pc->fast, iters, relres, converged);
}

bool nn_pcg_async_supported(const nn_pcg* pc) { return pc->fast != nullptr; }

// The single-kernel TMA iteration when the grid allows it, else two kernels.
nn_status nn_pcg_run_best(nn_pcg* pc, const float* d_b, float* d_x, double rtol, int max_iter, int* iters,
                          double* relres, int* converged)
{
    if (pc->fast) return nn_cg_run(pc->fast, d_b, d_x, rtol, max_iter, iters, relres, converged);
    return nn_pcg_run(pc, d_b, d_x, rtol, max_iter, iters, relres, converged);
}

// Right-hand side for tile timing: values in [0.5, 1.5) from a hash of the
// cell index (no solve reaches its residual target on it within a trial).
__global__ void k_pcg_trial_rhs(float* b, int64_t G)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < G; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = 0.5f + (float)(((uint32_t)i * 2654435761u) >> 22) * (1.0f / 1024.0f);
}

// Tile depth of the single-kernel iteration (0: the grid runs the two-kernel PCG).
int nn_pcg_tile_depth(const nn_pcg* pc) { return pc->fast ? nn_cg_plan_tile_depth(pc->fast) : 0; }
void nn_pcg_set_tile_depth(nn_pcg* pc, int zc)
{
    if (pc->fast && zc >= 4) nn_cg_plan_set_tile_depth(pc->fast, zc);
}

// Tile autotuner of the single-kernel iteration (nn_cg_plan_autotune) on
// scratch vectors; NN_ERR_UNSUPPORTED when the grid runs the two-kernel PCG.
nn_status nn_pcg_autotune_tiles(nn_pcg* pc, int iters, int* tile_z, float* ms_per_iter)
{
    if (!pc || iters < 1) return NN_ERR_INVALID_ARG;
    if (!pc->fast) return NN_ERR_UNSUPPORTED;
    nn_ctx* ctx = pc->ctx;
    const int64_t G = (int64_t)pc->nx * pc->ny * pc->nz;
    float *b = nullptr, *x = nullptr;
    NN_TRY(nn_alloc(ctx, &b, (size_t)G));
    nn_status st = nn_alloc(ctx, &x, (size_t)G);
    if (st == NN_OK) {
        k_pcg_trial_rhs<<<nn_grid_for(ctx, G, 256, 8), 256, 0, ctx->stream>>>(b, G);
        st = nn_cuda_check(ctx, cudaPeekAtLastError(), "k_pcg_trial_rhs");
    }
    if (st == NN_OK) st = nn_cg_plan_autotune(pc->fast, b, x, iters, tile_z, ms_per_iter);
    cudaStreamSynchronize(ctx->stream);
    nn_release(b);
    nn_release(x);
    return st;
}

// ========================================================= no allocation ==
// nn_pcg_solve_noalloc: the same Jacobi-PCG as nn_pcg_create + nn_pcg_solve,
// for callers that may not allocate device memory (a host framework that owns
// the GPU's memory budget, or a real-time loop that cannot take the device-wide
// synchronisation of cudaMalloc/cudaFree).  Its work vectors, reduction
// partials and flags live in the fixed file-scope array below, which every GPU
// that loads this library holds until the process exits.  One scratch serves
// all calls on a device within a process, so calls whose work overlaps on the
// GPU race (each process has its own copy of the array).

namespace {
constexpr size_t NA_ALIGN(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr int NA_MAX_BLOCKS = 4096;  // reduction partials: grid-stride blocks per kernel
constexpr size_t NA_VEC = NA_ALIGN((size_t)NN_PCG_NOALLOC_MAX_CELLS * sizeof(float));
constexpr size_t NA_OFF_R = 0, NA_OFF_P0 = NA_VEC, NA_OFF_P1 = 2 * NA_VEC, NA_OFF_AP = 3 * NA_VEC,
                 NA_OFF_INVD = 4 * NA_VEC, NA_OFF_SCAL = 5 * NA_VEC;
constexpr size_t NA_OFF_PART = NA_OFF_SCAL + NA_ALIGN(S_COUNT * sizeof(double));
constexpr size_t NA_OFF_TICKET = NA_OFF_PART + NA_ALIGN(3 * (size_t)NA_MAX_BLOCKS * sizeof(double));
constexpr size_t NA_OFF_FLAGS = NA_OFF_TICKET + 256;
constexpr size_t NA_BYTES = NA_OFF_FLAGS + 256;
constexpr int NA_MAX_DEVICES = 64;
}  // namespace

// Host code sees this name as a host-side stand-in; the device address comes
// from cudaGetSymbolAddress (see noalloc_scratch below).
static __device__ __align__(256) unsigned char g_pcg_noalloc_scratch[NA_BYTES];

// Device address of the scratch on the current device, looked up once per
// device (the first call on a device does this, which also loads the module on
// that device; make that first call before any stream capture).  The address
// is kept for the life of the process; a cudaDeviceReset destroys the context
// it belongs to, so the entry point is not for use on a device after a reset.
static nn_status noalloc_scratch(int dev, unsigned char** out)
{
    static std::mutex mu;
    static unsigned char* addr[NA_MAX_DEVICES] = {};
    if (dev < 0 || dev >= NA_MAX_DEVICES) return NN_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_pcg_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return NN_ERR_CUDA;
        }
        addr[dev] = (unsigned char*)p;
    }
    *out = addr[dev];
    return NN_OK;
}

extern "C" nn_status nn_pcg_solve_noalloc(void* stream, int nx, int ny, int nz, double alpha, double beta,
                                          const float* d_Dcell, const float* d_b, float* d_x, double rtol,
                                          int max_iter, int* iters, double* relres)
{
    if (nx < 1 || ny < 1 || nz < 1 || !d_b || !d_x || !(alpha >= 0.0) || !(beta > -1.0) || !(rtol > 0.0) ||
        max_iter < 0)
        return NN_ERR_INVALID_ARG;
    const int64_t G = (int64_t)nx * ny * nz;
    if (G > (int64_t)NN_PCG_NOALLOC_MAX_CELLS) return NN_ERR_UNSUPPORTED;  // larger than the fixed scratch
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return NN_ERR_NO_DEVICE;
    }
    unsigned char* base = nullptr;
    NN_TRY(noalloc_scratch(dev, &base));
    // A context on the caller's stream that owns nothing (its error text is
    // dropped on return: callers of this entry point get the status only).
    nn_ctx ctx;
    ctx.device = dev;
    ctx.stream = (cudaStream_t)stream;
    if (cudaDeviceGetAttribute(&ctx.num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return NN_ERR_CUDA;
    }
    nn_pcg pc;
    pc.ctx = &ctx;
    pc.nx = nx; pc.ny = ny; pc.nz = nz;
    pc.G = G;
    pc.alpha = alpha;
    pc.beta = beta;
    pc.Dcell = d_Dcell;
    pc.inv_diag_const = (float)(1.0 / (1.0 + beta + 6.0 * alpha));
    pc.nblocks = std::min(nn_grid_for(&ctx, G, PCG_THREADS, 8), NA_MAX_BLOCKS);
    pc.r = (float*)(base + NA_OFF_R);
    pc.p0 = (float*)(base + NA_OFF_P0);
    pc.p1 = (float*)(base + NA_OFF_P1);
    pc.Ap = (float*)(base + NA_OFF_AP);
    pc.invd = d_Dcell ? (float*)(base + NA_OFF_INVD) : nullptr;
    pc.scal = (double*)(base + NA_OFF_SCAL);
    pc.partials = (double*)(base + NA_OFF_PART);
    pc.ticket = (unsigned int*)(base + NA_OFF_TICKET);
    pc.flags = (int*)(base + NA_OFF_FLAGS);
    // what must start at zero: the arrival ticket and the first direction
    // buffer (the first update multiplies it by beta = 0)
    NN_CUDA(&ctx, cudaMemsetAsync(pc.ticket, 0, sizeof(unsigned int), ctx.stream));
    NN_CUDA(&ctx, cudaMemsetAsync(pc.p0, 0, sizeof(float) * (size_t)G, ctx.stream));
    if (d_Dcell) {
        Op o = make_op(&pc);
        k_pcg_invdiag<<<pc.nblocks, PCG_THREADS, 0, ctx.stream>>>(o, pc.invd);
        NN_CHECK_LAUNCH(&ctx, "k_pcg_invdiag");
    }
    int conv = 0;
    NN_TRY(nn_pcg_run(&pc, d_b, d_x, rtol, max_iter, iters, relres, &conv));
    return conv ? NN_OK : NN_ERR_NOT_CONVERGED;
}
