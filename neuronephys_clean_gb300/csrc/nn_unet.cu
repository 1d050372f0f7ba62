// Learned preconditioner for the paracrine CG (no counterpart in the
// reference): a two-grid preconditioner whose coarse-grid correction is a
// 3-level 3D convolutional U-Net (16/32/64 channels, BF16 activations and
// weights, FP32 accumulation on the tensor cores), used inside flexible CG.
//
//   M r:  z1 = w D^-1 r                       (Jacobi pre-smoothing)
//         r1 = r - A z1
//         rc = R r1                           (2x average restriction)
//         v  = P (s * N(rc / s, log D_c))     (U-Net, s = rms(rc); piecewise-
//                                              constant prolongation)
//         z2 = z1 + g v,  g = (v, r1) / (v, A v)   (energy-minimising step)
//         z  = z2 + w D^-1 (r - A z2)         (Jacobi post-smoothing)
// The step g makes the coarse correction never increase the A-norm of the
// error, so an imperfect (or untrained) network cannot make M worse than the
// smoothing alone; g is formed on the device.
//
// The network is trained on the GPU by the project's own forward and backward
// kernels (nn_conv.cu) with Adam on pairs the solver generates: for a
// right-hand side b with solution x*, any iterate x_k gives the pair
// (r_k = b - A x_k, e_k = x* - x_k) with A e_k = r_k; after the same
// pre-smoothing the coarse target is R (e_k - z1).  Flexible CG (Notay 2000:
// p_k = z_k - (z_k, A p_{k-1}) / (p_{k-1}, A p_{k-1}) p_{k-1}) iterates to
// the same relative residual as the plain Jacobi-PCG, so only the iteration
// count changes.
//
// U-Net (N = level-0 grid, levels N, N/2, N/4):
//   e0a 16->16, e0b 16->16 (skip0) | pool | e1a 16->32, e1b 32->32 (skip1) |
//   pool | b2a 32->64, b2b 64->64 | up, cat skip1 | d1a 96->32, d1b 32->32 |
//   up, cat skip0 | d0a 48->16, d0b 16->16 | out 16->16 (channel 0 used)
// every conv but `out` followed by ReLU.  Concatenation is free: the skip
// tensors are written straight into the upper channel blocks of the decoder
// input buffers.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "nn_conv.cuh"

namespace {
constexpr int UT = 256;

enum { L_E0A = 0, L_E0B, L_E1A, L_E1B, L_B2A, L_B2B, L_D1A, L_D1B, L_D0A, L_D0B, L_OUT, NL };
constexpr int LCIN[NL] = {16, 16, 16, 32, 32, 64, 96, 32, 48, 16, 16};
constexpr int LCOUT[NL] = {16, 16, 32, 32, 64, 64, 32, 32, 16, 16, 16};
constexpr int LLEVEL[NL] = {0, 0, 1, 1, 2, 2, 1, 1, 0, 0, 0};

__device__ __forceinline__ void unpack8(const uint4& u, float* f)
{
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        f[2 * i] = __uint_as_float(w[i] << 16);
        f[2 * i + 1] = __uint_as_float(w[i] & 0xFFFF0000u);
    }
}

__device__ __forceinline__ uint4 pack8(const float* f)
{
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
        w[i] = *reinterpret_cast<const uint32_t*>(&h);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

__device__ __forceinline__ int64_t vox(const nn_act_geom& g, int z, int y, int x)
{
    return (int64_t)(z + 1) * g.P + (int64_t)(y + 1) * g.R + x + 1;
}

#define GRID_LOOP(i, n) for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// coarse(c) = mean of its 8 children, per 8-channel block
__global__ void k_pool(const uint4* src, nn_act_geom gf, const uint4* dummy, uint4* dst, nn_act_geom gc, int groups)
{
    nn_grid_dep_wait();
    const int64_t G = (int64_t)gc.nz * gc.ny * gc.nx;
    GRID_LOOP(e, G * groups)
    {
        const int gb = (int)(e / G);
        const int64_t c = e - gb * G;
        const int x = (int)(c % gc.nx), y = (int)((c / gc.nx) % gc.ny), z = (int)(c / ((int64_t)gc.nx * gc.ny));
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int q = 0; q < 8; ++q) {
            float f[8];
            unpack8(src[gb * gf.S + gf.GD + vox(gf, 2 * z + (q >> 2), 2 * y + ((q >> 1) & 1), 2 * x + (q & 1))], f);
#pragma unroll
            for (int i = 0; i < 8; ++i) acc[i] += f[i];
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i] *= 0.125f;
        dst[gb * gc.S + gc.GD + vox(gc, z, y, x)] = pack8(acc);
    }
    (void)dummy;
}

// coarse(c) = sum of its 8 children   (adjoint of the nearest upsampling)
__global__ void k_sumpool(const uint4* src, nn_act_geom gf, uint4* dst, nn_act_geom gc, int groups)
{
    const int64_t G = (int64_t)gc.nz * gc.ny * gc.nx;
    GRID_LOOP(e, G * groups)
    {
        const int gb = (int)(e / G);
        const int64_t c = e - gb * G;
        const int x = (int)(c % gc.nx), y = (int)((c / gc.nx) % gc.ny), z = (int)(c / ((int64_t)gc.nx * gc.ny));
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int q = 0; q < 8; ++q) {
            float f[8];
            unpack8(src[gb * gf.S + gf.GD + vox(gf, 2 * z + (q >> 2), 2 * y + ((q >> 1) & 1), 2 * x + (q & 1))], f);
#pragma unroll
            for (int i = 0; i < 8; ++i) acc[i] += f[i];
        }
        dst[gb * gc.S + gc.GD + vox(gc, z, y, x)] = pack8(acc);
    }
}

// out = (a + up(b) / 8) * (mask > 0): gradient of a skip tensor that feeds
// both the concatenation (a) and the average pooling (b = gradient of the pooled tensor)
__global__ void k_skip_grad(const uint4* a, const uint4* b, nn_act_geom gc, const uint4* mask, uint4* out,
                            nn_act_geom gf, int groups)
{
    const int64_t G = (int64_t)gf.nz * gf.ny * gf.nx;
    GRID_LOOP(e, G * groups)
    {
        const int gb = (int)(e / G);
        const int64_t c = e - gb * G;
        const int x = (int)(c % gf.nx), y = (int)((c / gf.nx) % gf.ny), z = (int)(c / ((int64_t)gf.nx * gf.ny));
        const int64_t o = gb * gf.S + gf.GD + vox(gf, z, y, x);
        float fa[8], fb[8], fm[8], r[8];
        unpack8(a[o], fa);
        unpack8(b[gb * gc.S + gc.GD + vox(gc, z >> 1, y >> 1, x >> 1)], fb);
        unpack8(mask[o], fm);
#pragma unroll
        for (int i = 0; i < 8; ++i) r[i] = fm[i] > 0.0f ? fa[i] + 0.125f * fb[i] : 0.0f;
        out[o] = pack8(r);
    }
}

// network input: channel 0 = r / s, channel 1 = log D (0 if absent), 2..15 = 0
// (d given: the input is r / d, formed here)
__global__ void k_net_input(const float* r, const float* d, const float* logd, const double* s, uint4* in,
                            nn_act_geom g)
{
    nn_grid_dep_wait();
    const int64_t G = (int64_t)g.nz * g.ny * g.nx;
    const float inv = s[0] > 0.0 ? (float)(1.0 / s[0]) : 0.0f;
    GRID_LOOP(c, G)
    {
        const int x = (int)(c % g.nx), y = (int)((c / g.nx) % g.ny), z = (int)(c / ((int64_t)g.nx * g.ny));
        const float rc = d ? r[c] / d[c] : r[c];
        float f[8] = {rc * inv, logd ? logd[c] : 0.0f, 0, 0, 0, 0, 0, 0};
        in[g.GD + vox(g, z, y, x)] = pack8(f);
    }
}

// loss gradient: channel 0 = y - t / s, other channels 0; loss += sum (y - t/s)^2
__global__ void k_net_loss(const float* y32, const float* t, const double* s, uint4* gout, nn_act_geom g, double* loss)
{
    const int64_t G = (int64_t)g.nz * g.ny * g.nx;
    const float inv = s[0] > 0.0 ? (float)(1.0 / s[0]) : 0.0f;
    double acc = 0.0;
    GRID_LOOP(c, G)
    {
        const int x = (int)(c % g.nx), y = (int)((c / g.nx) % g.ny), z = (int)(c / ((int64_t)g.nx * g.ny));
        const float d = y32[c] - t[c] * inv;
        float f[8] = {d, 0, 0, 0, 0, 0, 0, 0};
        gout[g.GD + vox(g, z, y, x)] = pack8(f);
        acc += (double)d * d;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

// sum of squares -> s = sqrt(mean)
// s[0] = rms of v (of v / d with d given) in one launch: per-block FP64
// partial sums; the last block to finish adds them in block order and resets
// the ticket.  Its grid must be the partials' length.
__global__ void __launch_bounds__(UT) k_rms(const float* v, const float* d, int64_t n, double* partials,
                                            unsigned int* ticket, double* s)
{
    nn_grid_dep_wait();
    __shared__ double ws[UT / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double acc = 0.0;
    GRID_LOOP(i, n)
    {
        const float x = d ? v[i] / d[i] : v[i];
        acc += (double)x * x;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) ws[w] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int u = 0; u < UT / 32; ++u) t += ws[u];
        partials[blockIdx.x] = t;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const volatile double* pp = partials;
    double t = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += UT) t += pp[k];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    __syncthreads();
    if (lane == 0) ws[w] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int u = 0; u < UT / 32; ++u) tot += ws[u];
        s[0] = sqrt(tot / (double)n);
        *ticket = 0;
    }
}

__global__ void k_scale_out(const float* y, const double* s, float* z, int64_t n)
{
    const float sc = (float)s[0];
    GRID_LOOP(i, n) z[i] = y[i] * sc;
}

__global__ void k_init_normal(float* w, int64_t n, float stdv, uint64_t seed, uint32_t layer)
{
    GRID_LOOP(i, n)
    {
        const nn_u4 r = nn_philox(seed, (uint32_t)i, layer, 0x5eedu, 0x77u);
        const float u1 = nn_u01f_open(r.x), u2 = nn_u01f(r.y);
        w[i] = stdv * sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
    }
}

__global__ void k_adam(float* w, float* g, float* m, float* v, int64_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
    GRID_LOOP(i, n)
    {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        g[i] = 0.0f;
    }
}

// ---- fine-grid parts of the two-grid preconditioner (dense FP32) ----

struct Fine {
    int nx, ny, nz;
    const float* invd;  // per cell, or null
    float invd_c;
};

__device__ __forceinline__ float invd_at(const Fine& f, int64_t c) { return f.invd ? f.invd[c] : f.invd_c; }

__global__ void k_jacobi(Fine f, const float* r, float omega, float* z)
{
    const int64_t G = (int64_t)f.nx * f.ny * f.nz;
    GRID_LOOP(c, G) z[c] = omega * invd_at(f, c) * r[c];
}

// rc = mean over children of (r - t)
__global__ void k_restrict_diff(Fine f, const float* r, const float* t, float* rc)
{
    const int cx = f.nx / 2, cy = f.ny / 2, cz = f.nz / 2;
    const int64_t G = (int64_t)cx * cy * cz;
    const int64_t sy = f.nx, sz = (int64_t)f.nx * f.ny;
    GRID_LOOP(c, G)
    {
        const int x = (int)(c % cx), y = (int)((c / cx) % cy), z = (int)(c / ((int64_t)cx * cy));
        const int64_t b = 2 * x + sy * 2 * y + sz * 2 * z;
        float acc = 0.0f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int64_t o = b + (q & 1) + sy * ((q >> 1) & 1) + sz * (q >> 2);
            acc += r[o] - (t ? t[o] : 0.0f);
        }
        rc[c] = 0.125f * acc;
    }
}

// out = P ec (nearest)
__global__ void k_prolong(Fine f, const float* ec, float* out)
{
    const int cx = f.nx / 2, cy = f.ny / 2;
    const int64_t G = (int64_t)f.nx * f.ny * f.nz;
    GRID_LOOP(c, G)
    {
        const int x = (int)(c % f.nx), y = (int)((c / f.nx) % f.ny), z = (int)(c / ((int64_t)f.nx * f.ny));
        out[c] = ec[(x >> 1) + (int64_t)cx * ((y >> 1) + (int64_t)cy * (z >> 1))];
    }
}

// z += omega D^-1 (r - t)
__global__ void k_post_smooth(Fine f, const float* r, const float* t, float omega, float* z)
{
    const int64_t G = (int64_t)f.nx * f.ny * f.nz;
    GRID_LOOP(c, G) z[c] += omega * invd_at(f, c) * (r[c] - t[c]);
}

// training-pair transform: e1 = e - z1 (z1 = omega D^-1 r); rc from r - A z1 (given t = A z1)
__global__ void k_pair_target(Fine f, const float* e, const float* r, float omega, float* ec)
{
    const int cx = f.nx / 2, cy = f.ny / 2, cz = f.nz / 2;
    const int64_t G = (int64_t)cx * cy * cz;
    const int64_t sy = f.nx, sz = (int64_t)f.nx * f.ny;
    GRID_LOOP(c, G)
    {
        const int x = (int)(c % cx), y = (int)((c / cx) % cy), z = (int)(c / ((int64_t)cx * cy));
        const int64_t b = 2 * x + sy * 2 * y + sz * 2 * z;
        float acc = 0.0f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int64_t o = b + (q & 1) + sy * ((q >> 1) & 1) + sz * (q >> 2);
            acc += e[o] - omega * invd_at(f, o) * r[o];
        }
        ec[c] = 0.125f * acc;
    }
}

// log of the cell field averaged over each coarse cell's children
__global__ void k_logd_coarse(Fine f, const float* D, float* out)
{
    const int cx = f.nx / 2, cy = f.ny / 2, cz = f.nz / 2;
    const int64_t G = (int64_t)cx * cy * cz;
    const int64_t sy = f.nx, sz = (int64_t)f.nx * f.ny;
    GRID_LOOP(c, G)
    {
        const int x = (int)(c % cx), y = (int)((c / cx) % cy), z = (int)(c / ((int64_t)cx * cy));
        const int64_t b = 2 * x + sy * 2 * y + sz * 2 * z;
        float acc = 0.0f;
#pragma unroll
        for (int q = 0; q < 8; ++q) acc += logf(D[b + (q & 1) + sy * ((q >> 1) & 1) + sz * (q >> 2)]);
        out[c] = 0.125f * acc;
    }
}

// out[0] += (v, r - t), out[1] += (v, tv)
__global__ void k_dot_step(const float* v, const float* r, const float* t, const float* tv, int64_t n, double* out)
{
    double a = 0.0, b = 0.0;
    GRID_LOOP(i, n)
    {
        a += (double)v[i] * (r[i] - t[i]);
        b += (double)v[i] * tv[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&out[0], a);
        atomicAdd(&out[1], b);
    }
}

// z += g v, t += g tv with g = d[0] / d[1] (0 unless d[1] > 0)
__global__ void k_coarse_step(const double* d, const float* v, const float* tv, float* z, float* t, int64_t n)
{
    const float g = d[1] > 0.0 ? (float)(d[0] / d[1]) : 0.0f;
    GRID_LOOP(i, n)
    {
        z[i] += g * v[i];
        t[i] += g * tv[i];
    }
}

__global__ void k_dot(const float* a, const float* b, int64_t n, double* out)
{
    double acc = 0.0;
    GRID_LOOP(i, n) acc += (double)a[i] * b[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

// y += a x
__global__ void k_axpy(float a, const float* x, float* y, int64_t n) { GRID_LOOP(i, n) y[i] += a * x[i]; }
// p = z + b p
__global__ void k_xpby(const float* z, float b, float* p, int64_t n) { GRID_LOOP(i, n) p[i] = z[i] + b * p[i]; }
// r = b - t
__global__ void k_sub(const float* b, const float* t, float* r, int64_t n) { GRID_LOOP(i, n) r[i] = b[i] - t[i]; }
}  // namespace

// ------------------------------------------------------------- U-Net --

struct nn_unet {
    nn_ctx* ctx = nullptr;
    nn_act_geom g[3];
    int64_t G0 = 0;
    struct Layer {
        float *w = nullptr, *b = nullptr, *gw = nullptr, *gb = nullptr;
        float *mw = nullptr, *vw = nullptr, *mb = nullptr, *vb = nullptr;
        void *wp = nullptr, *wpa = nullptr;
        int64_t nw = 0;
    } L[NL];
    // activations
    void *I0 = nullptr, *E0a = nullptr, *CAT0 = nullptr, *D0a = nullptr, *D0b = nullptr, *OUT = nullptr;
    void *P1 = nullptr, *E1a = nullptr, *CAT1 = nullptr, *D1a = nullptr, *D1b = nullptr;
    void *P2 = nullptr, *B2a = nullptr, *B2b = nullptr;
    // gradients
    void *gOUT = nullptr, *gD0b = nullptr, *gD0a = nullptr, *gCAT0 = nullptr, *gSK0 = nullptr, *gE0a = nullptr;
    void *gD1b = nullptr, *gD1a = nullptr, *gCAT1 = nullptr, *gSK1 = nullptr, *gE1a = nullptr, *gP1 = nullptr;
    void *gB2b = nullptr, *gB2a = nullptr, *gP2 = nullptr;
    float* y32 = nullptr;
    double* scal = nullptr;  // [0] s, [1] loss
    double* partials = nullptr;  // k_rms block sums
    unsigned int* ticket = nullptr;
    int rms_blocks = 0;
    int* err = nullptr;
    int adam_t = 0;
    std::vector<void*> bufs;
};

static nn_status act_alloc(nn_unet* u, void** p, int level, int channels)
{
    const size_t bytes = nn_act_bytes(u->g[level], channels);
    unsigned char* q = nullptr;
    NN_TRY(nn_alloc(u->ctx, &q, bytes));
    u->bufs.push_back(q);
    NN_CUDA(u->ctx, cudaMemsetAsync(q, 0, bytes, u->ctx->stream));
    *p = q;
    return NN_OK;
}

template <class T>
static nn_status buf_alloc(nn_unet* u, T** p, size_t n)
{
    NN_TRY(nn_alloc(u->ctx, p, n));
    u->bufs.push_back((void*)*p);
    NN_CUDA(u->ctx, cudaMemsetAsync(*p, 0, n * sizeof(T), u->ctx->stream));
    return NN_OK;
}

static uint4* blk(void* act, const nn_act_geom& g, int group) { return (uint4*)act + group * g.S; }

static nn_status unet_repack(nn_unet* u, int l)
{
    NN_TRY(nn_conv_pack(u->ctx, LCIN[l], LCOUT[l], u->L[l].w, 0, u->L[l].wp));
    if (l != L_E0A) NN_TRY(nn_conv_pack(u->ctx, LCIN[l], LCOUT[l], u->L[l].w, 1, u->L[l].wpa));
    return NN_OK;
}

void nn_unet_free(nn_unet* u)
{
    if (!u) return;
    if (u->ctx) cudaStreamSynchronize(u->ctx->stream);
    for (void* p : u->bufs) cudaFree(p);
    nn_ctx* ctx = u->ctx;
    delete u;
    if (ctx) nn_ctx_release(ctx);
}

nn_status nn_unet_make(nn_ctx* ctx, int nz, int ny, int nx, uint64_t seed, nn_unet** out)
{
    *out = nullptr;
    if (nz < 4 || ny < 4 || nx < 4 || nz % 4 || ny % 4 || nx % 4)
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "U-Net grid %dx%dx%d: each side a multiple of 4", nz, ny, nx);
    nn_unet* u = new nn_unet();
    u->ctx = ctx;
    nn_ctx_retain(ctx);
    u->g[0] = nn_act_geometry(nz, ny, nx);
    u->g[1] = nn_act_geometry(nz / 2, ny / 2, nx / 2);
    u->g[2] = nn_act_geometry(nz / 4, ny / 4, nx / 4);
    u->G0 = (int64_t)nz * ny * nx;
    nn_status st = NN_OK;
    for (int l = 0; l < NL && st == NN_OK; ++l) {
        auto& L = u->L[l];
        L.nw = 27LL * LCIN[l] * LCOUT[l];
        unsigned char *wp = nullptr, *wpa = nullptr;
        st = buf_alloc(u, &L.w, L.nw);
        if (st == NN_OK) st = buf_alloc(u, &L.gw, L.nw);
        if (st == NN_OK) st = buf_alloc(u, &L.mw, L.nw);
        if (st == NN_OK) st = buf_alloc(u, &L.vw, L.nw);
        if (st == NN_OK) st = buf_alloc(u, &L.b, LCOUT[l]);
        if (st == NN_OK) st = buf_alloc(u, &L.gb, LCOUT[l]);
        if (st == NN_OK) st = buf_alloc(u, &L.mb, LCOUT[l]);
        if (st == NN_OK) st = buf_alloc(u, &L.vb, LCOUT[l]);
        if (st == NN_OK) st = buf_alloc(u, &wp, nn_conv_packed_weight_bytes(LCIN[l], LCOUT[l]));
        if (st == NN_OK) st = buf_alloc(u, &wpa, nn_conv_packed_weight_bytes(LCIN[l], LCOUT[l]));
        L.wp = wp;
        L.wpa = wpa;
        if (st == NN_OK) {
            // He initialisation (input layer: two real input channels; output layer scaled down)
            const int fan = 27 * (l == L_E0A ? 2 : LCIN[l]);
            const float sd = sqrtf(2.0f / fan) * (l == L_OUT ? 0.1f : 1.0f);
            k_init_normal<<<nn_grid_for(ctx, L.nw, UT, 4), UT, 0, ctx->stream>>>(L.w, L.nw, sd, seed, (uint32_t)l);
            st = nn_cuda_check(ctx, cudaGetLastError(), "k_init_normal");
            ctx->launches++;
        }
        if (st == NN_OK) st = unet_repack(u, l);
    }
    // activations: level 0
    if (st == NN_OK) st = act_alloc(u, &u->I0, 0, 16);
    if (st == NN_OK) st = act_alloc(u, &u->E0a, 0, 16);
    if (st == NN_OK) st = act_alloc(u, &u->CAT0, 0, 48);
    if (st == NN_OK) st = act_alloc(u, &u->D0a, 0, 16);
    if (st == NN_OK) st = act_alloc(u, &u->D0b, 0, 16);
    if (st == NN_OK) st = act_alloc(u, &u->OUT, 0, 16);
    if (st == NN_OK) st = act_alloc(u, &u->P1, 1, 16);
    if (st == NN_OK) st = act_alloc(u, &u->E1a, 1, 32);
    if (st == NN_OK) st = act_alloc(u, &u->CAT1, 1, 96);
    if (st == NN_OK) st = act_alloc(u, &u->D1a, 1, 32);
    if (st == NN_OK) st = act_alloc(u, &u->D1b, 1, 32);
    if (st == NN_OK) st = act_alloc(u, &u->P2, 2, 32);
    if (st == NN_OK) st = act_alloc(u, &u->B2a, 2, 64);
    if (st == NN_OK) st = act_alloc(u, &u->B2b, 2, 64);
    // gradients
    if (st == NN_OK) st = act_alloc(u, &u->gOUT, 0, 16);
    if (st == NN_OK) st = act_alloc(u, &u->gD0b, 0, 16);
    if (st == NN_OK) st = act_alloc(u, &u->gD0a, 0, 16);
    if (st == NN_OK) st = act_alloc(u, &u->gCAT0, 0, 48);
    if (st == NN_OK) st = act_alloc(u, &u->gSK0, 0, 16);
    if (st == NN_OK) st = act_alloc(u, &u->gE0a, 0, 16);
    if (st == NN_OK) st = act_alloc(u, &u->gD1b, 1, 32);
    if (st == NN_OK) st = act_alloc(u, &u->gD1a, 1, 32);
    if (st == NN_OK) st = act_alloc(u, &u->gCAT1, 1, 96);
    if (st == NN_OK) st = act_alloc(u, &u->gSK1, 1, 32);
    if (st == NN_OK) st = act_alloc(u, &u->gE1a, 1, 32);
    if (st == NN_OK) st = act_alloc(u, &u->gP1, 1, 16);
    if (st == NN_OK) st = act_alloc(u, &u->gB2b, 2, 64);
    if (st == NN_OK) st = act_alloc(u, &u->gB2a, 2, 64);
    if (st == NN_OK) st = act_alloc(u, &u->gP2, 2, 32);
    if (st == NN_OK) st = buf_alloc(u, &u->y32, (size_t)u->G0);
    if (st == NN_OK) st = buf_alloc(u, &u->scal, 4);
    u->rms_blocks = nn_grid_for(ctx, u->G0, UT, 8);
    if (st == NN_OK) st = buf_alloc(u, &u->partials, (size_t)u->rms_blocks);
    if (st == NN_OK) st = buf_alloc(u, &u->ticket, 1);
    if (st == NN_OK) st = buf_alloc(u, &u->err, 1);
    if (st != NN_OK) {
        nn_unet_free(u);
        return st;
    }
    *out = u;
    return NN_OK;
}

static nn_status conv(nn_unet* u, int l, const void* x, void* y, bool relu, const void* mask = nullptr,
                      float* y32 = nullptr, const double* y32_scale = nullptr, void* up = nullptr)
{
    // up: the output also upsampled into the next finer level's activation
    const nn_act_geom* gup = up ? &u->g[LLEVEL[l] - 1] : nullptr;
    return nn_conv_forward(u->ctx, u->g[LLEVEL[l]], LCIN[l], LCOUT[l], x, u->L[l].wp, u->L[l].b, relu ? 1 : 0, mask,
                           y, y32, u->err, y32_scale, up, gup);
}

// input gradient of layer l (adjoint weights), masked by `mask` (> 0) if given
static nn_status conv_adj(nn_unet* u, int l, const void* gy, void* gx, const void* mask)
{
    return nn_conv_forward(u->ctx, u->g[LLEVEL[l]], LCOUT[l], LCIN[l], gy, u->L[l].wpa, nullptr, 0, mask, gx,
                           nullptr, u->err);
}

static nn_status wgrad(nn_unet* u, int l, const void* x, const void* gy)
{
    return nn_conv_wgrad(u->ctx, u->g[LLEVEL[l]], LCIN[l], LCOUT[l], x, gy, u->L[l].gw, u->L[l].gb, u->err);
}

template <class K, class... A>
static nn_status launch(nn_ctx* ctx, int64_t work, const char* what, K kern, A... args)
{
    kern<<<nn_grid_for(ctx, work, UT, 8), UT, 0, ctx->stream>>>(args...);
    NN_CHECK_LAUNCH(ctx, what);
    return NN_OK;
}

// the same as a programmatic dependent of the kernel before it (the kernel
// starts with nn_grid_dep_wait)
template <class... KA, class... A>
static nn_status launch_pdl(nn_ctx* ctx, int64_t work, const char* what, void (*kern)(KA...), A... args)
{
    NN_CUDA(ctx, nn_launch_pdl(kern, dim3(nn_grid_for(ctx, work, UT, 8)), dim3(UT), 0, ctx->stream, args...));
    NN_CHECK_LAUNCH(ctx, what);
    return NN_OK;
}

// forward pass; rc: dense level-0 input (divided by d when d is given, then
// by its rms s in k_net_input).  out (nullable): the result times s, written
// by the output layer, instead of the unscaled y32.  Every kernel is a
// programmatic dependent of the one before it.
static nn_status unet_forward(nn_unet* u, const float* rc, const float* logd, const float* d = nullptr,
                              float* out = nullptr)
{
    nn_ctx* ctx = u->ctx;
    const nn_act_geom &g0 = u->g[0], &g1 = u->g[1], &g2 = u->g[2];
    NN_CUDA(ctx, nn_launch_pdl(k_rms, dim3(u->rms_blocks), dim3(UT), 0, ctx->stream, rc, d, u->G0, u->partials,
                               u->ticket, u->scal));
    NN_CHECK_LAUNCH(ctx, "k_rms");
    NN_TRY(launch_pdl(ctx, u->G0, "k_net_input", k_net_input, rc, d, logd, (const double*)u->scal, (uint4*)u->I0, g0));
    void* SK0 = blk(u->CAT0, g0, 4);  // skip0 = channels 32..47 of CAT0
    void* SK1 = blk(u->CAT1, g1, 8);  // skip1 = channels 64..95 of CAT1
    NN_TRY(conv(u, L_E0A, u->I0, u->E0a, true));
    NN_TRY(conv(u, L_E0B, u->E0a, SK0, true));
    const int64_t G1 = (int64_t)g1.nz * g1.ny * g1.nx, G2 = (int64_t)g2.nz * g2.ny * g2.nx;
    NN_TRY(launch_pdl(ctx, G1 * 2, "k_pool", k_pool, (const uint4*)SK0, g0, (const uint4*)nullptr, (uint4*)u->P1, g1, 2));
    NN_TRY(conv(u, L_E1A, u->P1, u->E1a, true));
    NN_TRY(conv(u, L_E1B, u->E1a, SK1, true));
    NN_TRY(launch_pdl(ctx, G2 * 4, "k_pool", k_pool, (const uint4*)SK1, g1, (const uint4*)nullptr, (uint4*)u->P2, g2, 4));
    NN_TRY(conv(u, L_B2A, u->P2, u->B2a, true));
    NN_TRY(conv(u, L_B2B, u->B2a, u->B2b, true, nullptr, nullptr, nullptr, u->CAT1));  // + upsampled into CAT1
    NN_TRY(conv(u, L_D1A, u->CAT1, u->D1a, true));
    NN_TRY(conv(u, L_D1B, u->D1a, u->D1b, true, nullptr, nullptr, nullptr, u->CAT0));  // + upsampled into CAT0
    NN_TRY(conv(u, L_D0A, u->CAT0, u->D0a, true));
    NN_TRY(conv(u, L_D0B, u->D0a, u->D0b, true));
    NN_TRY(conv(u, L_OUT, u->D0b, u->OUT, false, nullptr, out ? out : u->y32, out ? (const double*)u->scal : nullptr));
    return NN_OK;
}

static nn_status unet_backward(nn_unet* u)
{
    nn_ctx* ctx = u->ctx;
    const nn_act_geom &g0 = u->g[0], &g1 = u->g[1], &g2 = u->g[2];
    const int64_t G1 = (int64_t)g1.nz * g1.ny * g1.nx, G2 = (int64_t)g2.nz * g2.ny * g2.nx;
    void* SK0 = blk(u->CAT0, g0, 4);
    void* SK1 = blk(u->CAT1, g1, 8);
    // level 0 decoder
    NN_TRY(wgrad(u, L_OUT, u->D0b, u->gOUT));
    NN_TRY(conv_adj(u, L_OUT, u->gOUT, u->gD0b, u->D0b));
    NN_TRY(wgrad(u, L_D0B, u->D0a, u->gD0b));
    NN_TRY(conv_adj(u, L_D0B, u->gD0b, u->gD0a, u->D0a));
    NN_TRY(wgrad(u, L_D0A, u->CAT0, u->gD0a));
    NN_TRY(conv_adj(u, L_D0A, u->gD0a, u->gCAT0, u->CAT0));
    // up (level 1 -> 0): adjoint is the sum over the children
    NN_TRY(launch(ctx, G1 * 4, "k_sumpool", k_sumpool, (const uint4*)u->gCAT0, g0, (uint4*)u->gD1b, g1, 4));
    // level 1 decoder
    NN_TRY(wgrad(u, L_D1B, u->D1a, u->gD1b));
    NN_TRY(conv_adj(u, L_D1B, u->gD1b, u->gD1a, u->D1a));
    NN_TRY(wgrad(u, L_D1A, u->CAT1, u->gD1a));
    NN_TRY(conv_adj(u, L_D1A, u->gD1a, u->gCAT1, u->CAT1));
    NN_TRY(launch(ctx, G2 * 8, "k_sumpool", k_sumpool, (const uint4*)u->gCAT1, g1, (uint4*)u->gB2b, g2, 8));
    // bottleneck
    NN_TRY(wgrad(u, L_B2B, u->B2a, u->gB2b));
    NN_TRY(conv_adj(u, L_B2B, u->gB2b, u->gB2a, u->B2a));
    NN_TRY(wgrad(u, L_B2A, u->P2, u->gB2a));
    NN_TRY(conv_adj(u, L_B2A, u->gB2a, u->gP2, nullptr));
    // skip1: concatenation part + pooled part, through its ReLU
    NN_TRY(launch(ctx, G1 * 4, "k_skip_grad", k_skip_grad, (const uint4*)blk(u->gCAT1, g1, 8), (const uint4*)u->gP2,
                  g2, (const uint4*)SK1, (uint4*)u->gSK1, g1, 4));
    NN_TRY(wgrad(u, L_E1B, u->E1a, u->gSK1));
    NN_TRY(conv_adj(u, L_E1B, u->gSK1, u->gE1a, u->E1a));
    NN_TRY(wgrad(u, L_E1A, u->P1, u->gE1a));
    NN_TRY(conv_adj(u, L_E1A, u->gE1a, u->gP1, nullptr));
    NN_TRY(launch(ctx, u->G0 * 2, "k_skip_grad", k_skip_grad, (const uint4*)blk(u->gCAT0, g0, 4), (const uint4*)u->gP1,
                  g1, (const uint4*)SK0, (uint4*)u->gSK0, g0, 2));
    NN_TRY(wgrad(u, L_E0B, u->E0a, u->gSK0));
    NN_TRY(conv_adj(u, L_E0B, u->gSK0, u->gE0a, u->E0a));
    NN_TRY(wgrad(u, L_E0A, u->I0, u->gE0a));
    return NN_OK;
}

static nn_status unet_adam(nn_unet* u, float lr)
{
    nn_ctx* ctx = u->ctx;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    u->adam_t++;
    const float c1 = 1.0f / (1.0f - powf(b1, (float)u->adam_t)), c2 = 1.0f / (1.0f - powf(b2, (float)u->adam_t));
    for (int l = 0; l < NL; ++l) {
        auto& L = u->L[l];
        NN_TRY(launch(ctx, L.nw, "k_adam", k_adam, L.w, L.gw, L.mw, L.vw, L.nw, lr, b1, b2, eps, c1, c2));
        NN_TRY(launch(ctx, LCOUT[l], "k_adam", k_adam, L.b, L.gb, L.mb, L.vb, (int64_t)LCOUT[l], lr, b1, b2, eps, c1, c2));
        NN_TRY(unet_repack(u, l));
    }
    return NN_OK;
}

static nn_status check_err(nn_unet* u)
{
    int h = 0;
    NN_CUDA(u->ctx, cudaMemcpyAsync(&h, u->err, sizeof(int), cudaMemcpyDeviceToHost, u->ctx->stream));
    NN_CUDA(u->ctx, cudaStreamSynchronize(u->ctx->stream));
    if (h) return nn_fail(u->ctx, NN_ERR_TIMEOUT, "k_conv3: a pipeline wait timed out");
    return NN_OK;
}

// ------------------------------------------------ learned preconditioner --

struct nn_learned {
    nn_ctx* ctx = nullptr;
    nn_pcg* pc = nullptr;
    Fine f{};
    int64_t G = 0, Gc = 0;
    float omega = 0.8f;
    nn_unet* net = nullptr;
    float* logd = nullptr;  // coarse log D (null without D)
    float *t = nullptr, *z1 = nullptr, *rc = nullptr, *ec = nullptr;  // work
    float *v = nullptr, *tv = nullptr;
    double* step = nullptr;
    float *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;     // FCG vectors
    double* dots = nullptr;
    std::vector<float*> pair_r, pair_e;  // coarse training pairs
    uint64_t rng = 0x9E3779B97F4A7C15ull;
    int use_net = 1;
};

static nn_status learned_apply(nn_learned* lp, const float* r, float* z)
{
    nn_ctx* ctx = lp->ctx;
    NN_TRY(launch(ctx, lp->G, "k_jacobi", k_jacobi, lp->f, r, lp->omega, lp->z1));
    NN_TRY(nn_pcg_apply(lp->pc, lp->z1, lp->t));
    if (lp->use_net) {
        NN_TRY(launch(ctx, lp->Gc, "k_restrict_diff", k_restrict_diff, lp->f, r, (const float*)lp->t, lp->rc));
        NN_TRY(unet_forward(lp->net, lp->rc, lp->logd));
        NN_TRY(launch(ctx, lp->Gc, "k_scale_out", k_scale_out, (const float*)lp->net->y32, (const double*)lp->net->scal,
                      lp->ec, lp->Gc));
        NN_TRY(launch(ctx, lp->G, "k_prolong", k_prolong, lp->f, (const float*)lp->ec, lp->v));
        NN_TRY(nn_pcg_apply(lp->pc, lp->v, lp->tv));
        NN_CUDA(ctx, cudaMemsetAsync(lp->step, 0, 2 * sizeof(double), ctx->stream));
        NN_TRY(launch(ctx, lp->G, "k_dot_step", k_dot_step, (const float*)lp->v, r, (const float*)lp->t,
                      (const float*)lp->tv, lp->G, lp->step));
        NN_TRY(launch(ctx, lp->G, "k_coarse_step", k_coarse_step, (const double*)lp->step, (const float*)lp->v,
                      (const float*)lp->tv, lp->z1, lp->t, lp->G));
    }
    NN_CUDA(ctx, cudaMemcpyAsync(z, lp->z1, sizeof(float) * lp->G, cudaMemcpyDeviceToDevice, ctx->stream));
    NN_TRY(launch(ctx, lp->G, "k_post_smooth", k_post_smooth, lp->f, r, (const float*)lp->t, lp->omega, z));
    return NN_OK;
}

static nn_status dot(nn_learned* lp, const float* a, const float* b, double* out)
{
    nn_ctx* ctx = lp->ctx;
    NN_CUDA(ctx, cudaMemsetAsync(lp->dots, 0, sizeof(double), ctx->stream));
    NN_TRY(launch(ctx, lp->G, "k_dot", k_dot, a, b, lp->G, lp->dots));
    NN_CUDA(ctx, cudaMemcpyAsync(out, lp->dots, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return NN_OK;
}

extern "C" nn_status nn_learned_create(nn_pcg* pc, uint64_t seed, nn_learned** out)
{
    if (!pc || !out) return NN_ERR_INVALID_ARG;
    *out = nullptr;
    nn_ctx* ctx;
    int nx, ny, nz;
    const float* invd;
    float invd_c;
    const float* D;
    nn_pcg_info(pc, &ctx, &nx, &ny, &nz, &invd, &invd_c, &D);
    if (nx % 8 || ny % 8 || nz % 8)
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "learned preconditioner: grid sides must be multiples of 8");
    nn_learned* lp = new nn_learned();
    lp->ctx = ctx;
    nn_ctx_retain(ctx);
    lp->pc = pc;
    lp->f = Fine{nx, ny, nz, invd, invd_c};
    lp->G = (int64_t)nx * ny * nz;
    lp->Gc = lp->G / 8;
    nn_status st = nn_unet_make(ctx, nz / 2, ny / 2, nx / 2, seed, &lp->net);
    if (st == NN_OK) st = nn_alloc(ctx, &lp->t, lp->G);
    if (st == NN_OK) st = nn_alloc(ctx, &lp->z1, lp->G);
    if (st == NN_OK) st = nn_alloc(ctx, &lp->rc, lp->Gc);
    if (st == NN_OK) st = nn_alloc(ctx, &lp->ec, lp->Gc);
    if (st == NN_OK) st = nn_alloc(ctx, &lp->r, lp->G);
    if (st == NN_OK) st = nn_alloc(ctx, &lp->z, lp->G);
    if (st == NN_OK) st = nn_alloc(ctx, &lp->p, lp->G);
    if (st == NN_OK) st = nn_alloc(ctx, &lp->q, lp->G);
    if (st == NN_OK) st = nn_alloc(ctx, &lp->dots, 2);
    if (st == NN_OK) st = nn_alloc(ctx, &lp->v, lp->G);
    if (st == NN_OK) st = nn_alloc(ctx, &lp->tv, lp->G);
    if (st == NN_OK) st = nn_alloc(ctx, &lp->step, 2);
    if (st == NN_OK && D) {
        st = nn_alloc(ctx, &lp->logd, lp->Gc);
        if (st == NN_OK) st = launch(ctx, lp->Gc, "k_logd_coarse", k_logd_coarse, lp->f, D, lp->logd);
    }
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "nn_learned_create");
    if (st != NN_OK) {
        nn_learned_destroy(lp);
        return st;
    }
    *out = lp;
    return NN_OK;
}

extern "C" nn_status nn_learned_destroy(nn_learned* lp)
{
    if (!lp) return NN_OK;
    if (lp->ctx) cudaStreamSynchronize(lp->ctx->stream);
    nn_unet_free(lp->net);
    for (float* v : {lp->t, lp->z1, lp->rc, lp->ec, lp->r, lp->z, lp->p, lp->q, lp->logd, lp->v, lp->tv}) cudaFree(v);
    cudaFree(lp->dots);
    cudaFree(lp->step);
    for (float* v : lp->pair_r) cudaFree(v);
    for (float* v : lp->pair_e) cudaFree(v);
    nn_ctx* ctx = lp->ctx;
    delete lp;
    if (ctx) nn_ctx_release(ctx);
    return NN_OK;
}

extern "C" nn_status nn_learned_add_pair(nn_learned* lp, const float* d_r, const float* d_e)
{
    if (!lp || !d_r || !d_e) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = lp->ctx;
    float *rc = nullptr, *ec = nullptr;
    NN_TRY(nn_alloc(ctx, &rc, lp->Gc));
    nn_status st = nn_alloc(ctx, &ec, lp->Gc);
    if (st == NN_OK) st = launch(ctx, lp->G, "k_jacobi", k_jacobi, lp->f, d_r, lp->omega, lp->z1);
    if (st == NN_OK) st = nn_pcg_apply(lp->pc, lp->z1, lp->t);
    if (st == NN_OK) st = launch(ctx, lp->Gc, "k_restrict_diff", k_restrict_diff, lp->f, d_r, (const float*)lp->t, rc);
    if (st == NN_OK) st = launch(ctx, lp->Gc, "k_pair_target", k_pair_target, lp->f, d_e, d_r, lp->omega, ec);
    if (st != NN_OK) {
        nn_release(rc);
        nn_release(ec);
        return st;
    }
    lp->pair_r.push_back(rc);
    lp->pair_e.push_back(ec);
    return NN_OK;
}

extern "C" nn_status nn_learned_train(nn_learned* lp, int steps, float lr, float* mean_loss)
{
    if (!lp || steps < 0 || !(lr > 0.0f)) return NN_ERR_INVALID_ARG;
    if (lp->pair_r.empty()) return nn_fail(lp->ctx, NN_ERR_INVALID_ARG, "nn_learned_train: no training pairs");
    nn_ctx* ctx = lp->ctx;
    nn_unet* u = lp->net;
    NN_CUDA(ctx, cudaMemsetAsync(u->scal + 1, 0, sizeof(double), ctx->stream));
    NN_CUDA(ctx, cudaMemsetAsync(u->err, 0, sizeof(int), ctx->stream));
    for (int it = 0; it < steps; ++it) {
        lp->rng ^= lp->rng << 13;
        lp->rng ^= lp->rng >> 7;
        lp->rng ^= lp->rng << 17;
        const size_t k = (size_t)(lp->rng % lp->pair_r.size());
        NN_TRY(unet_forward(u, lp->pair_r[k], lp->logd));
        NN_TRY(launch(ctx, u->G0, "k_net_loss", k_net_loss, (const float*)u->y32, (const float*)lp->pair_e[k],
                      (const double*)u->scal, (uint4*)u->gOUT, u->g[0], u->scal + 1));
        NN_TRY(unet_backward(u));
        NN_TRY(unet_adam(u, lr));
    }
    NN_TRY(check_err(u));
    double loss = 0.0;
    NN_CUDA(ctx, nn_copy_sync(ctx, &loss, u->scal + 1, sizeof(double), cudaMemcpyDeviceToHost));
    if (mean_loss) *mean_loss = steps ? (float)(loss / ((double)steps * u->G0)) : 0.0f;
    return NN_OK;
}

extern "C" nn_status nn_learned_apply(nn_learned* lp, const float* d_r, float* d_z)
{
    if (!lp || !d_r || !d_z) return NN_ERR_INVALID_ARG;
    NN_CUDA(lp->ctx, cudaMemsetAsync(lp->net->err, 0, sizeof(int), lp->ctx->stream));
    NN_TRY(learned_apply(lp, d_r, d_z));
    return check_err(lp->net);
}

extern "C" nn_status nn_learned_use_network(nn_learned* lp, int enable)
{
    if (!lp) return NN_ERR_INVALID_ARG;
    lp->use_net = enable != 0;
    return NN_OK;
}

// Flexible CG with the learned preconditioner (x holds the initial guess).
extern "C" nn_status nn_learned_solve(nn_learned* lp, const float* d_b, float* d_x, double rtol, int max_iter,
                                      int* iters, double* relres)
{
    if (!lp || !d_b || !d_x || !(rtol > 0.0) || max_iter < 0) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = lp->ctx;
    const int64_t G = lp->G;
    NN_CUDA(ctx, cudaMemsetAsync(lp->net->err, 0, sizeof(int), ctx->stream));
    double bb = 0.0, rr = 0.0, rz = 0.0, pq = 0.0, zq = 0.0;
    NN_TRY(dot(lp, d_b, d_b, &bb));
    NN_TRY(nn_pcg_apply(lp->pc, d_x, lp->q));
    NN_TRY(launch(ctx, G, "k_sub", k_sub, d_b, (const float*)lp->q, lp->r, G));
    NN_TRY(dot(lp, lp->r, lp->r, &rr));
    const double stop = rtol * rtol * bb;
    int it = 0;
    if (rr > stop) {
        NN_TRY(learned_apply(lp, lp->r, lp->z));
        NN_CUDA(ctx, cudaMemcpyAsync(lp->p, lp->z, sizeof(float) * G, cudaMemcpyDeviceToDevice, ctx->stream));
        while (it < max_iter) {
            NN_TRY(nn_pcg_apply(lp->pc, lp->p, lp->q));
            NN_TRY(dot(lp, lp->p, lp->q, &pq));
            NN_TRY(dot(lp, lp->r, lp->z, &rz));
            if (!(pq > 0.0)) break;
            const double a = rz / pq;
            NN_TRY(launch(ctx, G, "k_axpy", k_axpy, (float)a, (const float*)lp->p, d_x, G));
            NN_TRY(launch(ctx, G, "k_axpy", k_axpy, (float)-a, (const float*)lp->q, lp->r, G));
            ++it;
            NN_TRY(dot(lp, lp->r, lp->r, &rr));
            if (rr <= stop || !std::isfinite(rr)) break;
            NN_TRY(learned_apply(lp, lp->r, lp->z));
            NN_TRY(dot(lp, lp->z, lp->q, &zq));
            NN_TRY(launch(ctx, G, "k_xpby", k_xpby, (const float*)lp->z, (float)(-zq / pq), lp->p, G));
        }
    }
    NN_TRY(check_err(lp->net));
    if (iters) *iters = it;
    const double rel = bb > 0.0 ? std::sqrt(rr / bb) : 0.0;
    if (relres) *relres = rel;
    if (!(rr <= stop))
        return nn_fail(ctx, NN_ERR_NOT_CONVERGED, "flexible CG did not reach rtol %g in %d iterations", rtol, max_iter);
    return NN_OK;
}

// Parameters as one flat FP32 vector: per layer w[27][cin][cout] then b[cout].
extern "C" nn_status nn_learned_num_params(nn_learned* lp, int64_t* n)
{
    if (!lp || !n) return NN_ERR_INVALID_ARG;
    int64_t s = 0;
    for (int l = 0; l < NL; ++l) s += lp->net->L[l].nw + LCOUT[l];
    *n = s;
    return NN_OK;
}

extern "C" nn_status nn_learned_get_params(nn_learned* lp, float* h_out)
{
    if (!lp || !h_out) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = lp->ctx;
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int64_t off = 0;
    for (int l = 0; l < NL; ++l) {
        const auto& L = lp->net->L[l];
        NN_CUDA(ctx, nn_copy_sync(ctx, h_out + off, L.w, sizeof(float) * L.nw, cudaMemcpyDeviceToHost));
        off += L.nw;
        NN_CUDA(ctx, nn_copy_sync(ctx, h_out + off, L.b, sizeof(float) * LCOUT[l], cudaMemcpyDeviceToHost));
        off += LCOUT[l];
    }
    return NN_OK;
}

extern "C" nn_status nn_learned_set_params(nn_learned* lp, const float* h_in)
{
    if (!lp || !h_in) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = lp->ctx;
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int64_t off = 0;
    for (int l = 0; l < NL; ++l) {
        auto& L = lp->net->L[l];
        NN_CUDA(ctx, nn_copy_sync(ctx, L.w, h_in + off, sizeof(float) * L.nw, cudaMemcpyHostToDevice));
        off += L.nw;
        NN_CUDA(ctx, nn_copy_sync(ctx, L.b, h_in + off, sizeof(float) * LCOUT[l], cudaMemcpyHostToDevice));
        off += LCOUT[l];
        NN_TRY(unet_repack(lp->net, l));
    }
    return nn_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "nn_learned_set_params");
}

// One forward + backward of the U-Net on a level-0 input and target (both
// dense FP32 on the coarse grid), without an optimiser step: the parameter
// gradients (same flat order as the parameters) go to h_grad, the loss
// 0.5 * sum (y - t / s)^2 to *loss.  For gradient checks.
extern "C" nn_status nn_learned_net_gradient(nn_learned* lp, const float* d_rc, const float* d_target, float* h_grad,
                                             double* loss, float* d_y)
{
    if (!lp || !d_rc || !d_target) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = lp->ctx;
    nn_unet* u = lp->net;
    NN_CUDA(ctx, cudaMemsetAsync(u->err, 0, sizeof(int), ctx->stream));
    for (int l = 0; l < NL; ++l) {
        NN_CUDA(ctx, cudaMemsetAsync(u->L[l].gw, 0, sizeof(float) * u->L[l].nw, ctx->stream));
        NN_CUDA(ctx, cudaMemsetAsync(u->L[l].gb, 0, sizeof(float) * LCOUT[l], ctx->stream));
    }
    NN_TRY(unet_forward(u, d_rc, lp->logd));
    NN_CUDA(ctx, cudaMemsetAsync(u->scal + 1, 0, sizeof(double), ctx->stream));
    NN_TRY(launch(ctx, u->G0, "k_net_loss", k_net_loss, (const float*)u->y32, d_target, (const double*)u->scal,
                  (uint4*)u->gOUT, u->g[0], u->scal + 1));
    NN_TRY(unet_backward(u));
    NN_TRY(check_err(u));
    if (d_y) NN_CUDA(ctx, nn_copy_sync(ctx, d_y, u->y32, sizeof(float) * u->G0, cudaMemcpyDeviceToDevice));
    double l2 = 0.0;
    NN_CUDA(ctx, nn_copy_sync(ctx, &l2, u->scal + 1, sizeof(double), cudaMemcpyDeviceToHost));
    if (loss) *loss = 0.5 * l2;
    if (h_grad) {
        int64_t off = 0;
        for (int l = 0; l < NL; ++l) {
            const auto& L = u->L[l];
            NN_CUDA(ctx, nn_copy_sync(ctx, h_grad + off, L.gw, sizeof(float) * L.nw, cudaMemcpyDeviceToHost));
            off += L.nw;
            NN_CUDA(ctx, nn_copy_sync(ctx, h_grad + off, L.gb, sizeof(float) * LCOUT[l], cudaMemcpyDeviceToHost));
            off += LCOUT[l];
        }
    }
    return NN_OK;
}

// ------------------------------------------ learned coarse-level solver --

namespace {
// out = b / d (the Jacobi-scaled right-hand side, whose solution has the
// scale of the input)
__global__ void k_div(const float* b, const float* d, float* out, int64_t n)
{
    GRID_LOOP(i, n) out[i] = b[i] / d[i];
}
}  // namespace
//
// A multigrid hierarchy (nn_mg, all levels) in which the treatment of one
// coarse level -- its pre-smoothing and every level below it -- is replaced
// by the U-Net: x_L = s N(D^-1 b_L / s, f), s = rms(D^-1 b_L), D the level's
// diagonal, f = log D minus its mean, followed by the V-cycle's
// post-smoothing on that level.  (D^-1 b has the scale of the solution; b
// itself is thousands of times larger on a coarse level.)  Training pairs: the right-hand sides that reach that level while
// the classical hierarchy solves given systems, and their solutions on that
// level (Jacobi-PCG to 1e-7).  Without the network (use_network = 0) the
// hierarchy is the classical one.

struct nn_lmg {
    nn_ctx* ctx = nullptr;
    nn_pcg* pc = nullptr;
    nn_mg* mg = nullptr;
    nn_unet* net = nullptr;
    int level = 0, nx = 0, ny = 0, nz = 0;
    int64_t Gc = 0, G = 0;  // cells of the network's level and of the fine grid
    float* feat = nullptr;
    const float* diag = nullptr;  // the level's diagonal (owned by the hierarchy)
    float* bs = nullptr;          // D^-1 b of the level solve
    std::vector<float*> pair_b, pair_e, rec;
    size_t max_pairs = 4096;
    uint64_t rng = 0x2545F4914F6CDD1Dull;
    int use_net = 1;
};

static nn_status lmg_level_solve(void* user, const float* b, float* x)
{
    nn_lmg* lm = static_cast<nn_lmg*>(user);
    // x = s N(D^-1 b / s, f): the division, the rms and the final scaling run
    // inside the network's first and last kernels
    return unet_forward(lm->net, b, lm->feat, lm->diag, x);
}

static nn_status lmg_record(void* user, const float* b)
{
    nn_lmg* lm = static_cast<nn_lmg*>(user);
    if (lm->pair_b.size() + lm->rec.size() >= lm->max_pairs) return NN_OK;
    float* v = nullptr;
    NN_TRY(nn_alloc(lm->ctx, &v, (size_t)lm->Gc));
    lm->rec.push_back(v);
    NN_CUDA(lm->ctx, cudaMemcpyAsync(v, b, sizeof(float) * lm->Gc, cudaMemcpyDeviceToDevice, lm->ctx->stream));
    return NN_OK;
}

// training input of a recorded right-hand side: D^-1 b (in place)
static nn_status lmg_scale_input(nn_lmg* lm, float* b)
{
    return launch(lm->ctx, lm->Gc, "k_div", k_div, (const float*)b, lm->diag, b, lm->Gc);
}

static nn_status lmg_apply_mode(nn_lmg* lm)
{
    return nn_mg_set_level_solver(lm->mg, lm->level, lm->use_net ? lmg_level_solve : nullptr, lm);
}

extern "C" nn_status nn_lmg_destroy(nn_lmg* lm)
{
    if (!lm) return NN_OK;
    if (lm->ctx) cudaStreamSynchronize(lm->ctx->stream);
    if (lm->mg) nn_mg_destroy(lm->mg);
    nn_unet_free(lm->net);
    cudaFree(lm->feat);
    cudaFree(lm->bs);
    for (float* v : lm->pair_b) cudaFree(v);
    for (float* v : lm->pair_e) cudaFree(v);
    for (float* v : lm->rec) cudaFree(v);
    nn_ctx* ctx = lm->ctx;
    delete lm;
    if (ctx) nn_ctx_release(ctx);
    return NN_OK;
}

extern "C" nn_status nn_lmg_create(nn_pcg* pc, int level, uint64_t seed, nn_lmg** out)
{
    if (!pc || !out || level < 1) return NN_ERR_INVALID_ARG;
    *out = nullptr;
    nn_ctx* ctx;
    int fx, fy, fz;
    const float* invd;
    float invd_c;
    const float* D;
    nn_pcg_info(pc, &ctx, &fx, &fy, &fz, &invd, &invd_c, &D);
    nn_lmg* lm = new nn_lmg();
    lm->ctx = ctx;
    nn_ctx_retain(ctx);
    lm->pc = pc;
    lm->level = level;
    lm->G = (int64_t)fx * fy * fz;
    nn_status st = nn_mg_create(pc, 0, &lm->mg);
    const float* diag = nullptr;
    if (st == NN_OK) st = nn_mg_level_dims(lm->mg, level, &lm->nx, &lm->ny, &lm->nz, &diag);
    if (st == NN_OK && (lm->nx % 4 || lm->ny % 4 || lm->nz % 4))
        st = nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_lmg_create: level %d is %dx%dx%d; the network needs sides that are "
                     "multiples of 4", level, lm->nx, lm->ny, lm->nz);
    if (st == NN_OK) {
        lm->Gc = (int64_t)lm->nx * lm->ny * lm->nz;
        st = nn_unet_make(ctx, lm->nz, lm->ny, lm->nx, seed, &lm->net);
    }
    if (st == NN_OK) st = nn_alloc(ctx, &lm->feat, (size_t)lm->Gc);
    if (st == NN_OK) st = nn_alloc(ctx, &lm->bs, (size_t)lm->Gc);
    lm->diag = diag;
    if (st == NN_OK) {
        // feature channel: log diag - mean
        std::vector<float> h((size_t)lm->Gc);
        st = nn_cuda_check(ctx, nn_copy_sync(ctx, h.data(), diag, sizeof(float) * h.size(), cudaMemcpyDeviceToHost),
                           "nn_lmg_create");
        if (st == NN_OK) {
            double mean = 0.0;
            for (float& v : h) {
                v = std::log(std::max(v, 1e-30f));
                mean += v;
            }
            mean /= (double)h.size();
            for (float& v : h) v = (float)(v - mean);
            st = nn_cuda_check(ctx, nn_copy_sync(ctx, lm->feat, h.data(), sizeof(float) * h.size(),
                                                 cudaMemcpyHostToDevice), "nn_lmg_create");
        }
    }
    // one forward pass on zeros, so that every kernel's attributes are set
    // before a solve may capture the network into a graph
    if (st == NN_OK) st = nn_cuda_check(ctx, nn_zero_async(ctx, lm->net->y32, sizeof(float) * lm->Gc), "nn_lmg_create");
    if (st == NN_OK) st = unet_forward(lm->net, lm->net->y32, lm->feat);
    if (st == NN_OK) st = check_err(lm->net);
    if (st == NN_OK) st = lmg_apply_mode(lm);
    if (st != NN_OK) {
        nn_lmg_destroy(lm);
        return st;
    }
    *out = lm;
    return NN_OK;
}

// Solve A x = b with the classical hierarchy from x = 0, record the
// right-hand sides that reach the network's level, and store each with its
// solution on that level as a training pair.
extern "C" nn_status nn_lmg_add_solve(nn_lmg* lm, const float* d_b, float* d_x, int* pairs_added)
{
    if (!lm || !d_b || !d_x) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = lm->ctx;
    NN_TRY(nn_mg_set_level_solver(lm->mg, lm->level, nullptr, nullptr));
    NN_TRY(nn_mg_set_recorder(lm->mg, lm->level, lmg_record, lm));
    NN_CUDA(ctx, nn_zero_async(ctx, d_x, sizeof(float) * lm->G));
    int it = 0;
    double rel = 0.0;
    nn_status st = nn_mg_solve(lm->mg, d_b, d_x, 1e-6, 500, &it, &rel);
    nn_mg_set_recorder(lm->mg, lm->level, nullptr, nullptr);
    int added = 0;
    for (float* b : lm->rec) {
        float* e = nullptr;
        if (st == NN_OK) st = nn_alloc(ctx, &e, (size_t)lm->Gc);
        if (st == NN_OK) st = nn_mg_level_cg(lm->mg, lm->level, b, e, 1e-7, 5000, nullptr);
        if (st == NN_OK) st = lmg_scale_input(lm, b);
        if (st == NN_OK) {
            lm->pair_b.push_back(b);
            lm->pair_e.push_back(e);
            ++added;
        } else {
            cudaFree(b);
            cudaFree(e);
        }
    }
    lm->rec.clear();
    const nn_status st2 = lmg_apply_mode(lm);
    if (pairs_added) *pairs_added = added;
    return st != NN_OK ? st : st2;
}

extern "C" nn_status nn_lmg_train(nn_lmg* lm, int steps, float lr, float* mean_loss)
{
    if (!lm || steps < 0 || !(lr > 0.0f)) return NN_ERR_INVALID_ARG;
    if (lm->pair_b.empty()) return nn_fail(lm->ctx, NN_ERR_INVALID_ARG, "nn_lmg_train: no training pairs");
    nn_ctx* ctx = lm->ctx;
    nn_unet* u = lm->net;
    NN_CUDA(ctx, cudaMemsetAsync(u->scal + 1, 0, sizeof(double), ctx->stream));
    NN_CUDA(ctx, cudaMemsetAsync(u->err, 0, sizeof(int), ctx->stream));
    for (int it = 0; it < steps; ++it) {
        lm->rng ^= lm->rng << 13;
        lm->rng ^= lm->rng >> 7;
        lm->rng ^= lm->rng << 17;
        const size_t k = (size_t)(lm->rng % lm->pair_b.size());
        NN_TRY(unet_forward(u, lm->pair_b[k], lm->feat));
        NN_TRY(launch(ctx, u->G0, "k_net_loss", k_net_loss, (const float*)u->y32, (const float*)lm->pair_e[k],
                      (const double*)u->scal, (uint4*)u->gOUT, u->g[0], u->scal + 1));
        NN_TRY(unet_backward(u));
        NN_TRY(unet_adam(u, lr));
    }
    NN_TRY(check_err(u));
    double loss = 0.0;
    NN_CUDA(ctx, nn_copy_sync(ctx, &loss, u->scal + 1, sizeof(double), cudaMemcpyDeviceToHost));
    if (mean_loss) *mean_loss = steps ? (float)(loss / ((double)steps * u->G0)) : 0.0f;
    // the weights changed: the solver's captured graph holds the repacked
    // buffers by address, which stay the same, so it remains valid
    return NN_OK;
}

extern "C" nn_status nn_lmg_use_network(nn_lmg* lm, int enable)
{
    if (!lm) return NN_ERR_INVALID_ARG;
    lm->use_net = enable != 0;
    return lmg_apply_mode(lm);
}

extern "C" nn_status nn_lmg_set_post_sweeps(nn_lmg* lm, int sweeps)
{
    if (!lm) return NN_ERR_INVALID_ARG;
    return nn_mg_set_level_sweeps(lm->mg, sweeps);
}

extern "C" nn_status nn_lmg_pairs(nn_lmg* lm, int* n)
{
    if (!lm || !n) return NN_ERR_INVALID_ARG;
    *n = (int)lm->pair_b.size();
    return NN_OK;
}

extern "C" nn_status nn_lmg_solve(nn_lmg* lm, const float* d_b, float* d_x, double rtol, int max_iter, int* iters,
                                  double* relres)
{
    if (!lm) return NN_ERR_INVALID_ARG;
    NN_CUDA(lm->ctx, cudaMemsetAsync(lm->net->err, 0, sizeof(int), lm->ctx->stream));
    const nn_status st = nn_mg_solve(lm->mg, d_b, d_x, rtol, max_iter, iters, relres);
    const nn_status st2 = check_err(lm->net);
    return st != NN_OK ? st : st2;
}

// The number of Jacobi sweeps after the network's correction, chosen by time:
// each candidate solves the nb right-hand sides d_bs[k] from zero (d_x:
// scratch) to rtol, once to warm (graph capture) and once timed; the smallest
// total time is kept.
extern "C" nn_status nn_lmg_autotune_post_sweeps(nn_lmg* lm, const float* const* d_bs, int nb, float* d_x, double rtol,
                                                 int* best, float* best_ms)
{
    if (!lm || !d_bs || nb < 1 || !d_x) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = lm->ctx;
    cudaStream_t cs = ctx->stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    NN_CUDA(ctx, cudaEventCreate(&e0));
    NN_CUDA(ctx, cudaEventCreate(&e1));
    int bsw = 2;
    float bms = 1e30f;
    nn_status st = NN_OK;
    for (int sw : {2, 4, 8, 12, 16, 20, 24}) {
        if (st != NN_OK) break;
        st = nn_mg_set_level_sweeps(lm->mg, sw);
        int it = 0;
        double rel = 0.0;
        float ms = 0.0f;
        for (int k = 0; k < nb && st == NN_OK; ++k)
            for (int rep = 0; rep < 2 && st == NN_OK; ++rep) {
                st = nn_cuda_check(ctx, cudaMemsetAsync(d_x, 0, sizeof(float) * (size_t)lm->G, cs), "memset");
                if (st == NN_OK && rep == 1) st = nn_cuda_check(ctx, cudaEventRecord(e0, cs), "event");
                if (st == NN_OK) st = nn_lmg_solve(lm, d_bs[k], d_x, rtol, 1000, &it, &rel);
                if (st == NN_OK && rep == 1) st = nn_cuda_check(ctx, cudaEventRecord(e1, cs), "event");
                float m = 0.0f;
                if (st == NN_OK && rep == 1) st = nn_cuda_check(ctx, cudaEventSynchronize(e1), "event");
                if (st == NN_OK && rep == 1) st = nn_cuda_check(ctx, cudaEventElapsedTime(&m, e0, e1), "event");
                ms += m;
            }
        if (st == NN_OK && ms < bms) {
            bms = ms;
            bsw = sw;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const nn_status st2 = nn_mg_set_level_sweeps(lm->mg, bsw);
    if (best) *best = bsw;
    if (best_ms) *best_ms = bms < 1e30f ? bms : 0.0f;
    return st != NN_OK ? st : st2;
}
