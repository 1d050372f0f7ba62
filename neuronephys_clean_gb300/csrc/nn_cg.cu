// Single-kernel-per-iteration preconditioned CG (Chronopoulos & Gear, "s-step
// iterative methods for symmetric linear systems", J. Comput. Appl. Math. 25,
// 1989) for the constant-coefficient 7-point backward-Euler operator
//   A = (1 + beta) I + alpha L_D,  (L_D v)_c = sum over the 6 faces f of
//   c_f (v_c - v_nb), zero values outside the grid (homogeneous Dirichlet),
// Jacobi preconditioner M = 1/diag.  With constant coefficients every c_f = 1;
// with a cell field D (the HET variant) c_f is the harmonic mean of D on the
// two sides of the face, D_c on a boundary face.
//
// The recurrences need one grid-wide reduction per iteration:
//   p_i = u_i + b_i p_{i-1}        s_i = w_i + b_i s_{i-1}      (s = A p)
//   x  += a_i p_i                  r  -= a_i s_i
//   u   = M r                      w   = A u
//   g = (r, u), d = (w, u), rho = (r, r)   -> one reduction
//   b_{i+1} = g / g_old,  a_{i+1} = g / (d - b_{i+1} g / a_i)
// One kernel does all of it: a block owns a 32 x 16 x zc tile (each thread two
// rows, iy and iy + 8) and marches in z; planes of r, w and s (with a one-cell
// halo, the TMA box starting 16-byte
// aligned at x0 - 4) are staged into shared memory by cp.async.bulk.tensor
// through a 4-deep mbarrier pipeline; out-of-range boxes are zero-filled by
// the TMA unit, which is exactly the Dirichlet boundary.  u = M r_new is formed
// for the tile plus halo in a 3-plane ring, w = A u for the plane behind it.
// The HET variant also stages D and 1/diag with the same halo and keeps D in
// a 3-plane ring beside u for the face coefficients (48 instead of 40 bytes
// of DRAM traffic per cell and iteration).
// r, w and s are double-buffered (the next iteration reads the halo of cells
// other blocks write); p and x are updated in place.  The last block to finish
// sums the block partials in FP64 and forms the next iteration's scalars, so
// no host round trip separates iterations.  Every mbarrier wait is bounded.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <type_traits>

#include "nn_internal.cuh"
#include "nn_ptx.cuh"

namespace {
constexpr int CG_THREADS = 256;
constexpr int TX = 32, TY = 16;            // tile; its depth in z (zc) is chosen per plan
constexpr int HY = TY / 2;                   // a thread's second row is 8 below its first
constexpr int BXW = 40, BYW = TY + 2;        // TMA box: x from x0 - 4, y from y0 - 1
constexpr int RX = TX + 2, RY = TY + 2;      // u region (tile + halo)
constexpr int PLANE_BYTES = BXW * BYW * 4;   // 2880
constexpr int PLANE_STRIDE = 2944;           // 128-byte multiple
static_assert(CG_THREADS == TX * HY && PLANE_STRIDE >= PLANE_BYTES && PLANE_STRIDE % 128 == 0, "tile shape");
constexpr int PX_BYTES = TX * TY * 4;        // p, x interior boxes (owned planes only)
constexpr int STAGES = 3;
constexpr int RING = 3;                      // u-ring slots: planes k-2 .. k
constexpr int U_BYTES = RING * RY * RX * 4;  // one ring over the u region

template <bool HET>
struct Layout {
    static constexpr int NARR = HET ? 5 : 3;  // r, w, s (+ D, 1/diag), with halo
    static constexpr int STAGE_BYTES = NARR * PLANE_STRIDE + 2 * PX_BYTES;
    static constexpr int RING_BYTES = (HET ? 2 : 1) * U_BYTES;  // u (+ D)
    static constexpr int SMEM_BYTES = 128 + STAGES * STAGE_BYTES + RING_BYTES + STAGES * 8 + 64;
};
static_assert(Layout<true>::SMEM_BYTES <= 227 * 1024, "shared memory");
constexpr uint32_t WAIT_LIMIT = 1u << 20;
constexpr int HALO_CELLS = 2 * RX + 2 * TY;  // 100

enum { C_GAMMA = 0, C_ALPHA, C_BETA, C_RR, C_BB, C_DELTA, C_COUNT };

struct CgArgs {
    int nx, ny, nz;
    int zc;                       // tile depth in z
    float op_alpha, onepb, invd;  // invd: 1/diag for constant coefficients
    const float* D;               // HET: cell field
    const float* invdv;           // HET: 1/diag per cell
    float* p;
    float* x;
    float* r_out;
    float* w_out;
    float* s_out;
    double* scal;
    double* partials;
    unsigned int* ticket;
    int* flags;  // [0] stop (1 converged, 2 max_iter, 3 error) [1] iterations [2] wait timeout
    double rtol2;
    int max_iter;
};

// Bounded mbarrier wait of this kernel (nn_ptx.cuh), WAIT_LIMIT polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase) { return nn_mbar_wait(bar, phase, WAIT_LIMIT); }

// Abort path: wait (bounded) for the copies of planes first .. last to land.
__device__ __noinline__ void drain_planes(uint64_t* bars, int first, int last, int stages)
{
    for (int q = first; q <= last; ++q) mbar_wait(&bars[q % stages], (uint32_t)((q / stages) & 1));
}

__device__ __forceinline__ void tma_load_plane(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar)
{
    nn_tma_load_3d(dst, map, x, y, z, bar);
}

__device__ __forceinline__ float warp_sumf(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block partials of nsum values (FP32 per thread and warp, FP64 across warps
// and blocks); the last block to arrive writes the grid totals to out[].
__device__ bool cg_reduce(int nsum, const float* v, double* partials, unsigned int* ticket, double* out)
{
    __shared__ double ws[3][CG_THREADS / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = 0; q < nsum; ++q) {
        const float s = warp_sumf(v[q]);
        if (lane == 0) ws[q][w] = (double)s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 0; q < nsum; ++q) {
            double s = 0.0;
            for (int u = 0; u < CG_THREADS / 32; ++u) s += ws[q][u];
            partials[(size_t)q * gridDim.x + blockIdx.x] = s;
        }
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    for (int q = 0; q < nsum; ++q) {
        const volatile double* pp = partials + (size_t)q * gridDim.x;
        double s = 0.0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += CG_THREADS) s += pp[b];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        __syncthreads();
        if (lane == 0) ws[q][w] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int u = 0; u < CG_THREADS / 32; ++u) t += ws[q][u];
            out[q] = t;
        }
    }
    if (threadIdx.x == 0) *ticket = 0;
    __syncthreads();
    return true;
}

__device__ __forceinline__ float face_coef(float dc, float dn, bool inside)
{
    return inside ? __fdividef(2.0f * dc * dn, dc + dn) : dc;
}

// (A v)_c with v read through v(index) (zero outside the grid).
template <bool HET, class V>
__device__ __forceinline__ float apply_A(const CgArgs& a, int64_t c, int i, int j, int k, V v)
{
    const int64_t sy = a.nx, sz = (int64_t)a.nx * a.ny;
    const bool in[6] = {i > 0, i < a.nx - 1, j > 0, j < a.ny - 1, k > 0, k < a.nz - 1};
    const int64_t off[6] = {-1, 1, -sy, sy, -sz, sz};
    const float vc = v(c);
    if (!HET) {
        float nb = 0.0f;
#pragma unroll
        for (int f = 0; f < 6; ++f) nb += in[f] ? v(c + off[f]) : 0.0f;
        return (a.onepb + 6.0f * a.op_alpha) * vc - a.op_alpha * nb;
    }
    const float dc = a.D[c];
    float acc = 0.0f;
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        const float cf = face_coef(dc, in[f] ? a.D[c + off[f]] : 0.0f, in[f]);
        acc += cf * (vc - (in[f] ? v(c + off[f]) : 0.0f));
    }
    return a.onepb * vc + a.op_alpha * acc;
}

// r0 = b - A x0 (neighbour loads; once per solve); bb = (b, b)
template <bool HET>
__global__ void __launch_bounds__(CG_THREADS) k_cg_init_r(CgArgs a, const float* b, const float* x, float* r)
{
    const int64_t sz = (int64_t)a.nx * a.ny, G = sz * a.nz;
    float bb = 0.0f;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < G; c += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % a.nx), j = (int)((c / a.nx) % a.ny), k = (int)(c / sz);
        const float ax = apply_A<HET>(a, c, i, j, k, [&](int64_t q) { return x[q]; });
        const float bv = b[c];
        r[c] = bv - ax;
        bb += bv * bv;
    }
    float v[1] = {bb};
    double out[1];
    if (cg_reduce(1, v, a.partials, a.ticket, out) && threadIdx.x == 0) a.scal[C_BB] = out[0];
}

// w0 = A (M r0), p = 0, s = 0; g0, d0, rho0 -> a0, b0 = 0
template <bool HET>
__global__ void __launch_bounds__(CG_THREADS) k_cg_init_w(CgArgs a, const float* r, float* w, float* s)
{
    const int64_t sz = (int64_t)a.nx * a.ny, G = sz * a.nz;
    float g = 0.0f, d = 0.0f, rr = 0.0f;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < G; c += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % a.nx), j = (int)((c / a.nx) % a.ny), k = (int)(c / sz);
        const float rc = r[c];
        float uc, wc;
        if (HET) {
            uc = a.invdv[c] * rc;
            wc = apply_A<true>(a, c, i, j, k, [&](int64_t q) { return a.invdv[q] * r[q]; });
        } else {
            uc = a.invd * rc;
            wc = a.invd * apply_A<false>(a, c, i, j, k, [&](int64_t q) { return r[q]; });
        }
        w[c] = wc;
        s[c] = 0.0f;
        a.p[c] = 0.0f;
        g += rc * uc;
        d += wc * uc;
        rr += rc * rc;
    }
    float v[3] = {g, d, rr};
    double out[3];
    if (cg_reduce(3, v, a.partials, a.ticket, out) && threadIdx.x == 0) {
        a.scal[C_GAMMA] = out[0];
        a.scal[C_DELTA] = out[1];
        a.scal[C_RR] = out[2];
        a.scal[C_ALPHA] = out[1] != 0.0 ? out[0] / out[1] : 0.0;
        a.scal[C_BETA] = 0.0;
        a.flags[1] = 0;
        a.flags[2] = 0;
        a.flags[0] = (out[2] <= a.rtol2 * a.scal[C_BB]) ? 1 : 0;
    }
}

__device__ void cg_finish(const CgArgs& a, float acc_g, float acc_d, float acc_r);

// One CG iteration (see the file comment).  One tile per block.  tm_d and
// tm_m (D and 1/diag) are read only by the HET variant.
template <bool HET>
__global__ void __launch_bounds__(CG_THREADS, 4) k_cg_iter(const __grid_constant__ CUtensorMap tm_r,
                                                        const __grid_constant__ CUtensorMap tm_w,
                                                        const __grid_constant__ CUtensorMap tm_s,
                                                        const __grid_constant__ CUtensorMap tm_d,
                                                        const __grid_constant__ CUtensorMap tm_m,
                                                        const __grid_constant__ CUtensorMap tm_p,
                                                        const __grid_constant__ CUtensorMap tm_x, CgArgs a)
{
    using L = Layout<HET>;
    constexpr int STAGE_BYTES = L::STAGE_BYTES;
    constexpr int PX_OFF = L::NARR * PLANE_STRIDE;  // p, x boxes after the halo planes
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
    unsigned char* stage_base = smem;
    float* U = (float*)(smem + STAGES * STAGE_BYTES);  // [RING][RY][RX]
    float* Dr = U + RING * RY * RX;                     // HET: D ring [RING][RY][RX]
    uint64_t* bars = (uint64_t*)(smem + STAGES * STAGE_BYTES + L::RING_BYTES);
    __shared__ int abort_flag;

    const int tid = threadIdx.x;
    const int tiles_x = (a.nx + TX - 1) / TX, tiles_y = (a.ny + TY - 1) / TY;
    const int tx = blockIdx.x % tiles_x;
    const int ty = (blockIdx.x / tiles_x) % tiles_y;
    const int tz = blockIdx.x / (tiles_x * tiles_y);
    const int x0 = tx * TX, y0 = ty * TY, z0 = tz * a.zc;
    const int z1 = min(z0 + a.zc, a.nz);
    const int np = z1 - z0 + 2;  // planes z0-1 .. z1
    const int sy = a.nx, sz = a.nx * a.ny;  // grids below 2^31 cells (plan check)

    if (tid == 0) {
        abort_flag = 0;
        for (int q = 0; q < STAGES; ++q) nn_mbar_init(&bars[q], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // launched as a programmatic dependent of the previous iteration (in a
    // synchronous solve): its scalars, flags and vectors are complete only now
    nn_grid_dep_wait();
    if (a.flags[0]) return;
    const float alpha = (float)a.scal[C_ALPHA], beta = (float)a.scal[C_BETA];
    // plane j (z = z0 - 1 + j) into stage j % STAGES: r, w, s with halo, and
    // for owned planes p, x of the tile
    auto issue = [&](int j) {
        unsigned char* st = stage_base + (j % STAGES) * STAGE_BYTES;
        uint64_t* bar = &bars[j % STAGES];
        const int kz = z0 - 1 + j;
        const bool own = j >= 1 && j <= np - 2;
        nn_mbar_expect_tx(bar, L::NARR * PLANE_BYTES + (own ? 2 * PX_BYTES : 0));
        tma_load_plane(st, &tm_r, x0 - 4, y0 - 1, kz, bar);
        tma_load_plane(st + PLANE_STRIDE, &tm_w, x0 - 4, y0 - 1, kz, bar);
        tma_load_plane(st + 2 * PLANE_STRIDE, &tm_s, x0 - 4, y0 - 1, kz, bar);
        if (HET) {
            tma_load_plane(st + 3 * PLANE_STRIDE, &tm_d, x0 - 4, y0 - 1, kz, bar);
            tma_load_plane(st + 4 * PLANE_STRIDE, &tm_m, x0 - 4, y0 - 1, kz, bar);
        }
        if (own) {
            tma_load_plane(st + PX_OFF, &tm_p, x0, y0, kz, bar);
            tma_load_plane(st + PX_OFF + PX_BYTES, &tm_x, x0, y0, kz, bar);
        }
    };
    if (tid == 0)
        for (int j = 0; j < STAGES && j < np; ++j) issue(j);

    // per-thread invariants: interior cells (rows iy and iy + HY), their
    // offsets in a staged plane, in the u region and in a p/x box, the global
    // index of the first without z; the halo cell this thread fills
    // (tid < HALO_CELLS)
    const int ix = tid & 31, iy = tid >> 5;
    const int gx = x0 + ix, gy = y0 + iy;
    const bool col_in[2] = {gx < a.nx && gy < a.ny, gx < a.nx && gy + HY < a.ny};
    const int ib = (iy + 1) * BXW + ix + 4;
    const int iu = (iy + 1) * RX + ix + 1;
    const int ip = iy * TX + ix;
    const int cxy = gx + sy * gy;
    int hb = 0, hu = 0;
    bool hcol = false;
    if (tid < HALO_CELLS) {
        int bx, by;
        if (tid < RX) { bx = 3 + tid; by = 0; }
        else if (tid < 2 * RX) { bx = 3 + tid - RX; by = RY - 1; }
        else if (tid < 2 * RX + TY) { bx = 3; by = 1 + tid - 2 * RX; }
        else { bx = 3 + RX - 1; by = 1 + tid - 2 * RX - TY; }
        const int hx = x0 - 4 + bx, hy = y0 - 1 + by;
        hcol = hx >= 0 && hx < a.nx && hy >= 0 && hy < a.ny;
        hb = by * BXW + bx;
        hu = by * RX + bx - 3;
    }
    float acc_g = 0.0f, acc_r = 0.0f, acc_d = 0.0f;

    // One plane j; SL = j % 3 names both its stage buffer and its u-ring slot,
    // so every shared-memory offset below is a compile-time constant.
    auto plane = [&](auto sl_c, int j) -> bool {
        constexpr int SL = decltype(sl_c)::value;
        constexpr int SM = (SL + 1) % RING, SC = (SL + 2) % RING;  // ring slots of planes k - 2 and k - 1
        const int k = z0 - 1 + j;
        // one thread polls the barrier (spinning threads would take issue
        // slots from the working warps); the block barrier then publishes the
        // landed plane to everyone and orders the previous plane's w-phase
        // before this plane's writes to the u ring
        if (tid == 0 && !mbar_wait(&bars[SL], (uint32_t)((j / STAGES) & 1))) {
            // let the copies still in flight (planes j .. j + STAGES - 1) land
            // before the block leaves
            drain_planes(bars, j, min(np - 1, j + STAGES - 1), STAGES);
            abort_flag = 1;
        }
        __syncthreads();
        if (abort_flag) return false;
        const unsigned char* st = stage_base + SL * STAGE_BYTES;
        const float* R = (const float*)st;
        const float* W = (const float*)(st + PLANE_STRIDE);
        const float* S = (const float*)(st + 2 * PLANE_STRIDE);
        const float* Dst = (const float*)(st + 3 * PLANE_STRIDE);
        const float* Mst = (const float*)(st + 4 * PLANE_STRIDE);
        const float* Ps = (const float*)(st + PX_OFF);
        const float* Xs = (const float*)(st + PX_OFF + PX_BYTES);
        float* Uk = U + SL * RY * RX;
        float* Dk = Dr + SL * RY * RX;
        const bool plane_in = k >= 0 && k < a.nz;
        // interior cells: s, r, u and the pointwise p, x updates for owned planes
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int bh = ib + h * HY * BXW, uh = iu + h * HY * RX, ph = ip + h * HY * TX;
            const float sv = W[bh] + beta * S[bh];
            const float rv_old = R[bh];
            const float rv = rv_old - alpha * sv;
            const bool in = col_in[h] && plane_in;
            const float mi = HET ? Mst[bh] : a.invd;
            const float uv = in ? mi * rv : 0.0f;
            Uk[uh] = uv;
            if (HET) Dk[uh] = Dst[bh];
            if (in && k >= z0 && k < z1) {
                const int c = cxy + h * HY * sy + sz * k;
                const float pv = mi * rv_old + beta * Ps[ph];
                a.p[c] = pv;
                a.x[c] = Xs[ph] + alpha * pv;
                a.s_out[c] = sv;
                a.r_out[c] = rv;
                acc_g += rv * uv;
                acc_r += rv * rv;
            }
        }
        // halo ring of the u region
        if (tid < HALO_CELLS) {
            const float hsv = W[hb] + beta * S[hb];
            const float hrv = R[hb] - alpha * hsv;
            const float hmi = HET ? Mst[hb] : a.invd;
            Uk[hu] = (hcol && plane_in) ? hmi * hrv : 0.0f;
            if (HET) Dk[hu] = Dst[hb];
        }
        __syncthreads();
        // refill this stage with the plane STAGES ahead
        if (tid == 0 && j + STAGES < np) issue(j + STAGES);
        // w = A u for the plane behind (k - 1), owned when j >= 2
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (!(j >= 2 && col_in[h] && k - 1 < z1)) continue;
            const int kb = k - 1;
            const int uh = iu + h * HY * RX;
            const float* Um = U + SM * RY * RX;
            const float* Uc = U + SC * RY * RX;
            const float uc = Uc[uh];
            float wv;
            if (HET) {
                const float* Dm = Dr + SM * RY * RX;
                const float* Dc = Dr + SC * RY * RX;
                const int gyh = gy + h * HY;
                const float dc = Dc[uh];
                float acc = face_coef(dc, Dc[uh - 1], gx > 0) * (uc - Uc[uh - 1]);
                acc += face_coef(dc, Dc[uh + 1], gx < a.nx - 1) * (uc - Uc[uh + 1]);
                acc += face_coef(dc, Dc[uh - RX], gyh > 0) * (uc - Uc[uh - RX]);
                acc += face_coef(dc, Dc[uh + RX], gyh < a.ny - 1) * (uc - Uc[uh + RX]);
                acc += face_coef(dc, Dm[uh], kb > 0) * (uc - Um[uh]);
                acc += face_coef(dc, Dk[uh], kb < a.nz - 1) * (uc - Uk[uh]);
                wv = a.onepb * uc + a.op_alpha * acc;
            } else {
                const float nb = Uc[uh - 1] + Uc[uh + 1] + Uc[uh - RX] + Uc[uh + RX] + Um[uh] + Uk[uh];
                wv = (a.onepb + 6.0f * a.op_alpha) * uc - a.op_alpha * nb;
            }
            a.w_out[cxy + h * HY * sy + sz * kb] = wv;
            acc_d += wv * uc;
        }
        return true;
    };
    static_assert(STAGES == 3 && RING == 3, "the plane loop is unrolled by the 3 stages / 3 ring slots");
    for (int j = 0; j < np; j += 3) {
        if (!plane(std::integral_constant<int, 0>{}, j)) break;
        if (j + 1 < np && !plane(std::integral_constant<int, 1>{}, j + 1)) break;
        if (j + 2 < np && !plane(std::integral_constant<int, 2>{}, j + 2)) break;
    }
    if (abort_flag) {
        if (tid == 0) {
            a.flags[2] = 1;
            a.flags[0] = 3;
        }
        return;
    }
    cg_finish(a, acc_g, acc_d, acc_r);
}

// The iteration's reduction of (r, u), (w, u), (r, r) and, in the last block
// to arrive, the next iteration's scalars and the stop flag.
__device__ void cg_finish(const CgArgs& a, float acc_g, float acc_d, float acc_r)
{
    float v[3] = {acc_g, acc_d, acc_r};
    double out[3];
    if (cg_reduce(3, v, a.partials, a.ticket, out) && threadIdx.x == 0) {
        const double g = out[0], d = out[1], rr = out[2];
        const int it = a.flags[1] + 1;
        a.flags[1] = it;
        a.scal[C_RR] = rr;
        const double bnew = g / a.scal[C_GAMMA];
        const double denom = d - bnew * g / a.scal[C_ALPHA];
        a.scal[C_BETA] = bnew;
        a.scal[C_ALPHA] = denom != 0.0 ? g / denom : 0.0;
        a.scal[C_GAMMA] = g;
        a.scal[C_DELTA] = d;
        if (rr <= a.rtol2 * a.scal[C_BB]) a.flags[0] = 1;
        else if (it >= a.max_iter) a.flags[0] = 2;
        else if (!(std::isfinite(a.scal[C_ALPHA]) && std::isfinite(a.scal[C_BETA]))) a.flags[0] = 3;
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
        else
            cudaGetLastError();
    }
    return fn;
}

bool make_map(CUtensorMap* m, float* base, int nx, int ny, int nz, bool halo_box)
{
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t gdim[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
    cuuint64_t gstride[2] = {(cuuint64_t)nx * 4, (cuuint64_t)nx * ny * 4};
    cuuint32_t box[3] = {halo_box ? (cuuint32_t)BXW : (cuuint32_t)TX, halo_box ? (cuuint32_t)BYW : (cuuint32_t)TY, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}
}  // namespace

// --------------------------------------------------------------- host side --

struct nn_cg_plan {
    nn_ctx* ctx = nullptr;
    int nx = 0, ny = 0, nz = 0;
    int64_t G = 0;
    float op_alpha = 0, onepb = 0, invd = 0;
    const float* D = nullptr;      // caller's cell field (HET), not owned
    const float* invdv = nullptr;  // 1/diag per cell (HET), not owned
    float *r[2] = {}, *w[2] = {}, *s[2] = {}, *p = nullptr;
    CUtensorMap map_r[2], map_w[2], map_s[2], map_p, map_d, map_m;
    double* scal = nullptr;
    double* partials = nullptr;
    unsigned int* ticket = nullptr;
    int* flags = nullptr;
    int tiles = 0, init_blocks = 0, zc = 16;
    // timing of the iteration kernels
    bool timing = false;
    std::vector<cudaEvent_t> ev_a, ev_b;
    float last_ms = 0.0f;
    int last_iters = 0;
    // asynchronous solve in progress (nn_cg_async_*)
    struct {
        bool active = false;
        float* x = nullptr;
        CUtensorMap map_x;
        double rtol = 0.0;
        int max_iter = 0;
        int enqueued = 0;
        cudaStream_t cs = nullptr;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
    } as;
};

void nn_cg_plan_destroy(nn_cg_plan* pl)
{
    if (!pl) return;
    if (pl->ctx) cudaStreamSynchronize(pl->ctx->stream);
    for (int q = 0; q < 2; ++q) {
        nn_release(pl->r[q]);
        nn_release(pl->w[q]);
        nn_release(pl->s[q]);
    }
    nn_release(pl->p);
    nn_release(pl->scal);
    nn_release(pl->partials);
    nn_release(pl->ticket);
    nn_release(pl->flags);
    for (auto e : pl->ev_a) cudaEventDestroy(e);
    for (auto e : pl->ev_b) cudaEventDestroy(e);
    if (pl->as.e0) cudaEventDestroy(pl->as.e0);
    if (pl->as.e1) cudaEventDestroy(pl->as.e1);
    nn_ctx* ctx = pl->ctx;
    delete pl;
    nn_ctx_release(ctx);
}

// The TMA path needs rows that are a multiple of 16 bytes (nx % 4 == 0),
// 16-byte aligned D and 1/diag, and a driver exposing cuTensorMapEncodeTiled;
// otherwise it reports UNSUPPORTED and the caller keeps the two-kernel PCG.
// D and invdv (both null for constant coefficients) stay owned by the caller.
nn_status nn_cg_plan_create(nn_ctx* ctx, int nx, int ny, int nz, double alpha, double beta, const float* D,
                            const float* invdv, nn_cg_plan** out)
{
    *out = nullptr;
    if (nx % 4 != 0 || nx < 4 || ny < 1 || nz < 1 || !encode_fn()) return NN_ERR_UNSUPPORTED;
    if ((int64_t)nx * ny * nz > INT32_MAX) return NN_ERR_UNSUPPORTED;
    if ((D == nullptr) != (invdv == nullptr) || ((uintptr_t)D & 15) || ((uintptr_t)invdv & 15))
        return NN_ERR_UNSUPPORTED;
    nn_cg_plan* pl = new nn_cg_plan();
    pl->ctx = ctx;
    nn_ctx_retain(ctx);
    pl->nx = nx; pl->ny = ny; pl->nz = nz;
    pl->G = (int64_t)nx * ny * nz;
    pl->op_alpha = (float)alpha;
    pl->onepb = (float)(1.0 + beta);
    pl->invd = (float)(1.0 / (1.0 + beta + 6.0 * alpha));
    pl->D = D;
    pl->invdv = invdv;
    pl->init_blocks = nn_grid_for(ctx, pl->G, CG_THREADS, 8);
    const size_t G = (size_t)pl->G;
    const int max_tiles = ((nx + TX - 1) / TX) * ((ny + TY - 1) / TY) * ((nz + 3) / 4);  // zc >= 4
    const int nparts = std::max(max_tiles, pl->init_blocks);
    nn_status st = NN_OK;
    for (int q = 0; q < 2 && st == NN_OK; ++q) {
        st = nn_alloc(ctx, &pl->r[q], G);
        if (st == NN_OK) st = nn_alloc(ctx, &pl->w[q], G);
        if (st == NN_OK) st = nn_alloc(ctx, &pl->s[q], G);
    }
    if (st == NN_OK) st = nn_alloc(ctx, &pl->p, G);
    if (st == NN_OK) st = nn_alloc(ctx, &pl->scal, C_COUNT);
    if (st == NN_OK) st = nn_alloc(ctx, &pl->partials, (size_t)3 * nparts);
    if (st == NN_OK) st = nn_alloc(ctx, &pl->ticket, 1);
    if (st == NN_OK) st = nn_alloc(ctx, &pl->flags, 4);
    for (int q = 0; q < 2 && st == NN_OK; ++q)
        if (!make_map(&pl->map_r[q], pl->r[q], nx, ny, nz, true) ||
            !make_map(&pl->map_w[q], pl->w[q], nx, ny, nz, true) ||
            !make_map(&pl->map_s[q], pl->s[q], nx, ny, nz, true))
            st = NN_ERR_UNSUPPORTED;
    if (st == NN_OK && !make_map(&pl->map_p, pl->p, nx, ny, nz, false)) st = NN_ERR_UNSUPPORTED;
    if (st == NN_OK && D &&
        (!make_map(&pl->map_d, const_cast<float*>(D), nx, ny, nz, true) ||
         !make_map(&pl->map_m, const_cast<float*>(invdv), nx, ny, nz, true)))
        st = NN_ERR_UNSUPPORTED;
    if (st == NN_OK) {
        cudaError_t e = D ? cudaFuncSetAttribute(k_cg_iter<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 Layout<true>::SMEM_BYTES)
                          : cudaFuncSetAttribute(k_cg_iter<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 Layout<false>::SMEM_BYTES);
        if (e != cudaSuccess) st = nn_cuda_check(ctx, e, "cudaFuncSetAttribute(k_cg_iter)");
        // all of the unified L1/shared storage as shared memory: the most blocks per SM
        e = D ? cudaFuncSetAttribute(k_cg_iter<true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100)
              : cudaFuncSetAttribute(k_cg_iter<false>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        if (st == NN_OK && e != cudaSuccess) st = nn_cuda_check(ctx, e, "cudaFuncSetAttribute(carveout)");
    }
    if (st == NN_OK) {
        // tile depth: the fewest plane steps per block over the waves the grid
        // needs at the kernel's occupancy; each z-chunk of depth zc streams
        // zc + 2 planes
        int per_sm = 0;
        cudaError_t e = D ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_iter<true>, CG_THREADS,
                                                                          Layout<true>::SMEM_BYTES)
                          : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_iter<false>, CG_THREADS,
                                                                          Layout<false>::SMEM_BYTES);
        if (e != cudaSuccess) st = nn_cuda_check(ctx, e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        const int64_t slots = (int64_t)std::max(per_sm, 1) * ctx->num_sms;
        const int64_t cols = (int64_t)((nx + TX - 1) / TX) * ((ny + TY - 1) / TY);
        int64_t best = -1;
        for (int zc : {16, 12, 8, 6, 4}) {
            const int64_t tiles = cols * ((nz + zc - 1) / zc);
            const int64_t cost = ((tiles + slots - 1) / slots) * (zc + 2);
            if (best < 0 || cost < best) {
                best = cost;
                pl->zc = zc;
                pl->tiles = (int)tiles;
            }
        }
    }
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaMemsetAsync(pl->ticket, 0, sizeof(unsigned int), ctx->stream), "memset");
    if (st != NN_OK) {
        nn_cg_plan_destroy(pl);
        return st;
    }
    *out = pl;
    return NN_OK;
}

void nn_cg_set_timing(nn_cg_plan* pl, bool on) { pl->timing = on; }
void nn_cg_last_timing(const nn_cg_plan* pl, float* ms, int* iters)
{
    *ms = pl->last_ms;
    *iters = pl->last_iters;
}

static CgArgs cg_args(nn_cg_plan* pl, float* x, double rtol, int max_iter, int parity_out)
{
    CgArgs a;
    a.nx = pl->nx; a.ny = pl->ny; a.nz = pl->nz;
    a.zc = pl->zc;
    a.op_alpha = pl->op_alpha; a.onepb = pl->onepb; a.invd = pl->invd;
    a.D = pl->D;
    a.invdv = pl->invdv;
    a.p = pl->p;
    a.x = x;
    a.r_out = pl->r[parity_out];
    a.w_out = pl->w[parity_out];
    a.s_out = pl->s[parity_out];
    a.scal = pl->scal;
    a.partials = pl->partials;
    a.ticket = pl->ticket;
    a.flags = pl->flags;
    a.rtol2 = rtol * rtol;
    a.max_iter = max_iter;
    return a;
}

// init kernels (r0, w0, scalars) on stream cs
static nn_status enqueue_init(nn_cg_plan* pl, const float* d_b, float* d_x, double rtol, int max_iter, cudaStream_t cs)
{
    nn_ctx* ctx = pl->ctx;
    NN_CUDA(ctx, cudaMemsetAsync(pl->ticket, 0, sizeof(unsigned int), cs));  // clean after an aborted solve
    CgArgs a0 = cg_args(pl, d_x, rtol, max_iter, 0);
    if (pl->D) {
        k_cg_init_r<true><<<pl->init_blocks, CG_THREADS, 0, cs>>>(a0, d_b, d_x, pl->r[0]);
        NN_CHECK_LAUNCH(ctx, "k_cg_init_r");
        k_cg_init_w<true><<<pl->init_blocks, CG_THREADS, 0, cs>>>(a0, pl->r[0], pl->w[0], pl->s[0]);
    } else {
        k_cg_init_r<false><<<pl->init_blocks, CG_THREADS, 0, cs>>>(a0, d_b, d_x, pl->r[0]);
        NN_CHECK_LAUNCH(ctx, "k_cg_init_r");
        k_cg_init_w<false><<<pl->init_blocks, CG_THREADS, 0, cs>>>(a0, pl->r[0], pl->w[0], pl->s[0]);
    }
    NN_CHECK_LAUNCH(ctx, "k_cg_init_w");
    return NN_OK;
}

// iterations it0 .. it0 + n - 1 (each a no-op once the device flag is set)
// pdl: each iteration a programmatic dependent of the kernel before it
// (synchronous solves; an overlapped solve's waiting blocks would hold SM
// room the neuron updates use)
static nn_status enqueue_iters(nn_cg_plan* pl, float* d_x, const CUtensorMap& map_x, double rtol, int max_iter, int it0,
                               int n, cudaStream_t cs, bool pdl = false)
{
    nn_ctx* ctx = pl->ctx;
    for (int it = it0; it < it0 + n; ++it) {
        const int pin = it & 1, pout = pin ^ 1;
        CgArgs a = cg_args(pl, d_x, rtol, max_iter, pout);
        if (pdl) {
            if (pl->D)
                NN_CUDA(ctx, nn_launch_pdl(k_cg_iter<true>, dim3(pl->tiles), dim3(CG_THREADS),
                                           (size_t)Layout<true>::SMEM_BYTES, cs, pl->map_r[pin], pl->map_w[pin],
                                           pl->map_s[pin], pl->map_d, pl->map_m, pl->map_p, map_x, a));
            else
                NN_CUDA(ctx, nn_launch_pdl(k_cg_iter<false>, dim3(pl->tiles), dim3(CG_THREADS),
                                           (size_t)Layout<false>::SMEM_BYTES, cs, pl->map_r[pin], pl->map_w[pin],
                                           pl->map_s[pin], pl->map_p, pl->map_p, pl->map_p, map_x, a));
            ctx->launches++;
            continue;
        }
        if (pl->D)
            k_cg_iter<true><<<pl->tiles, CG_THREADS, Layout<true>::SMEM_BYTES, cs>>>(
                pl->map_r[pin], pl->map_w[pin], pl->map_s[pin], pl->map_d, pl->map_m, pl->map_p, map_x, a);
        else
            k_cg_iter<false><<<pl->tiles, CG_THREADS, Layout<false>::SMEM_BYTES, cs>>>(
                pl->map_r[pin], pl->map_w[pin], pl->map_s[pin], pl->map_p, pl->map_p, pl->map_p, map_x, a);
        NN_CHECK_LAUNCH(ctx, "k_cg_iter");
    }
    return NN_OK;
}

// Asynchronous solve on stream cs: the init and n iterations are enqueued
// with no host read; nn_cg_async_more adds iterations; nn_cg_async_finish
// waits for the stream, completes the solve if n was not enough and reports.
nn_status nn_cg_async_begin(nn_cg_plan* pl, const float* d_b, float* d_x, double rtol, int max_iter, int n,
                            cudaStream_t cs)
{
    nn_ctx* ctx = pl->ctx;
    if (((uintptr_t)d_x & 15) || !make_map(&pl->as.map_x, d_x, pl->nx, pl->ny, pl->nz, false))
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_cg_async_begin: x must be a 16-byte aligned device vector");
    if (!pl->as.e0) NN_CUDA(ctx, cudaEventCreate(&pl->as.e0));
    if (!pl->as.e1) NN_CUDA(ctx, cudaEventCreate(&pl->as.e1));
    pl->as.active = true;
    pl->as.x = d_x;
    pl->as.rtol = rtol;
    pl->as.max_iter = max_iter;
    pl->as.cs = cs;
    pl->as.enqueued = 0;
    if (pl->timing) NN_CUDA(ctx, cudaEventRecord(pl->as.e0, cs));
    NN_TRY(enqueue_init(pl, d_b, d_x, rtol, max_iter, cs));
    return nn_cg_async_more(pl, n);
}

nn_status nn_cg_async_more(nn_cg_plan* pl, int n)
{
    if (!pl->as.active) return NN_ERR_INVALID_ARG;
    n = std::min(n, pl->as.max_iter - pl->as.enqueued);
    if (n <= 0) return NN_OK;
    NN_TRY(enqueue_iters(pl, pl->as.x, pl->as.map_x, pl->as.rtol, pl->as.max_iter, pl->as.enqueued, n, pl->as.cs));
    pl->as.enqueued += n;
    if (pl->timing) NN_CUDA(pl->ctx, cudaEventRecord(pl->as.e1, pl->as.cs));
    return NN_OK;
}

nn_status nn_cg_async_finish(nn_cg_plan* pl, int* iters, double* relres, int* converged)
{
    nn_ctx* ctx = pl->ctx;
    if (!pl->as.active) return NN_ERR_INVALID_ARG;
    cudaStream_t cs = pl->as.cs;
    int h_flags[4] = {0, 0, 0, 0};
    while (true) {
        NN_CUDA(ctx, cudaMemcpyAsync(h_flags, pl->flags, sizeof h_flags, cudaMemcpyDeviceToHost, cs));
        NN_CUDA(ctx, cudaStreamSynchronize(cs));
        if (h_flags[0] || pl->as.enqueued >= pl->as.max_iter) break;
        NN_TRY(nn_cg_async_more(pl, 16));
    }
    double h_scal[C_COUNT];
    NN_CUDA(ctx, cudaMemcpyAsync(h_scal, pl->scal, sizeof h_scal, cudaMemcpyDeviceToHost, cs));
    NN_CUDA(ctx, cudaStreamSynchronize(cs));
    pl->as.active = false;
    if (h_flags[2]) return nn_fail(ctx, NN_ERR_TIMEOUT, "k_cg_iter: a TMA pipeline wait timed out");
    if (pl->timing) {
        float ms = 0.0f;
        NN_CUDA(ctx, cudaEventElapsedTime(&ms, pl->as.e0, pl->as.e1));
        pl->last_ms = ms;
        pl->last_iters = h_flags[1];
    }
    if (iters) *iters = h_flags[1];
    if (relres) *relres = h_scal[C_BB] > 0 ? std::sqrt(h_scal[C_RR] / h_scal[C_BB]) : 0.0;
    if (converged) *converged = h_flags[0] == 1;
    return NN_OK;
}

// Solve A x = b (x holds the initial guess).  Iterations are enqueued in
// chunks; the host reads the device flags once per chunk.
nn_status nn_cg_run(nn_cg_plan* pl, const float* d_b, float* d_x, double rtol, int max_iter, int* iters,
                    double* relres, int* converged)
{
    nn_ctx* ctx = pl->ctx;
    cudaStream_t cs = ctx->stream;
    NN_CUDA(ctx, cudaMemsetAsync(pl->ticket, 0, sizeof(unsigned int), cs));  // clean after an aborted solve
    CUtensorMap map_x;  // the caller's solution vector
    if (((uintptr_t)d_x & 15) || !make_map(&map_x, d_x, pl->nx, pl->ny, pl->nz, false))
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_cg_run: x must be a 16-byte aligned device vector");
    CgArgs a0 = cg_args(pl, d_x, rtol, max_iter, 0);
    const bool het = pl->D != nullptr;
    if (het) {
        k_cg_init_r<true><<<pl->init_blocks, CG_THREADS, 0, cs>>>(a0, d_b, d_x, pl->r[0]);
        NN_CHECK_LAUNCH(ctx, "k_cg_init_r");
        k_cg_init_w<true><<<pl->init_blocks, CG_THREADS, 0, cs>>>(a0, pl->r[0], pl->w[0], pl->s[0]);
    } else {
        k_cg_init_r<false><<<pl->init_blocks, CG_THREADS, 0, cs>>>(a0, d_b, d_x, pl->r[0]);
        NN_CHECK_LAUNCH(ctx, "k_cg_init_r");
        k_cg_init_w<false><<<pl->init_blocks, CG_THREADS, 0, cs>>>(a0, pl->r[0], pl->w[0], pl->s[0]);
    }
    NN_CHECK_LAUNCH(ctx, "k_cg_init_w");
    int h_flags[4] = {0, 0, 0, 0};
    int it = 0, nchunks = 0;
    const int chunk = 16;
    while (true) {
        NN_CUDA(ctx, cudaMemcpyAsync(h_flags, pl->flags, sizeof h_flags, cudaMemcpyDeviceToHost, cs));
        NN_CUDA(ctx, cudaStreamSynchronize(cs));
        if (h_flags[0] || it >= max_iter) break;
        if (pl->timing) {
            if ((int)pl->ev_a.size() <= nchunks) {
                cudaEvent_t e1, e2;
                NN_CUDA(ctx, cudaEventCreate(&e1));
                NN_CUDA(ctx, cudaEventCreate(&e2));
                pl->ev_a.push_back(e1);
                pl->ev_b.push_back(e2);
            }
            NN_CUDA(ctx, cudaEventRecord(pl->ev_a[nchunks], cs));
        }
        const int n = std::min(chunk, max_iter - it);
        NN_TRY(enqueue_iters(pl, d_x, map_x, rtol, max_iter, it, n, cs, true));
        it += n;
        if (pl->timing) NN_CUDA(ctx, cudaEventRecord(pl->ev_b[nchunks], cs));
        ++nchunks;
    }
    double h_scal[C_COUNT];
    NN_CUDA(ctx, cudaMemcpyAsync(h_scal, pl->scal, sizeof h_scal, cudaMemcpyDeviceToHost, cs));
    NN_CUDA(ctx, cudaStreamSynchronize(cs));
    if (h_flags[2]) return nn_fail(ctx, NN_ERR_TIMEOUT, "k_cg_iter: a TMA pipeline wait timed out");
    if (pl->timing) {
        float tot = 0.0f;
        for (int c = 0; c < nchunks; ++c) {
            float ms = 0.0f;
            NN_CUDA(ctx, cudaEventElapsedTime(&ms, pl->ev_a[c], pl->ev_b[c]));
            tot += ms;
        }
        pl->last_ms = tot;
        pl->last_iters = h_flags[1];
    }
    if (iters) *iters = h_flags[1];
    if (relres) *relres = h_scal[C_BB] > 0 ? std::sqrt(h_scal[C_RR] / h_scal[C_BB]) : 0.0;
    if (converged) *converged = h_flags[0] == 1;
    return NN_OK;
}

// Tile-depth autotuner: time `iters` iterations (after two untimed ones) of
// every candidate depth on this plan's own operator -- right-hand side d_b,
// d_x as scratch (overwritten) -- and keep the fastest.  The residual target
// is never reached, so every timed iteration does its full work.
nn_status nn_cg_plan_autotune(nn_cg_plan* pl, const float* d_b, float* d_x, int iters, int* zc_out, float* ms_out)
{
    nn_ctx* ctx = pl->ctx;
    cudaStream_t cs = ctx->stream;
    if (iters < 1) return NN_ERR_INVALID_ARG;
    CUtensorMap map_x;
    if (((uintptr_t)d_x & 15) || !make_map(&map_x, d_x, pl->nx, pl->ny, pl->nz, false))
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_cg_plan_autotune: x must be a 16-byte aligned device vector");
    const int64_t cols = (int64_t)((pl->nx + TX - 1) / TX) * ((pl->ny + TY - 1) / TY);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    NN_CUDA(ctx, cudaEventCreate(&e0));
    NN_CUDA(ctx, cudaEventCreate(&e1));
    const int zc0 = pl->zc, tiles0 = pl->tiles;
    int best_zc = zc0, best_tiles = tiles0;
    float best = 1e30f;
    nn_status st = NN_OK;
    const double rtol = 1e-30;
    const int max_iter = 1 << 30;
    int prev_zc = 0;
    for (int zc : {4, 6, 8, 12, 16, 24, 32}) {
        if (st != NN_OK || prev_zc >= pl->nz) break;  // deeper tiles than the grid change nothing
        prev_zc = zc;
        pl->zc = zc;
        pl->tiles = (int)(cols * ((pl->nz + zc - 1) / zc));
        st = nn_cuda_check(ctx, cudaMemsetAsync(d_x, 0, sizeof(float) * (size_t)pl->G, cs), "memset");
        if (st == NN_OK) st = enqueue_init(pl, d_b, d_x, rtol, max_iter, cs);
        if (st == NN_OK) st = enqueue_iters(pl, d_x, map_x, rtol, max_iter, 0, 2, cs);
        if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventRecord(e0, cs), "event");
        if (st == NN_OK) st = enqueue_iters(pl, d_x, map_x, rtol, max_iter, 2, iters, cs);
        if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventRecord(e1, cs), "event");
        int h_flags[4] = {0, 0, 0, 0};
        if (st == NN_OK)
            st = nn_cuda_check(ctx, cudaMemcpyAsync(h_flags, pl->flags, sizeof h_flags, cudaMemcpyDeviceToHost, cs),
                               "copy");
        if (st == NN_OK) st = nn_cuda_check(ctx, cudaStreamSynchronize(cs), "nn_cg_plan_autotune");
        if (st == NN_OK && h_flags[2]) st = nn_fail(ctx, NN_ERR_TIMEOUT, "k_cg_iter: a TMA pipeline wait timed out");
        float ms = 0.0f;
        if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventElapsedTime(&ms, e0, e1), "event");
        // iterations that stopped early (exact solution, non-finite) are no timing
        if (st == NN_OK && h_flags[0] == 0 && ms / iters < best) {
            best = ms / iters;
            best_zc = zc;
            best_tiles = pl->tiles;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    pl->zc = st == NN_OK ? best_zc : zc0;
    pl->tiles = st == NN_OK ? best_tiles : tiles0;
    if (zc_out) *zc_out = pl->zc;
    if (ms_out) *ms_out = best < 1e30f ? best : 0.0f;
    return st;
}

int nn_cg_plan_tile_depth(const nn_cg_plan* pl) { return pl->zc; }

// Set the tile depth (4 .. 32).
void nn_cg_plan_set_tile_depth(nn_cg_plan* pl, int zc)
{
    const int64_t cols = (int64_t)((pl->nx + TX - 1) / TX) * ((pl->ny + TY - 1) / TY);
    pl->zc = zc;
    pl->tiles = (int)(cols * ((pl->nz + zc - 1) / zc));
}
