// Geometric multigrid preconditioner and flexible CG for the 7-point
// backward-Euler operator of an nn_pcg:
//
//   (A v)_c = (1 + beta) v_c + alpha * sum_f cf (v_c - v_nb)      (v = 0 outside)
//
// with cf the harmonic mean of the cell field across face f (the cell's own
// value on a boundary face), or 1 without a cell field.
//
// No counterpart in the reference: its solver runs at most 20 unpreconditioned
// CG iterations on a 27-point Crank-Nicolson operator (src/paracrine.cu:63-134).
//
// Hierarchy.  Cell-centred, 2x coarsening per axis while every side stays even
// and the coarsest level has more than 16^3 cells (or to a requested depth).
// Coarse operators keep the 7-point form in coarse-volume units: the mass term
// is the sum over the eight children; each face conductance is half the sum of
// the four fine conductances across the coarse face, and each boundary
// conductance half the sum of the children's (for a constant field this is the
// operator discretised on the coarse grid).  Restriction sums the eight
// children; prolongation is cell-centred trilinear interpolation (weights 3/4
// and 1/4 per axis, zero outside the grid).  Smoother: damped Jacobi
// (omega = 0.8), two sweeps before and two after the coarse correction, eight
// on the coarsest level.  Restriction is not the transpose of prolongation, so
// the V-cycle is not symmetric and runs inside flexible CG (Notay, SIAM J. Sci.
// Comput. 22 (2000) 1444), which stops at the same relative residual as
// nn_pcg_solve.
//
// Kernels.  Every kernel walks grid rows (j, k) -- one division per row, none
// per cell -- with threads along x.  On the fine level a thread owns four
// consecutive cells (16-byte loads of the cell and its y/z neighbours, two
// scalar x neighbours, five x-face harmonic means for four cells) when the x
// side is a multiple of four.  Fusions on the fine level: the first two
// smoothing sweeps from a zero guess are one pass (the first sweep's values
// at the neighbours are recomputed from b and 1/diag); the direction update
// p = z + beta p runs inside the operator application (p ping-pongs between
// two buffers); the FCG dot products (r, z) and (z, q) run inside the last
// smoothing sweep.  Reductions: FP32 per thread and warp, FP64 across warps
// and blocks; the last block to arrive finalises the scalars in a fixed order
// (deterministic).  Two FCG iterations are one CUDA graph; each of their
// kernels returns at once when the device-side convergence flag is set, so
// the host launches the graph in chunks and reads the flag once per chunk.
#include <algorithm>
#include <cmath>
#include <vector>

#include "nn_internal.cuh"

namespace {

constexpr int MG_THREADS = 256;
#ifndef NN_MG_VEC
#define NN_MG_VEC 4  // cells per thread on the fine level (4 or 2) when the x side allows
#endif
#ifndef NN_MG_MIN_BLOCKS
// resident blocks per SM the stencils are compiled for: 4 (64 registers) is
// the fastest of 1, 3, 4, 5, 6 on the 256^3 solve (more spill, fewer leave
// too few warps to cover the load latency)
#define NN_MG_MIN_BLOCKS 4
#endif
constexpr int MG_MAX_LEVELS = 8;
constexpr int MG_COARSE_CELLS = 4096;  // stop coarsening at this size

enum { S_BB = 0, S_RR, S_RZ, S_PQ, S_BETA, S_TOL, S_COUNT };
enum { F_DONE = 0, F_ITERS, F_STATE, F_MAXIT, F_COUNT };  // F_STATE: 0 ok, 1 non-finite, 2 breakdown

// rows (j, k) of an ny x nz grid of rows, blockDim.y rows per block step
#define MG_ROWS(ny_, nz_, row) \
    for (int row = blockIdx.x * blockDim.y + threadIdx.y; row < (ny_) * (nz_); row += gridDim.x * blockDim.y)

// ------------------------------------------------------------ vector I/O --

template <int V>
__device__ __forceinline__ void ldv(const float* p, float (&o)[V])
{
    if constexpr (V == 4) {
        const float4 t = *reinterpret_cast<const float4*>(p);
        o[0] = t.x; o[1] = t.y; o[2] = t.z; o[3] = t.w;
    } else if constexpr (V == 2) {
        const float2 t = *reinterpret_cast<const float2*>(p);
        o[0] = t.x; o[1] = t.y;
    } else {
#pragma unroll
        for (int v = 0; v < V; ++v) o[v] = p[v];
    }
}

template <int V>
__device__ __forceinline__ void stv(float* p, const float (&o)[V])
{
    if constexpr (V == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(o[0], o[1], o[2], o[3]);
    } else if constexpr (V == 2) {
        *reinterpret_cast<float2*>(p) = make_float2(o[0], o[1]);
    } else {
#pragma unroll
        for (int v = 0; v < V; ++v) p[v] = o[v];
    }
}

// Fields whose values the stencils read at a cell and its neighbours.
struct FPlain {  // a[i]
    const float* a;
    __device__ __forceinline__ float one(int i) const { return a[i]; }
    template <int V>
    __device__ __forceinline__ void vec(int i, float (&o)[V]) const { ldv<V>(a + i, o); }
};
struct FLin {  // z[i] + beta p[i]
    const float *z, *p;
    float beta;
    __device__ __forceinline__ float one(int i) const { return z[i] + beta * p[i]; }
    template <int V>
    __device__ __forceinline__ void vec(int i, float (&o)[V]) const
    {
        float t[V];
        ldv<V>(z + i, o);
        ldv<V>(p + i, t);
#pragma unroll
        for (int v = 0; v < V; ++v) o[v] += beta * t[v];
    }
};
struct FInvd {  // omega b[i] invd[i] (invd null: the constant invd_c)
    const float *b, *invd;
    float invd_c, omega;
    __device__ __forceinline__ float one(int i) const { return omega * b[i] * (invd ? invd[i] : invd_c); }
    template <int V>
    __device__ __forceinline__ void vec(int i, float (&o)[V]) const
    {
        ldv<V>(b + i, o);
        if (invd) {
            float t[V];
            ldv<V>(invd + i, t);
#pragma unroll
            for (int v = 0; v < V; ++v) o[v] *= omega * t[v];
        } else {
#pragma unroll
            for (int v = 0; v < V; ++v) o[v] *= omega * invd_c;
        }
    }
};
struct FDiv {  // omega b[i] / diag[i]
    const float *b, *diag;
    float omega;
    __device__ __forceinline__ float one(int i) const { return omega * __fdividef(b[i], diag[i]); }
    template <int V>
    __device__ __forceinline__ void vec(int i, float (&o)[V]) const
    {
#pragma unroll
        for (int v = 0; v < V; ++v) o[v] = one(i + v);
    }
};

// A field at V consecutive cells of a row and at their six neighbours
// (zero outside the grid).
template <int V>
struct Nb {
    float c[V], ym[V], yp[V], zm[V], zp[V];
    float xm, xp;
};

template <int V, class F>
__device__ __forceinline__ void gather(const F& f, int c, int i0, int j, int k, int nx, int ny, int nz, Nb<V>& n)
{
    const int sy = nx, sz = nx * ny;
    f.template vec<V>(c, n.c);
    n.xm = i0 > 0 ? f.one(c - 1) : 0.0f;
    n.xp = i0 + V < nx ? f.one(c + V) : 0.0f;
    if (j > 0) f.template vec<V>(c - sy, n.ym);
    else {
#pragma unroll
        for (int v = 0; v < V; ++v) n.ym[v] = 0.0f;
    }
    if (j < ny - 1) f.template vec<V>(c + sy, n.yp);
    else {
#pragma unroll
        for (int v = 0; v < V; ++v) n.yp[v] = 0.0f;
    }
    if (k > 0) f.template vec<V>(c - sz, n.zm);
    else {
#pragma unroll
        for (int v = 0; v < V; ++v) n.zm[v] = 0.0f;
    }
    if (k < nz - 1) f.template vec<V>(c + sz, n.zp);
    else {
#pragma unroll
        for (int v = 0; v < V; ++v) n.zp[v] = 0.0f;
    }
}

__device__ __forceinline__ float hmean(float a, float b) { return __fdividef(2.0f * a * b, a + b); }

// ------------------------------------------------------------- operators --

// Level 0: coefficients from the cell field (or a constant coefficient).
struct Op0 {
    int nx, ny, nz;
    const float* D;      // null: constant coefficient 1
    const float* invd;   // 1 / diag per cell (null: invd_c)
    float invd_c;
    float alpha, onepb;

    // (A x) and the diagonal at V consecutive cells, x given with neighbours
    template <int V>
    __device__ __forceinline__ void apply(int c, int i0, int j, int k, const Nb<V>& x, float (&ax)[V],
                                          float (&dg)[V]) const
    {
        if (!D) {
            const float d = onepb + 6.0f * alpha;
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const float w = v > 0 ? x.c[v - 1] : x.xm;
                const float e = v < V - 1 ? x.c[v + 1] : x.xp;
                dg[v] = d;
                ax[v] = d * x.c[v] - alpha * (w + e + x.ym[v] + x.yp[v] + x.zm[v] + x.zp[v]);
            }
            return;
        }
        Nb<V> Dn;
        gather(FPlain{D}, c, i0, j, k, nx, ny, nz, Dn);
        // x faces 0..V: face v lies between cells v-1 and v
        float fx[V + 1];
#pragma unroll
        for (int v = 0; v <= V; ++v) {
            const float dl = v > 0 ? Dn.c[v - 1] : Dn.xm;
            const float dr = v < V ? Dn.c[v] : Dn.xp;
            const bool in = v == 0 ? i0 > 0 : (v == V ? i0 + V < nx : true);
            fx[v] = in ? hmean(dl, dr) : (v == 0 ? Dn.c[0] : Dn.c[V - 1]);
        }
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const float dc = Dn.c[v];
            const float fs = j > 0 ? hmean(dc, Dn.ym[v]) : dc;
            const float fn = j < ny - 1 ? hmean(dc, Dn.yp[v]) : dc;
            const float fd = k > 0 ? hmean(dc, Dn.zm[v]) : dc;
            const float fu = k < nz - 1 ? hmean(dc, Dn.zp[v]) : dc;
            const float w = v > 0 ? x.c[v - 1] : x.xm;
            const float e = v < V - 1 ? x.c[v + 1] : x.xp;
            dg[v] = onepb + alpha * (fx[v] + fx[v + 1] + fs + fn + fd + fu);
            ax[v] = dg[v] * x.c[v] -
                    alpha * (fx[v] * w + fx[v + 1] * e + fs * x.ym[v] + fn * x.yp[v] + fd * x.zm[v] + fu * x.zp[v]);
        }
    }
    // field of the first smoothing sweep from zero: omega b / diag
    __device__ __forceinline__ FInvd first(const float* b, float omega) const { return FInvd{b, invd, invd_c, omega}; }

    // interior-face conductances (-x, +x, -y, +y, -z, +z) and the boundary
    // conductance of one cell (coarsening)
    __device__ __forceinline__ void faces(int c, int i, int j, int k, float w[6], float& wb) const
    {
        const int sy = nx, sz = nx * ny;
        const bool in[6] = {i > 0, i < nx - 1, j > 0, j < ny - 1, k > 0, k < nz - 1};
        const int off[6] = {-1, 1, -sy, sy, -sz, sz};
        const float dc = D ? D[c] : 1.0f;
        wb = 0.0f;
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            const float cf = !in[f] ? dc : (D ? hmean(dc, D[c + off[f]]) : 1.0f);
            w[f] = in[f] ? alpha * cf : 0.0f;
            if (!in[f]) wb += alpha * cf;
        }
    }
};

// Coarse levels: stored conductances to the +x/+y/+z neighbours (0 on the far
// boundary), boundary conductances and the diagonal.
struct OpF {
    int nx, ny, nz;
    const float *wx, *wy, *wz, *wb, *diag;

    template <int V>
    __device__ __forceinline__ void apply(int c, int i0, int j, int k, const Nb<V>& x, float (&ax)[V],
                                          float (&dg)[V]) const
    {
        const int sy = nx, sz = nx * ny;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int cc = c + v;
            const float fw = (i0 + v) > 0 ? wx[cc - 1] : 0.0f;
            const float fe = wx[cc];
            const float fs = j > 0 ? wy[cc - sy] : 0.0f;
            const float fn = wy[cc];
            const float fd = k > 0 ? wz[cc - sz] : 0.0f;
            const float fu = wz[cc];
            const float w = v > 0 ? x.c[v - 1] : x.xm;
            const float e = v < V - 1 ? x.c[v + 1] : x.xp;
            dg[v] = diag[cc];
            ax[v] = dg[v] * x.c[v] - (fw * w + fe * e + fs * x.ym[v] + fn * x.yp[v] + fd * x.zm[v] + fu * x.zp[v]);
        }
    }
    __device__ __forceinline__ FDiv first(const float* b, float omega) const { return FDiv{b, diag, omega}; }

    __device__ __forceinline__ void faces(int c, int i, int j, int k, float w[6], float& b) const
    {
        const int sy = nx, sz = nx * ny;
        w[0] = i > 0 ? wx[c - 1] : 0.0f;
        w[1] = wx[c];
        w[2] = j > 0 ? wy[c - sy] : 0.0f;
        w[3] = wy[c];
        w[4] = k > 0 ? wz[c - sz] : 0.0f;
        w[5] = wz[c];
        b = wb[c];
    }
};

// ------------------------------------------------------------ reductions --

// Block partials of NSUM values; the last block to arrive writes the grid
// totals to out[] (fixed order) and returns true in every thread of that block.
template <int NSUM>
__device__ bool mg_reduce(const float* v, double* partials, unsigned int* ticket, double* out)
{
    __shared__ double ws[NSUM][MG_THREADS / 32];
    __shared__ bool last;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int lane = tid & 31, w = tid >> 5;
#pragma unroll
    for (int q = 0; q < NSUM; ++q) {
        float s = v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) ws[q][w] = (double)s;
    }
    __syncthreads();
    if (tid == 0) {
        for (int q = 0; q < NSUM; ++q) {
            double s = 0.0;
            for (int u = 0; u < MG_THREADS / 32; ++u) s += ws[q][u];
            partials[(size_t)q * gridDim.x + blockIdx.x] = s;
        }
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    for (int q = 0; q < NSUM; ++q) {
        const volatile double* pp = partials + (size_t)q * gridDim.x;
        double s = 0.0;
        for (unsigned b = tid; b < gridDim.x; b += MG_THREADS) s += pp[b];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        __syncthreads();
        if (lane == 0) ws[q][w] = s;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int u = 0; u < MG_THREADS / 32; ++u) t += ws[q][u];
            out[q] = t;
        }
    }
    if (tid == 0) *ticket = 0;
    __syncthreads();
    return true;
}

struct Red {
    double* partials;
    unsigned int* ticket;
    double* scal;
    int* flags;
};

__device__ __forceinline__ bool is_tid0() { return threadIdx.x == 0 && threadIdx.y == 0; }

// ---------------------------------------------------------------- V-cycle --

// y = omega D^-1 b (one sweep from a zero guess)
template <class Op>
__global__ void __launch_bounds__(MG_THREADS) k_mg_smooth0(Op op, const float* b, float omega, float* y,
                                                           const int* flags)
{
    if (flags && flags[F_DONE]) return;
    MG_ROWS(op.ny, op.nz, row)
    {
        const int j = row % op.ny, k = row / op.ny;
        for (int i = threadIdx.x; i < op.nx; i += blockDim.x) {
            const int c = i + op.nx * row;
            Nb<1> xn{};
            float ax[1], dg[1];
            op.template apply<1>(c, i, j, k, xn, ax, dg);
            y[c] = omega * __fdividef(b[c], dg[0]);
        }
    }
}

// Two sweeps from a zero guess in one pass: x1 = omega D^-1 b (recomputed at
// the neighbours), y = x1 + omega D^-1 (b - A x1).
template <int V, class Op>
__global__ void __launch_bounds__(MG_THREADS, NN_MG_MIN_BLOCKS) k_mg_pre2(Op op, const float* b, float omega, float* y,
                                                        const int* flags)
{
    if (flags && flags[F_DONE]) return;
    const int gx = op.nx / V;
    MG_ROWS(op.ny, op.nz, row)
    {
        const int j = row % op.ny, k = row / op.ny;
        for (int g = threadIdx.x; g < gx; g += blockDim.x) {
            const int i0 = g * V, c = i0 + op.nx * row;
            Nb<V> xn;
            gather(op.first(b, omega), c, i0, j, k, op.nx, op.ny, op.nz, xn);
            float ax[V], dg[V], bv[V], out[V];
            op.template apply<V>(c, i0, j, k, xn, ax, dg);
            ldv<V>(b + c, bv);
#pragma unroll
            for (int v = 0; v < V; ++v) out[v] = xn.c[v] + omega * __fdividef(bv[v] - ax[v], dg[v]);
            stv<V>(y + c, out);
        }
    }
}

// y = x + omega D^-1 (b - A x).  DOTS (fine level, inside FCG): b is the
// residual r; also (r, y) and (y, q) -> RZ and BETA = -(y, q) / PQ.
template <int V, bool DOTS, class Op>
__global__ void __launch_bounds__(MG_THREADS, NN_MG_MIN_BLOCKS) k_mg_jacobi(Op op, const float* b, const float* x, float omega,
                                                          float* y, const int* flags, const float* q, Red red)
{
    if (flags && flags[F_DONE]) return;
    const int gx = op.nx / V;
    float acc[2] = {0.0f, 0.0f};
    MG_ROWS(op.ny, op.nz, row)
    {
        const int j = row % op.ny, k = row / op.ny;
        for (int g = threadIdx.x; g < gx; g += blockDim.x) {
            const int i0 = g * V, c = i0 + op.nx * row;
            Nb<V> xn;
            gather(FPlain{x}, c, i0, j, k, op.nx, op.ny, op.nz, xn);
            float ax[V], dg[V], bv[V], out[V];
            op.template apply<V>(c, i0, j, k, xn, ax, dg);
            ldv<V>(b + c, bv);
#pragma unroll
            for (int v = 0; v < V; ++v) out[v] = xn.c[v] + omega * __fdividef(bv[v] - ax[v], dg[v]);
            stv<V>(y + c, out);
            if constexpr (DOTS) {
                float qv[V];
                ldv<V>(q + c, qv);
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    acc[0] += bv[v] * out[v];
                    acc[1] += out[v] * qv[v];
                }
            }
        }
    }
    if constexpr (DOTS) {
        double o[2];
        if (mg_reduce<2>(acc, red.partials, red.ticket, o) && is_tid0()) {
            red.scal[S_RZ] = o[0];
            red.scal[S_BETA] = -o[1] / red.scal[S_PQ];
        }
    }
}

// bc = R (b - A x): each coarse cell sums the residual of its eight children.
// A thread owns VC consecutive coarse cells (2 VC fine cells per fine row).
template <int VC, class Op>
__global__ void __launch_bounds__(MG_THREADS) k_mg_restrict(Op op, const float* b, const float* x, float* bc,
                                                            const int* flags)
{
    if (flags && flags[F_DONE]) return;
    constexpr int V = 2 * VC;
    const int cx = op.nx / 2, cy = op.ny / 2, cz = op.nz / 2;
    const int gx = cx / VC;
    MG_ROWS(cy, cz, crow)
    {
        const int J = crow % cy, K = crow / cy;
        for (int g = threadIdx.x; g < gx; g += blockDim.x) {
            const int I0 = g * VC, i0 = 2 * I0;
            float acc[VC];
#pragma unroll
            for (int u = 0; u < VC; ++u) acc[u] = 0.0f;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int j = 2 * J + (q & 1), k = 2 * K + (q >> 1);
                const int c = i0 + op.nx * (j + op.ny * k);
                Nb<V> xn;
                gather(FPlain{x}, c, i0, j, k, op.nx, op.ny, op.nz, xn);
                float ax[V], dg[V], bv[V];
                op.template apply<V>(c, i0, j, k, xn, ax, dg);
                ldv<V>(b + c, bv);
#pragma unroll
                for (int u = 0; u < VC; ++u) acc[u] += (bv[2 * u] - ax[2 * u]) + (bv[2 * u + 1] - ax[2 * u + 1]);
            }
            stv<VC>(bc + I0 + cx * crow, acc);
        }
    }
}

// x += P xc (cell-centred trilinear; zero outside the coarse grid)
__global__ void __launch_bounds__(MG_THREADS) k_mg_prolong_add(int nx, int ny, int nz, const float* xc, float* x,
                                                               const int* flags)
{
    if (flags && flags[F_DONE]) return;
    const int cx = nx / 2, cy = ny / 2, cz = nz / 2;
    MG_ROWS(ny, nz, row)
    {
        const int j = row % ny, k = row / ny;
        const int J = j >> 1, K = k >> 1;
        const int J2 = (j & 1) ? J + 1 : J - 1, K2 = (k & 1) ? K + 1 : K - 1;
        const bool oj = J2 >= 0 && J2 < cy, ok = K2 >= 0 && K2 < cz;
        // the four coarse rows this fine row interpolates from, with weights
        const float* r00 = xc + cx * (J + cy * K);
        const float* r10 = xc + cx * ((oj ? J2 : J) + cy * K);
        const float* r01 = xc + cx * (J + cy * (ok ? K2 : K));
        const float* r11 = xc + cx * ((oj ? J2 : J) + cy * (ok ? K2 : K));
        const float wj2 = oj ? 0.25f : 0.0f, wk2 = ok ? 0.25f : 0.0f;
        const float w00 = 0.75f * 0.75f, w10 = wj2 * 0.75f, w01 = 0.75f * wk2, w11 = wj2 * wk2;
        for (int i = threadIdx.x; i < nx; i += blockDim.x) {
            const int I = i >> 1, I2 = (i & 1) ? I + 1 : I - 1;
            const bool oi = I2 >= 0 && I2 < cx;
            const int Ib = oi ? I2 : I;
            const float wi2 = oi ? 0.25f : 0.0f;
            const float a = w00 * r00[I] + w10 * r10[I] + w01 * r01[I] + w11 * r11[I];
            const float e = w00 * r00[Ib] + w10 * r10[Ib] + w01 * r01[Ib] + w11 * r11[Ib];
            x[i + nx * row] += 0.75f * a + wi2 * e;
        }
    }
}

// ------------------------------------------------------------------ setup --

// Coarse conductances from the fine operator: face = half the sum of the four
// fine faces across it; boundary = half the children's boundary sum.
template <class Op>
__global__ void __launch_bounds__(MG_THREADS) k_mg_coarsen(Op op, float* wx, float* wy, float* wz, float* wb)
{
    const int cx = op.nx / 2, cy = op.ny / 2, cz = op.nz / 2;
    MG_ROWS(cy, cz, crow)
    {
        const int J = crow % cy, K = crow / cy;
        for (int I = threadIdx.x; I < cx; I += blockDim.x) {
            float sx = 0.0f, sy = 0.0f, sz = 0.0f, sb = 0.0f;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int di = q & 1, dj = (q >> 1) & 1, dk = q >> 2;
                const int i = 2 * I + di, j = 2 * J + dj, k = 2 * K + dk;
                const int c = i + op.nx * (j + op.ny * k);
                float w[6], bnd;
                op.faces(c, i, j, k, w, bnd);
                if (di) sx += w[1];
                if (dj) sy += w[3];
                if (dk) sz += w[5];
                sb += bnd;
            }
            const int C = I + cx * crow;
            wx[C] = I < cx - 1 ? 0.5f * sx : 0.0f;
            wy[C] = J < cy - 1 ? 0.5f * sy : 0.0f;
            wz[C] = K < cz - 1 ? 0.5f * sz : 0.0f;
            wb[C] = 0.5f * sb;
        }
    }
}

// diag = mass + boundary + sum of the six face conductances
__global__ void __launch_bounds__(MG_THREADS) k_mg_diag(int nx, int ny, int nz, const float* wx, const float* wy,
                                                        const float* wz, const float* wb, float mass, float* diag)
{
    MG_ROWS(ny, nz, row)
    {
        const int j = row % ny, k = row / ny;
        for (int i = threadIdx.x; i < nx; i += blockDim.x) {
            const int c = i + nx * row;
            float s = mass + wb[c] + wx[c] + wy[c] + wz[c];
            if (i > 0) s += wx[c - 1];
            if (j > 0) s += wy[c - nx];
            if (k > 0) s += wz[c - nx * ny];
            diag[c] = s;
        }
    }
}

// -------------------------------------------------------- flexible CG --

// The call's tolerance and iteration limit (read by the captured iteration).
__global__ void k_fcg_set(double* scal, int* flags, double rtol2, int max_iter)
{
    scal[S_TOL] = rtol2;
    flags[F_MAXIT] = max_iter;
}

// r = b - A x; (b, b), (r, r); converged at once when (r, r) <= rtol2 (b, b)
template <int V>
__global__ void __launch_bounds__(MG_THREADS, NN_MG_MIN_BLOCKS) k_fcg_init(Op0 op, const float* b, const float* x, float* r, Red red)
{
    const int gx = op.nx / V;
    float acc[2] = {0.0f, 0.0f};
    MG_ROWS(op.ny, op.nz, row)
    {
        const int j = row % op.ny, k = row / op.ny;
        for (int g = threadIdx.x; g < gx; g += blockDim.x) {
            const int i0 = g * V, c = i0 + op.nx * row;
            Nb<V> xn;
            gather(FPlain{x}, c, i0, j, k, op.nx, op.ny, op.nz, xn);
            float ax[V], dg[V], bv[V], rv[V];
            op.template apply<V>(c, i0, j, k, xn, ax, dg);
            ldv<V>(b + c, bv);
#pragma unroll
            for (int v = 0; v < V; ++v) {
                rv[v] = bv[v] - ax[v];
                acc[0] += bv[v] * bv[v];
                acc[1] += rv[v] * rv[v];
            }
            stv<V>(r + c, rv);
        }
    }
    double o[2];
    if (mg_reduce<2>(acc, red.partials, red.ticket, o) && is_tid0()) {
        const double rtol2 = red.scal[S_TOL];
        red.scal[S_BB] = o[0];
        red.scal[S_RR] = o[1];
        red.flags[F_ITERS] = 0;
        red.flags[F_STATE] = isfinite(o[1]) ? 0 : 1;
        red.flags[F_DONE] = (o[1] <= rtol2 * o[0] || !isfinite(o[1]) || red.flags[F_MAXIT] <= 0) ? 1 : 0;
    }
}

// p = z; (r, z); beta = 0 (the first direction update keeps p = z)
__global__ void __launch_bounds__(MG_THREADS) k_fcg_first(const float* r, const float* z, float* p, int G, Red red)
{
    if (red.flags[F_DONE]) return;
    float acc[1] = {0.0f};
    const int tid = blockIdx.x * MG_THREADS + threadIdx.y * blockDim.x + threadIdx.x;
    for (int c = tid; c < G; c += gridDim.x * MG_THREADS) {
        p[c] = z[c];
        acc[0] += r[c] * z[c];
    }
    double o[1];
    if (mg_reduce<1>(acc, red.partials, red.ticket, o) && is_tid0()) {
        red.scal[S_RZ] = o[0];
        red.scal[S_BETA] = 0.0;
    }
}

// p_new = z + beta p_old; q = A p_new; (p_new, q)
template <int V>
__global__ void __launch_bounds__(MG_THREADS, NN_MG_MIN_BLOCKS) k_fcg_ap_dir(Op0 op, const float* z, const float* p_old, float* p_new,
                                                           float* q, Red red)
{
    if (red.flags[F_DONE]) return;
    const float beta = (float)red.scal[S_BETA];
    const int gx = op.nx / V;
    float acc[1] = {0.0f};
    MG_ROWS(op.ny, op.nz, row)
    {
        const int j = row % op.ny, k = row / op.ny;
        for (int g = threadIdx.x; g < gx; g += blockDim.x) {
            const int i0 = g * V, c = i0 + op.nx * row;
            Nb<V> pn;
            gather(FLin{z, p_old, beta}, c, i0, j, k, op.nx, op.ny, op.nz, pn);
            float qv[V], dg[V];
            op.template apply<V>(c, i0, j, k, pn, qv, dg);
            stv<V>(p_new + c, pn.c);
            stv<V>(q + c, qv);
#pragma unroll
            for (int v = 0; v < V; ++v) acc[0] += pn.c[v] * qv[v];
        }
    }
    double o[1];
    if (mg_reduce<1>(acc, red.partials, red.ticket, o) && is_tid0()) red.scal[S_PQ] = o[0];
}

// a = (r, z) / (p, q); x += a p; r -= a q; (r, r); convergence and limit tests
template <int V>
__global__ void __launch_bounds__(MG_THREADS) k_fcg_update(float* x, float* r, const float* p, const float* q, int G,
                                                           Red red)
{
    if (red.flags[F_DONE]) return;
    const double pq = red.scal[S_PQ];
    const float a = pq > 0.0 ? (float)(red.scal[S_RZ] / pq) : 0.0f;
    float acc[1] = {0.0f};
    const int tid = blockIdx.x * MG_THREADS + threadIdx.y * blockDim.x + threadIdx.x;
    for (int c = tid * V; c < G; c += gridDim.x * MG_THREADS * V) {
        float xv[V], rv[V], pv[V], qv[V];
        ldv<V>(x + c, xv);
        ldv<V>(r + c, rv);
        ldv<V>(p + c, pv);
        ldv<V>(q + c, qv);
#pragma unroll
        for (int v = 0; v < V; ++v) {
            xv[v] += a * pv[v];
            rv[v] -= a * qv[v];
            acc[0] += rv[v] * rv[v];
        }
        stv<V>(x + c, xv);
        stv<V>(r + c, rv);
    }
    double o[1];
    if (mg_reduce<1>(acc, red.partials, red.ticket, o) && is_tid0()) {
        red.scal[S_RR] = o[0];
        const int it = red.flags[F_ITERS] + 1;
        red.flags[F_ITERS] = it;
        if (!(pq > 0.0)) {
            red.flags[F_STATE] = 2;
            red.flags[F_DONE] = 1;
        } else if (!isfinite(o[0])) {
            red.flags[F_STATE] = 1;
            red.flags[F_DONE] = 1;
        } else if (o[0] <= red.scal[S_TOL] * red.scal[S_BB] || it >= red.flags[F_MAXIT]) {
            red.flags[F_DONE] = 1;
        }
    }
}

// ---------------------------------------------- Jacobi-PCG on one level --
// (training targets for a learned level solver; host-driven, small grids)

// x = 0; r = b; p = D^-1 r; (r, D^-1 r), (b, b)
__global__ void __launch_bounds__(MG_THREADS) k_lcg_init(OpF op, const float* b, float* x, float* r, float* p, Red red)
{
    float acc[2] = {0.0f, 0.0f};
    MG_ROWS(op.ny, op.nz, row)
    {
        for (int i = threadIdx.x; i < op.nx; i += blockDim.x) {
            const int c = i + op.nx * row;
            const float bc = b[c];
            x[c] = 0.0f;
            r[c] = bc;
            const float z = __fdividef(bc, op.diag[c]);
            p[c] = z;
            acc[0] += bc * z;
            acc[1] += bc * bc;
        }
    }
    double o[2];
    if (mg_reduce<2>(acc, red.partials, red.ticket, o) && is_tid0()) {
        red.scal[S_RZ] = o[0];
        red.scal[S_BB] = o[1];
        red.scal[S_RR] = o[1];
    }
}

// q = A p; (p, q)
__global__ void __launch_bounds__(MG_THREADS) k_lcg_ap(OpF op, const float* p, float* q, Red red)
{
    float acc[1] = {0.0f};
    MG_ROWS(op.ny, op.nz, row)
    {
        const int j = row % op.ny, k = row / op.ny;
        for (int i = threadIdx.x; i < op.nx; i += blockDim.x) {
            const int c = i + op.nx * row;
            Nb<1> pn;
            gather(FPlain{p}, c, i, j, k, op.nx, op.ny, op.nz, pn);
            float qv[1], dg[1];
            op.template apply<1>(c, i, j, k, pn, qv, dg);
            q[c] = qv[0];
            acc[0] += pn.c[0] * qv[0];
        }
    }
    double o[1];
    if (mg_reduce<1>(acc, red.partials, red.ticket, o) && is_tid0()) red.scal[S_PQ] = o[0];
}

// a = (r, z) / (p, q); x += a p; r -= a q; new (r, z) and (r, r); beta
__global__ void __launch_bounds__(MG_THREADS) k_lcg_update(OpF op, float* x, float* r, const float* p, const float* q,
                                                           Red red)
{
    const double pq = red.scal[S_PQ];
    const float a = pq > 0.0 ? (float)(red.scal[S_RZ] / pq) : 0.0f;
    float acc[2] = {0.0f, 0.0f};
    MG_ROWS(op.ny, op.nz, row)
    {
        for (int i = threadIdx.x; i < op.nx; i += blockDim.x) {
            const int c = i + op.nx * row;
            x[c] += a * p[c];
            const float rc = r[c] - a * q[c];
            r[c] = rc;
            acc[0] += rc * __fdividef(rc, op.diag[c]);
            acc[1] += rc * rc;
        }
    }
    double o[2];
    if (mg_reduce<2>(acc, red.partials, red.ticket, o) && is_tid0()) {
        const double rz_old = red.scal[S_RZ];
        red.scal[S_BETA] = rz_old > 0.0 ? o[0] / rz_old : 0.0;
        red.scal[S_RZ] = o[0];
        red.scal[S_RR] = o[1];
    }
}

// p = D^-1 r + beta p
__global__ void __launch_bounds__(MG_THREADS) k_lcg_dir(OpF op, const float* r, float* p, Red red)
{
    const float bt = (float)red.scal[S_BETA];
    MG_ROWS(op.ny, op.nz, row)
    {
        for (int i = threadIdx.x; i < op.nx; i += blockDim.x) {
            const int c = i + op.nx * row;
            p[c] = __fdividef(r[c], op.diag[c]) + bt * p[c];
        }
    }
}

}  // namespace

// ================================================================ object ==

struct MgLevel {
    int nx = 0, ny = 0, nz = 0;
    int G = 0;
    float mass = 0.0f;
    float *wx = nullptr, *wy = nullptr, *wz = nullptr, *wb = nullptr, *diag = nullptr;  // levels >= 1
    float *b = nullptr, *x = nullptr, *t = nullptr;                                     // work
    OpF op() const { return OpF{nx, ny, nz, wx, wy, wz, wb, diag}; }
};

struct nn_mg {
    nn_ctx* ctx = nullptr;
    nn_pcg* pc = nullptr;
    Op0 op0{};
    int vec0 = 1;                // cells per thread on the fine level (4 when nx % 4 == 0)
    std::vector<MgLevel> lv;
    float omega = 0.8f;
    int nu = 2, coarse_sweeps = 8;
    float *r = nullptr, *z = nullptr, *q = nullptr;  // FCG vectors
    float* p[2] = {nullptr, nullptr};                // directions (ping-pong)
    double* scal = nullptr;
    int* flags = nullptr;        // device
    int* h_flags = nullptr;      // pinned host copy
    double* partials = nullptr;
    unsigned int* ticket = nullptr;
    int nblocks = 1;             // grid of the reducing kernels
    cudaGraphExec_t graph = nullptr;  // two FCG iterations
    float* graph_x = nullptr;    // solution array the graph was captured for
    int64_t graph_launches = 0;
    int last_iters = 0;
    // optional replacement of one level's coarse treatment (that level's
    // pre-smoothing and everything below it) by a caller's solver
    int hook_level = -1;
    nn_mg_level_fn hook_fn = nullptr;
    void* hook_user = nullptr;
    int hook_sweeps = 2;  // smoothing sweeps after the level solver
    // optional recorder of the right-hand sides that reach one level (solves
    // then run without the captured graph)
    int rec_level = -1;
    nn_mg_record_fn rec_fn = nullptr;
    void* rec_user = nullptr;
};

namespace {

// Launch shape for a kernel walking rows of gx thread-groups each.
struct Shape {
    dim3 grid, block;
};

Shape shape_for(const nn_ctx* ctx, int gx, int rows)
{
    int bx = 32;
    while (bx < gx && bx < MG_THREADS) bx *= 2;
    const int by = MG_THREADS / bx;
    int64_t blocks = ((int64_t)rows + by - 1) / by;
    blocks = std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)ctx->num_sms * 8));
    return Shape{dim3((unsigned)blocks), dim3(bx, by)};
}

Red red_of(const nn_mg* mg) { return Red{mg->partials, mg->ticket, mg->scal, mg->flags}; }

template <class Op>
nn_status launch_smooth0(nn_mg* mg, const Op& op, const float* b, float* y, const int* flags)
{
    const Shape s = shape_for(mg->ctx, op.nx, op.ny * op.nz);
    k_mg_smooth0<Op><<<s.grid, s.block, 0, mg->ctx->stream>>>(op, b, mg->omega, y, flags);
    NN_CHECK_LAUNCH(mg->ctx, "k_mg_smooth0");
    return NN_OK;
}

template <int V, class Op>
nn_status launch_pre2(nn_mg* mg, const Op& op, const float* b, float* y, const int* flags)
{
    const Shape s = shape_for(mg->ctx, op.nx / V, op.ny * op.nz);
    k_mg_pre2<V, Op><<<s.grid, s.block, 0, mg->ctx->stream>>>(op, b, mg->omega, y, flags);
    NN_CHECK_LAUNCH(mg->ctx, "k_mg_pre2");
    return NN_OK;
}

template <int V, bool DOTS, class Op>
nn_status launch_jacobi(nn_mg* mg, const Op& op, const float* b, const float* x, float* y, const int* flags,
                        const float* q = nullptr)
{
    Shape s = shape_for(mg->ctx, op.nx / V, op.ny * op.nz);
    if (DOTS) s.grid = dim3(mg->nblocks);  // the partials buffer holds nblocks entries
    k_mg_jacobi<V, DOTS, Op><<<s.grid, s.block, 0, mg->ctx->stream>>>(op, b, x, mg->omega, y, flags, q, red_of(mg));
    NN_CHECK_LAUNCH(mg->ctx, "k_mg_jacobi");
    return NN_OK;
}

template <int VC, class Op>
nn_status launch_restrict(nn_mg* mg, const Op& op, const float* b, const float* x, float* bc, const int* flags)
{
    const Shape s = shape_for(mg->ctx, op.nx / 2 / VC, (op.ny / 2) * (op.nz / 2));
    k_mg_restrict<VC, Op><<<s.grid, s.block, 0, mg->ctx->stream>>>(op, b, x, bc, flags);
    NN_CHECK_LAUNCH(mg->ctx, "k_mg_restrict");
    return NN_OK;
}

nn_status vcycle(nn_mg* mg, int l, const float* b, float* out, const int* flags, const float* dots_q);

// One level of the V-cycle with V cells per thread: pre-smoothing from zero,
// the coarse correction, post-smoothing into out.  dots_q (fine level inside
// FCG): the last sweep also forms the FCG dot products with this q.
template <int V, class Op>
nn_status vlevel(nn_mg* mg, int l, const Op& op, const float* b, float* out, const int* flags, const float* dots_q)
{
    MgLevel& L = mg->lv[l];
    if (mg->rec_fn && l == mg->rec_level) NN_TRY(mg->rec_fn(mg->rec_user, b));
    if (mg->hook_fn && l == mg->hook_level) {
        // the caller's solver for this level, then hook_sweeps smoothing sweeps
        float* cur = L.x;
        float* oth = L.t;
        NN_TRY(mg->hook_fn(mg->hook_user, b, cur));
        for (int s = 0; s < mg->hook_sweeps; ++s) {
            float* dst = (s == mg->hook_sweeps - 1 && out != cur) ? out : oth;
            NN_TRY((launch_jacobi<V, false>(mg, op, b, cur, dst, flags)));
            oth = cur;
            cur = dst;
        }
        if (cur != out)
            NN_CUDA(mg->ctx, cudaMemcpyAsync(out, cur, sizeof(float) * L.G, cudaMemcpyDeviceToDevice, mg->ctx->stream));
        return NN_OK;
    }
    const bool coarsest = l + 1 == (int)mg->lv.size();
    const int sweeps = coarsest ? mg->coarse_sweeps : mg->nu;
    // pre-smoothing (or the coarsest solve): ping-pong, ending in L.x
    const int after_first = sweeps >= 2 ? sweeps - 2 : sweeps - 1;
    float* cur = (after_first % 2) ? L.t : L.x;
    float* oth = (after_first % 2) ? L.x : L.t;
    if (sweeps >= 2) NN_TRY((launch_pre2<V>(mg, op, b, cur, flags)));
    else NN_TRY(launch_smooth0(mg, op, b, cur, flags));
    for (int s = 0; s < after_first; ++s) {
        NN_TRY((launch_jacobi<V, false>(mg, op, b, cur, oth, flags)));
        std::swap(cur, oth);
    }
    if (coarsest) {
        if (cur != out)
            NN_CUDA(mg->ctx, cudaMemcpyAsync(out, cur, sizeof(float) * L.G, cudaMemcpyDeviceToDevice, mg->ctx->stream));
        return NN_OK;
    }
    MgLevel& C = mg->lv[l + 1];
    if (V == 4 && (op.nx / 2) % 2 == 0) NN_TRY((launch_restrict<2>(mg, op, b, cur, C.b, flags)));
    else NN_TRY((launch_restrict<1>(mg, op, b, cur, C.b, flags)));
    NN_TRY(vcycle(mg, l + 1, C.b, C.x, flags, nullptr));
    {
        const Shape s = shape_for(mg->ctx, L.nx, L.ny * L.nz);
        k_mg_prolong_add<<<s.grid, s.block, 0, mg->ctx->stream>>>(L.nx, L.ny, L.nz, C.x, cur, flags);
        NN_CHECK_LAUNCH(mg->ctx, "k_mg_prolong_add");
    }
    // post-smoothing: nu sweeps, the last one into out (never in place)
    for (int s = 0; s < mg->nu; ++s) {
        const bool last = s == mg->nu - 1;
        float* dst = (last && out != cur) ? out : oth;
        if (last && dots_q) NN_TRY((launch_jacobi<V, true>(mg, op, b, cur, dst, flags, dots_q)));
        else NN_TRY((launch_jacobi<V, false>(mg, op, b, cur, dst, flags)));
        oth = cur;
        cur = dst;
    }
    if (cur != out)
        NN_CUDA(mg->ctx, cudaMemcpyAsync(out, cur, sizeof(float) * L.G, cudaMemcpyDeviceToDevice, mg->ctx->stream));
    return NN_OK;
}

nn_status vcycle(nn_mg* mg, int l, const float* b, float* out, const int* flags, const float* dots_q)
{
    if (l == 0) {
        if (mg->vec0 == 4) return vlevel<4>(mg, 0, mg->op0, b, out, flags, dots_q);
        if (mg->vec0 == 2) return vlevel<2>(mg, 0, mg->op0, b, out, flags, dots_q);
        return vlevel<1>(mg, 0, mg->op0, b, out, flags, dots_q);
    }
    return vlevel<1>(mg, l, mg->lv[l].op(), b, out, flags, nullptr);
}

template <int V>
nn_status enqueue_iteration_v(nn_mg* mg, float* x, int parity)
{
    nn_ctx* ctx = mg->ctx;
    cudaStream_t cs = ctx->stream;
    const MgLevel& L = mg->lv[0];
    const Red red = red_of(mg);
    const dim3 blk = shape_for(ctx, L.nx / V, L.ny * L.nz).block;
    float* p_old = mg->p[parity];
    float* p_new = mg->p[1 - parity];
    k_fcg_ap_dir<V><<<mg->nblocks, blk, 0, cs>>>(mg->op0, mg->z, p_old, p_new, mg->q, red);
    NN_CHECK_LAUNCH(ctx, "k_fcg_ap_dir");
    k_fcg_update<V><<<mg->nblocks, dim3(MG_THREADS), 0, cs>>>(x, mg->r, p_new, mg->q, L.G, red);
    NN_CHECK_LAUNCH(ctx, "k_fcg_update");
    return vcycle(mg, 0, mg->r, mg->z, mg->flags, mg->q);
}

// Two FCG iterations (p ping-pongs back to buffer 0).
nn_status enqueue_iterations(nn_mg* mg, float* x)
{
    for (int parity = 0; parity < 2; ++parity) {
        if (mg->vec0 == 4) NN_TRY(enqueue_iteration_v<4>(mg, x, parity));
        else if (mg->vec0 == 2) NN_TRY(enqueue_iteration_v<2>(mg, x, parity));
        else NN_TRY(enqueue_iteration_v<1>(mg, x, parity));
    }
    return NN_OK;
}

void drop_graph(nn_mg* mg)
{
    if (mg->graph) cudaGraphExecDestroy(mg->graph);
    mg->graph = nullptr;
    mg->graph_x = nullptr;
}

nn_status ensure_graph(nn_mg* mg, float* x)
{
    if (mg->graph && mg->graph_x == x) return NN_OK;
    drop_graph(mg);
    nn_ctx* ctx = mg->ctx;
    cudaStream_t cs = ctx->stream;
    const int64_t launches0 = ctx->launches;
    NN_CUDA(ctx, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    nn_status st = enqueue_iterations(mg, x);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(cs, &g);
    mg->graph_launches = ctx->launches - launches0;
    ctx->launches = launches0;
    if (st != NN_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return nn_cuda_check(ctx, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&mg->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        mg->graph = nullptr;
        return nn_cuda_check(ctx, e, "cudaGraphInstantiate");
    }
    mg->graph_x = x;
    return NN_OK;
}

}  // namespace

extern "C" nn_status nn_mg_destroy(nn_mg* mg)
{
    if (!mg) return NN_OK;
    if (mg->ctx) cudaStreamSynchronize(mg->ctx->stream);
    drop_graph(mg);
    for (MgLevel& L : mg->lv)
        for (float* v : {L.wx, L.wy, L.wz, L.wb, L.diag, L.b, L.x, L.t}) cudaFree(v);
    for (float* v : {mg->r, mg->z, mg->q, mg->p[0], mg->p[1]}) cudaFree(v);
    cudaFree(mg->scal);
    cudaFree(mg->flags);
    cudaFree(mg->partials);
    cudaFree(mg->ticket);
    if (mg->h_flags) cudaFreeHost(mg->h_flags);
    nn_ctx* ctx = mg->ctx;
    delete mg;
    if (ctx) nn_ctx_release(ctx);
    return NN_OK;
}

extern "C" nn_status nn_mg_create(nn_pcg* pc, int levels, nn_mg** out)
{
    if (!pc || !out || levels < 0 || levels > MG_MAX_LEVELS) return NN_ERR_INVALID_ARG;
    *out = nullptr;
    nn_ctx* ctx;
    int nx, ny, nz;
    const float* invd;
    float invd_c;
    const float* D;
    double alpha, beta;
    nn_pcg_info(pc, &ctx, &nx, &ny, &nz, &invd, &invd_c, &D);
    nn_pcg_coefficients(pc, &alpha, &beta);
    if ((int64_t)nx * ny * nz > INT32_MAX / 2)
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_mg_create: grid of more than 2^30 cells");
    int nl = 1;
    {
        int a = nx, b = ny, c = nz;
        while (nl < MG_MAX_LEVELS) {
            if (levels ? nl >= levels : (int64_t)a * b * c <= MG_COARSE_CELLS) break;
            if (a % 2 || b % 2 || c % 2 || a < 4 || b < 4 || c < 4) break;
            a /= 2;
            b /= 2;
            c /= 2;
            ++nl;
        }
        if (levels && nl < levels)
            return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_mg_create: %dx%dx%d does not coarsen to %d levels", nx, ny,
                           nz, levels);
    }
    nn_mg* mg = new nn_mg();
    mg->ctx = ctx;
    nn_ctx_retain(ctx);
    mg->pc = pc;
    mg->op0 = Op0{nx, ny, nz, D, invd, invd_c, (float)alpha, (float)(1.0 + beta)};
    mg->vec0 = nx % NN_MG_VEC == 0 ? NN_MG_VEC : (nx % 2 == 0 ? 2 : 1);
    mg->lv.resize(nl);
    nn_status st = NN_OK;
    float mass = (float)(1.0 + beta);
    for (int l = 0; l < nl && st == NN_OK; ++l) {
        MgLevel& L = mg->lv[l];
        L.nx = nx >> l;
        L.ny = ny >> l;
        L.nz = nz >> l;
        L.G = L.nx * L.ny * L.nz;
        L.mass = mass;
        mass *= 8.0f;
        st = nn_alloc(ctx, &L.x, L.G);
        if (st == NN_OK) st = nn_alloc(ctx, &L.t, L.G);
        if (l == 0) continue;
        if (st == NN_OK) st = nn_alloc(ctx, &L.b, L.G);
        for (float** a : {&L.wx, &L.wy, &L.wz, &L.wb, &L.diag})
            if (st == NN_OK) st = nn_alloc(ctx, a, L.G);
    }
    const int G = mg->lv[0].G;
    for (float** a : {&mg->r, &mg->z, &mg->q, &mg->p[0], &mg->p[1]})
        if (st == NN_OK) st = nn_alloc(ctx, a, G);
    mg->nblocks = std::max(1, std::min((G + MG_THREADS - 1) / MG_THREADS, ctx->num_sms * 8));
    if (st == NN_OK) st = nn_alloc(ctx, &mg->scal, S_COUNT);
    if (st == NN_OK) st = nn_alloc(ctx, &mg->flags, F_COUNT);
    if (st == NN_OK) st = nn_alloc(ctx, &mg->partials, (size_t)2 * std::max(mg->nblocks, ctx->num_sms * 8));
    if (st == NN_OK) st = nn_alloc(ctx, &mg->ticket, 1);
    if (st == NN_OK)
        st = nn_cuda_check(ctx, cudaMallocHost((void**)&mg->h_flags, sizeof(int) * F_COUNT), "cudaMallocHost");
    if (st == NN_OK) st = nn_cuda_check(ctx, nn_zero_async(ctx, mg->ticket, sizeof(unsigned int)), "nn_mg_create");
    if (st == NN_OK) st = nn_cuda_check(ctx, nn_zero_async(ctx, mg->flags, sizeof(int) * F_COUNT), "nn_mg_create");
    // coarse operators
    for (int l = 1; l < nl && st == NN_OK; ++l) {
        MgLevel& L = mg->lv[l];
        const Shape s = shape_for(ctx, L.nx, L.ny * L.nz);
        if (l == 1)
            k_mg_coarsen<Op0><<<s.grid, s.block, 0, ctx->stream>>>(mg->op0, L.wx, L.wy, L.wz, L.wb);
        else
            k_mg_coarsen<OpF><<<s.grid, s.block, 0, ctx->stream>>>(mg->lv[l - 1].op(), L.wx, L.wy, L.wz, L.wb);
        st = nn_cuda_check(ctx, cudaGetLastError(), "k_mg_coarsen");
        if (st != NN_OK) break;
        k_mg_diag<<<s.grid, s.block, 0, ctx->stream>>>(L.nx, L.ny, L.nz, L.wx, L.wy, L.wz, L.wb, L.mass, L.diag);
        st = nn_cuda_check(ctx, cudaGetLastError(), "k_mg_diag");
    }
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "nn_mg_create");
    if (st != NN_OK) {
        nn_mg_destroy(mg);
        return st;
    }
    *out = mg;
    return NN_OK;
}

extern "C" nn_status nn_mg_levels(nn_mg* mg, int* levels)
{
    if (!mg || !levels) return NN_ERR_INVALID_ARG;
    *levels = (int)mg->lv.size();
    return NN_OK;
}

// One V-cycle: z = M r.
extern "C" nn_status nn_mg_apply(nn_mg* mg, const float* d_r, float* d_z)
{
    if (!mg || !d_r || !d_z) return NN_ERR_INVALID_ARG;
    NN_TRY(vcycle(mg, 0, d_r, d_z, nullptr, nullptr));
    return nn_cuda_check(mg->ctx, cudaStreamSynchronize(mg->ctx->stream), "nn_mg_apply");
}

// Flexible CG preconditioned by one V-cycle per iteration (x holds the initial
// guess).
extern "C" nn_status nn_mg_solve(nn_mg* mg, const float* d_b, float* d_x, double rtol, int max_iter, int* iters,
                                 double* relres)
{
    if (!mg || !d_b || !d_x || !(rtol > 0.0) || max_iter < 0) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = mg->ctx;
    cudaStream_t cs = ctx->stream;
    const MgLevel& L = mg->lv[0];
    const double rtol2 = rtol * rtol;
    const Red red = red_of(mg);
    if (!mg->rec_fn) NN_TRY(ensure_graph(mg, d_x));
    k_fcg_set<<<1, 1, 0, cs>>>(mg->scal, mg->flags, rtol2, max_iter);
    NN_CHECK_LAUNCH(ctx, "k_fcg_set");
    const dim3 blk = shape_for(ctx, L.nx / mg->vec0, L.ny * L.nz).block;
    if (mg->vec0 == 4) k_fcg_init<4><<<mg->nblocks, blk, 0, cs>>>(mg->op0, d_b, d_x, mg->r, red);
    else if (mg->vec0 == 2) k_fcg_init<2><<<mg->nblocks, blk, 0, cs>>>(mg->op0, d_b, d_x, mg->r, red);
    else k_fcg_init<1><<<mg->nblocks, blk, 0, cs>>>(mg->op0, d_b, d_x, mg->r, red);
    NN_CHECK_LAUNCH(ctx, "k_fcg_init");
    NN_TRY(vcycle(mg, 0, mg->r, mg->z, mg->flags, nullptr));
    k_fcg_first<<<mg->nblocks, dim3(MG_THREADS), 0, cs>>>(mg->r, mg->z, mg->p[0], L.G, red);
    NN_CHECK_LAUNCH(ctx, "k_fcg_first");
    // graph launches (two iterations each); the first chunk covers the last
    // solve's iteration count.  While recording, the iterations are enqueued
    // directly instead (the recorder copies to a new place each time).
    int launched = 0;
    int chunk = mg->last_iters > 0 ? (mg->last_iters + 1) / 2 : 4;
    while (launched < max_iter) {
        const int k = std::min(chunk, (max_iter - launched + 1) / 2);
        for (int q = 0; q < k; ++q) {
            if (mg->rec_fn) NN_TRY(enqueue_iterations(mg, d_x));
            else NN_CUDA(ctx, cudaGraphLaunch(mg->graph, cs));
        }
        if (!mg->rec_fn) ctx->launches += mg->graph_launches * k;
        launched += 2 * k;
        NN_CUDA(ctx, cudaMemcpyAsync(mg->h_flags, mg->flags, sizeof(int) * F_COUNT, cudaMemcpyDeviceToHost, cs));
        NN_CUDA(ctx, cudaStreamSynchronize(cs));
        if (mg->h_flags[F_DONE]) break;
        chunk = 1;
    }
    NN_CUDA(ctx, cudaMemcpyAsync(mg->h_flags, mg->flags, sizeof(int) * F_COUNT, cudaMemcpyDeviceToHost, cs));
    double sc[S_COUNT];
    NN_CUDA(ctx, nn_copy_sync(ctx, sc, mg->scal, sizeof sc, cudaMemcpyDeviceToHost));
    const int it = mg->h_flags[F_ITERS];
    mg->last_iters = it;
    if (iters) *iters = it;
    const double rel = sc[S_BB] > 0.0 ? std::sqrt(sc[S_RR] / sc[S_BB]) : 0.0;
    if (relres) *relres = rel;
    if (mg->h_flags[F_STATE] == 1) return nn_fail(ctx, NN_ERR_NUMERIC, "multigrid FCG: non-finite residual");
    if (!(sc[S_RR] <= rtol2 * sc[S_BB]))
        return nn_fail(ctx, NN_ERR_NOT_CONVERGED, "multigrid FCG did not reach rtol %g in %d iterations", rtol,
                       max_iter);
    return NN_OK;
}

// ------------------------------------------------ hooks for level solvers --

nn_status nn_mg_set_level_solver(nn_mg* mg, int level, nn_mg_level_fn fn, void* user)
{
    if (!mg || (fn && (level < 1 || level >= (int)mg->lv.size()))) return NN_ERR_INVALID_ARG;
    drop_graph(mg);
    mg->hook_level = fn ? level : -1;
    mg->hook_fn = fn;
    mg->hook_user = user;
    mg->last_iters = 0;
    return NN_OK;
}

nn_status nn_mg_set_level_sweeps(nn_mg* mg, int sweeps)
{
    if (!mg || sweeps < 0) return NN_ERR_INVALID_ARG;
    drop_graph(mg);
    mg->hook_sweeps = sweeps;
    return NN_OK;
}

nn_status nn_mg_set_recorder(nn_mg* mg, int level, nn_mg_record_fn fn, void* user)
{
    if (!mg || (fn && (level < 1 || level >= (int)mg->lv.size()))) return NN_ERR_INVALID_ARG;
    mg->rec_level = fn ? level : -1;
    mg->rec_fn = fn;
    mg->rec_user = user;
    return NN_OK;
}

nn_status nn_mg_level_dims(const nn_mg* mg, int level, int* nx, int* ny, int* nz, const float** diag)
{
    if (!mg || level < 1 || level >= (int)mg->lv.size()) return NN_ERR_INVALID_ARG;
    const MgLevel& L = mg->lv[level];
    *nx = L.nx;
    *ny = L.ny;
    *nz = L.nz;
    *diag = L.diag;
    return NN_OK;
}

nn_status nn_mg_level_cg(nn_mg* mg, int level, const float* d_b, float* d_x, double rtol, int max_iter, int* iters)
{
    if (!mg || !d_b || !d_x || level < 1 || level >= (int)mg->lv.size()) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = mg->ctx;
    cudaStream_t cs = ctx->stream;
    MgLevel& L = mg->lv[level];
    const OpF op = L.op();
    const Red red = red_of(mg);
    const Shape sh = shape_for(ctx, L.nx, L.ny * L.nz);
    // work vectors: the level's own x / t buffers serve as r and p, the
    // next-finer level's t as q (all larger than this level)
    float* r = L.x;
    float* p = L.t;
    float* q = mg->lv[level - 1].t;
    k_lcg_init<<<sh.grid, sh.block, 0, cs>>>(op, d_b, d_x, r, p, red);
    NN_CHECK_LAUNCH(ctx, "k_lcg_init");
    double sc[S_COUNT];
    int it = 0;
    for (; it < max_iter; ++it) {
        NN_CUDA(ctx, nn_copy_sync(ctx, sc, mg->scal, sizeof sc, cudaMemcpyDeviceToHost));
        if (!(sc[S_RR] > rtol * rtol * sc[S_BB])) break;
        k_lcg_ap<<<sh.grid, sh.block, 0, cs>>>(op, p, q, red);
        NN_CHECK_LAUNCH(ctx, "k_lcg_ap");
        k_lcg_update<<<sh.grid, sh.block, 0, cs>>>(op, d_x, r, p, q, red);
        NN_CHECK_LAUNCH(ctx, "k_lcg_update");
        k_lcg_dir<<<sh.grid, sh.block, 0, cs>>>(op, r, p, red);
        NN_CHECK_LAUNCH(ctx, "k_lcg_dir");
    }
    if (iters) *iters = it;
    if (!std::isfinite(sc[S_RR])) return nn_fail(ctx, NN_ERR_NUMERIC, "level CG: non-finite residual");
    return NN_OK;
}
