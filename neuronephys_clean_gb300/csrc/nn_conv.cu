// 3x3x3 convolutions of the learned preconditioner on the tcgen05 tensor
// cores (BF16 operands, FP32 accumulation in tensor memory).
//
// Forward (and input-gradient, with adjoint-packed weights): one CTA of 128
// threads computes a tile of 128 consecutive padded voxels x all COUT output
// channels as an implicit GEMM, M = 128 voxels, N = COUT, K = 27 * CIN.  For
// each of the 9 (dz, dy) pairs the bulk-copy engine stages one window of 130
// voxels per 8-channel block (2,080 contiguous bytes, the layout of
// nn_conv.cuh) and the packed weights of the three dx taps; the three dx taps
// are the same window read at byte offsets 0, 16, 32, which the no-swizzle
// K-major operand layout (8-row x 16-byte core matrices, rows 16 bytes
// apart) allows.  Up to nine stages are in flight at once (all nine when
// they fit in 96 KB, so a small grid pays one copy round trip, not nine); one
// thread issues CIN/16 MMAs (K = 16) per tap, commits them to an mbarrier,
// and the epilogue (bias, ReLU, optional gradient mask, BF16 store with zeros
// on pads) reads the accumulator back with tcgen05.ld.
//
// Weight gradient: for each (dz, dy) pair one GEMM on the tensor cores with
// M = COUT (padded to 128), N = 3 * CIN (the three dx taps), K = voxels, over
// staged gradient tiles and x windows read as MN-major operands (channels
// contiguous; see k_conv3_wgrad).  Persistent CTAs accumulate over many tiles
// in tensor memory and add to the FP32 gradient once.
#include <cuda_bf16.h>

#include "nn_conv.cuh"
#include "nn_ptx.cuh"

// Extra dynamic shared memory per conv CTA (bytes); 0 in normal builds.
#ifndef NN_CONV_SMEM_SLACK
#define NN_CONV_SMEM_SLACK 0
#endif

namespace {
constexpr int TILE = 128;
constexpr int WIN = TILE + 2;
constexpr int WIN_BYTES = WIN * 16;  // 2080
constexpr int CONV_THREADS = 128;
constexpr uint32_t CONV_WAIT_LIMIT = 1u << 22;

template <int CIN, int COUT>
struct ConvCfg {
    static_assert(CIN % 16 == 0 && COUT % 16 == 0 && COUT <= 256, "channel counts");
    static constexpr int G_IN = CIN / 8;
    static constexpr int ACT_BYTES = G_IN * WIN_BYTES;
    static constexpr int W_BYTES = 3 * CIN * COUT * 2;  // the three dx taps of one (dz, dy)
    static constexpr int STAGE_STRIDE = (ACT_BYTES + W_BYTES + 127) / 128 * 128;
    // (dz, dy) stages in flight on small grids: all nine when they fit in
    // 96 KB, else as many as fit (at least two); large grids use two, which
    // leaves room for more CTAs per SM
    static constexpr int STAGES = 96 * 1024 / STAGE_STRIDE >= 9 ? 9 : (96 * 1024 / STAGE_STRIDE < 2 ? 2 : 96 * 1024 / STAGE_STRIDE);
    // grids of at most one tile per SM: as many stages as 200 KB hold
    static constexpr int STAGES_BIG = 200 * 1024 / STAGE_STRIDE >= 9 ? 9 : (200 * 1024 / STAGE_STRIDE < 2 ? 2 : 200 * 1024 / STAGE_STRIDE);
    static constexpr int SMEM = 128 + STAGES_BIG * STAGE_STRIDE + NN_CONV_SMEM_SLACK;  // the most a launch uses
    static int smem(int stages) { return 128 + stages * STAGE_STRIDE + NN_CONV_SMEM_SLACK; }
    static constexpr uint32_t TMEM_COLS = COUT <= 32 ? 32 : (COUT <= 64 ? 64 : (COUT <= 128 ? 128 : 256));
    static_assert(SMEM <= 227 * 1024, "shared memory");
};

struct ConvArgs {
    const uint4* x;
    const unsigned char* w;
    const float* bias;
    const uint4* mask;
    uint4* y;
    float* y32;
    nn_act_geom g;
    int relu;
    int* err;
    int stages;  // (dz, dy) stages in flight, 2 .. ConvCfg::STAGES_BIG
    const double* y32_scale;
    uint4* up;        // (nullable) the result also written, nearest-upsampled, into this finer activation
    nn_act_geom gu;   // its geometry (twice the sides)
};

__device__ __forceinline__ unsigned char* align128(unsigned char* p)
{
    return (unsigned char*)(((uintptr_t)p + 127) & ~(uintptr_t)127);
}

__device__ __forceinline__ void unpack_bf16x8(const uint4& u, float* f)
{
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        f[2 * i] = __uint_as_float(w[i] << 16);
        f[2 * i + 1] = __uint_as_float(w[i] & 0xFFFF0000u);
    }
}

__device__ __forceinline__ uint4 pack_bf16x8(const float* f)
{
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
        w[i] = *reinterpret_cast<const uint32_t*>(&h);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

// padded voxel -> interior coordinates; false for pads
__device__ __forceinline__ bool interior(const nn_act_geom& g, int64_t o, int& z, int& y, int& x)
{
    z = (int)(o / g.P);
    const int64_t rem = o - (int64_t)z * g.P;
    y = (int)(rem / g.R);
    x = (int)(rem - (int64_t)y * g.R);
    return z >= 1 && z <= g.nz && y >= 1 && y <= g.ny && x >= 1 && x <= g.nx;
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(CONV_THREADS) k_conv3(ConvArgs a)
{
    using C = ConvCfg<CIN, COUT>;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* sm = align128(smem_raw);
    const int S = a.stages;
    __shared__ uint64_t full[C::STAGES_BIG], done[C::STAGES_BIG], acc_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int64_t o0 = a.g.o_first + (int64_t)blockIdx.x * TILE;

    if (tid == 0) {
        for (int q = 0; q < S; ++q) {
            nn_mbar_init(&full[q], 1);
            nn_mbar_init(&done[q], 1);
        }
        nn_mbar_init(&acc_bar, 1);
        nn_mbar_fence_init();
        abort_flag = 0;
    }
    if (warp == 0) nn_tmem_alloc(&tmem_slot, C::TMEM_COLS);
    nn_tc_fence_before();
    __syncthreads();
    nn_tc_fence_after();
    const uint32_t tmem = tmem_slot;
    // the kernel before this one has finished with the activations
    nn_grid_dep_wait();

    if (tid == 0) {
        int issued = 0;
        auto issue = [&](int st) {
            const int q = st % S;
            unsigned char* buf = sm + q * C::STAGE_STRIDE;
            const int dz = st / 3 - 1, dy = st % 3 - 1;
            const int64_t start = o0 + dz * a.g.P + dy * a.g.R - 1;
            nn_mbar_expect_tx(&full[q], C::ACT_BYTES + C::W_BYTES);
#pragma unroll
            for (int gi = 0; gi < C::G_IN; ++gi)
                nn_bulk_g2s(buf + gi * WIN_BYTES, a.x + gi * a.g.S + a.g.GD + start, WIN_BYTES, &full[q]);
            nn_bulk_g2s(buf + C::ACT_BYTES, a.w + (size_t)st * C::W_BYTES, C::W_BYTES, &full[q]);
            ++issued;
        };
        for (int st = 0; st < S; ++st) issue(st);
        constexpr uint32_t idesc = nn_umma_idesc_bf16(128, COUT);
        bool ok = true;
        int consumed = 0;
        for (int st = 0; st < 9; ++st) {
            const int b = st % S;
            ok = nn_mbar_wait(&full[b], (st / S) & 1, CONV_WAIT_LIMIT);
            if (!ok) break;
            ++consumed;
            nn_tc_fence_after();
            unsigned char* buf = sm + b * C::STAGE_STRIDE;
            const uint32_t abase = nn_smem_u32(buf), wbase = nn_smem_u32(buf + C::ACT_BYTES);
#pragma unroll
            for (int dx = 0; dx < 3; ++dx)
#pragma unroll
                for (int kc = 0; kc < CIN / 16; ++kc) {
                    const uint64_t ad = nn_umma_sdesc(abase + 2 * kc * WIN_BYTES + dx * 16, WIN_BYTES, 128);
                    const uint64_t bd = nn_umma_sdesc(wbase + (dx * (CIN / 16) + kc) * 2 * COUT * 16, COUT * 16, 128);
                    nn_umma_bf16(tmem, ad, bd, idesc, (st | dx | kc) != 0);
                }
            nn_umma_commit(&done[b]);
            if (st + S < 9) {
                ok = nn_mbar_wait(&done[b], (st / S) & 1, CONV_WAIT_LIMIT);
                if (!ok) break;
                issue(st + S);
            }
        }
        nn_umma_commit(&acc_bar);
        if (!ok) {
            abort_flag = 1;
            // let copies already in flight land before the CTA leaves
            for (int st = consumed; st < issued; ++st) nn_mbar_wait(&full[st % S], (st / S) & 1, CONV_WAIT_LIMIT);
        }
    }
    // lanes 1-31 of warp 0 wait here for lane 0's issue loop (spinning on
    // the mbarrier beside it would stall that loop at every wait); one thread
    // then waits for the accumulator and the block barrier releases the rest,
    // whose polls would otherwise take issue slots from the other CTAs
    __syncwarp();
    if (tid == 0 && !nn_mbar_wait(&acc_bar, 0, CONV_WAIT_LIMIT)) abort_flag = 1;
    __syncthreads();
    nn_tc_fence_after();
    if (abort_flag) {  // block-uniform: the TMEM loads below are warp-collective
        if (tid == 0) atomicExch(a.err, 1);
    } else {
        const int64_t o = o0 + tid;  // TMEM lane == tile row == voxel
        int z, y, x;
        const bool in = interior(a.g, o, z, y, x);
        float v[COUT];
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) nn_tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + c0, v + c0);
#pragma unroll
        for (int gb = 0; gb < COUT / 8; ++gb) {
            float t[8], mk[8];
            if (a.mask) unpack_bf16x8(a.mask[gb * a.g.S + a.g.GD + o], mk);
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                float q = v[gb * 8 + i] + (a.bias ? a.bias[gb * 8 + i] : 0.0f);
                if (a.relu) q = fmaxf(q, 0.0f);
                if (a.mask && !(mk[i] > 0.0f)) q = 0.0f;
                t[i] = in ? q : 0.0f;
            }
            const uint4 pk = pack_bf16x8(t);
            a.y[gb * a.g.S + a.g.GD + o] = pk;
            if (a.up && in) {
                // the eight children of interior voxel (z, y, x) (1-based) in the finer grid
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    const int64_t fz = 2 * (z - 1) + (c >> 2) + 1, fy = 2 * (y - 1) + ((c >> 1) & 1) + 1,
                                  fx = 2 * (x - 1) + (c & 1) + 1;
                    a.up[gb * a.gu.S + a.gu.GD + fz * a.gu.P + fy * a.gu.R + fx] = pk;
                }
            }
            if (gb == 0 && a.y32 && in)
                a.y32[((int64_t)(z - 1) * a.g.ny + (y - 1)) * a.g.nx + (x - 1)] =
                    a.y32_scale ? t[0] * (float)a.y32_scale[0] : t[0];
        }
    }
    nn_tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        nn_tc_fence_after();
        nn_tmem_dealloc(tmem, C::TMEM_COLS);
    }
}

// ------------------------------------------------------------- wgrad --

// dW[(dz, dy, dx)][ci][co] += sum over voxels o of x(o + shift)[ci] gy(o)[co]:
// per (dz, dy) one GEMM D (M x N) = A (M x K) B^T for all three dx taps, with
// M = 128 rows (TMEM lane = output channel; rows past COUT are discarded),
// N = 3 * CIN (column dx * CIN + ci), K = the voxels of a tile.  A is the
// staged gradient tile; both operands are read MN-major: 16 bytes hold 8
// channels of one voxel, so a core matrix is 8 consecutive voxels (128
// contiguous bytes).  For narrow inputs (CIN <= 32) B is the x window staged
// three times, shifted by dx voxels, so that one MMA per K step covers the
// three taps; wider inputs stage the 130-voxel window once and issue one MMA
// per tap (N = CIN), reading it at byte offsets 0, 16, 32 (fewer bytes per
// slot, more CTAs per SM).  The rows of A past COUT read whatever in-bounds
// shared memory follows (their results are never used).  The accumulator covers all of the CTA's tiles;
// STAGES slots double-buffer the bulk copies against the MMAs, and the
// epilogue adds D to the FP32 gradient once.
constexpr int WG_THREADS = 128;
constexpr int WG_MP = 128;                             // M
constexpr int WG_BLOCK = TILE * 16;                    // one 8-channel block of a tile (2,048 bytes)
constexpr int WG_A_SPAN = (WG_MP / 8) * WG_BLOCK;      // bytes the 128 rows of A address

template <int CIN, int COUT>
struct WgCfg {
    static constexpr bool MERGE = CIN <= 32;                    // the three taps in one MMA
    static constexpr int N = 3 * CIN;
    static constexpr int NSPLIT = MERGE ? 1 : 3;                // MMAs per K step
    static constexpr int NM = N / NSPLIT;                       // N of one MMA
    static constexpr int B_BSTRIDE = MERGE ? WG_BLOCK : WIN_BYTES;  // between 8-channel blocks of B
    static constexpr int A_BYTES = (COUT / 8) * WG_BLOCK;       // gradient tile
    static constexpr int B_BYTES = MERGE ? 3 * (CIN / 8) * WG_BLOCK : (CIN / 8) * WIN_BYTES;  // x
    static constexpr int SLOT = A_BYTES + B_BYTES;
    static constexpr int TAIL = WG_A_SPAN > SLOT ? WG_A_SPAN - SLOT : 0;  // A rows of the last slot past it
    static constexpr int STAGES = 2 * SLOT + TAIL <= 150 * 1024 && 3 * SLOT + TAIL <= 150 * 1024 ? 3 : 2;
    static constexpr int SMEM = 128 + STAGES * SLOT + TAIL;
    static constexpr uint32_t TMEM_COLS = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : N <= 256 ? 256 : 512;
    static_assert(CIN % 8 == 0 && COUT % 8 == 0 && COUT <= WG_MP && N <= 512, "channel counts");
    static_assert(NM % 16 == 0 && NM <= 256 && N % NSPLIT == 0, "MMA shape");
    static_assert(SMEM <= 227 * 1024, "shared memory");
};

// blockIdx.y = (dz, dy); tiles blockIdx.x, blockIdx.x + gridDim.x, ...
template <int CIN, int COUT>
__global__ void __launch_bounds__(WG_THREADS) k_conv3_wgrad(const uint4* __restrict__ x, const uint4* __restrict__ gy,
                                                            nn_act_geom g, float* dw, int* err)
{
    using C = WgCfg<CIN, COUT>;
    constexpr int S = C::STAGES;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* sm = align128(smem_raw);
    __shared__ uint64_t full[S], done[S], acc_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int st9 = blockIdx.y, dz = st9 / 3 - 1, dy = st9 % 3 - 1;
    const int64_t ntiles =
        (int64_t)blockIdx.x < g.tiles ? (g.tiles - 1 - (int64_t)blockIdx.x) / gridDim.x + 1 : 0;
    if (tid == 0) {
        for (int q = 0; q < S; ++q) {
            nn_mbar_init(&full[q], 1);
            nn_mbar_init(&done[q], 1);
        }
        nn_mbar_init(&acc_bar, 1);
        nn_mbar_fence_init();
        abort_flag = 0;
    }
    if (warp == 0) nn_tmem_alloc(&tmem_slot, C::TMEM_COLS);
    nn_tc_fence_before();
    __syncthreads();
    nn_tc_fence_after();
    const uint32_t tmem = tmem_slot;

    if (tid == 0) {
        int64_t issued = 0, consumed = 0;
        // tile j into slot j % S: the gradient blocks, then x at shifts dx = 0, 1, 2
        auto issue = [&](int64_t j) {
            const int q = (int)(j % S);
            const int64_t o0 = g.o_first + (blockIdx.x + j * gridDim.x) * TILE;
            const int64_t start = o0 + dz * g.P + dy * g.R - 1;
            unsigned char* buf = sm + q * C::SLOT;
            nn_mbar_expect_tx(&full[q], C::A_BYTES + C::B_BYTES);
#pragma unroll
            for (int ob = 0; ob < COUT / 8; ++ob)
                nn_bulk_g2s(buf + ob * WG_BLOCK, gy + ob * g.S + g.GD + o0, WG_BLOCK, &full[q]);
            if (C::MERGE) {
#pragma unroll
                for (int dx = 0; dx < 3; ++dx)
#pragma unroll
                    for (int cb = 0; cb < CIN / 8; ++cb)
                        nn_bulk_g2s(buf + C::A_BYTES + (dx * (CIN / 8) + cb) * WG_BLOCK,
                                    x + cb * g.S + g.GD + start + dx, WG_BLOCK, &full[q]);
            } else {
#pragma unroll
                for (int cb = 0; cb < CIN / 8; ++cb)
                    nn_bulk_g2s(buf + C::A_BYTES + cb * WIN_BYTES, x + cb * g.S + g.GD + start, WIN_BYTES, &full[q]);
            }
            ++issued;
        };
        // A and B both MN-major (bits 15, 16 of the instruction descriptor)
        constexpr uint32_t idesc = nn_umma_idesc_bf16(WG_MP, C::NM) | (1u << 15) | (1u << 16);
        bool ok = true;
        for (int64_t j = 0; j < S && j < ntiles; ++j) issue(j);
        for (int64_t j = 0; j < ntiles; ++j) {
            const int q = (int)(j % S);
            ok = nn_mbar_wait(&full[q], (uint32_t)((j / S) & 1), CONV_WAIT_LIMIT);
            if (!ok) break;
            ++consumed;
            nn_tc_fence_after();
            const uint32_t abase = nn_smem_u32(sm + q * C::SLOT), bbase = abase + C::A_BYTES;
#pragma unroll
            for (int kk = 0; kk < TILE / 16; ++kk)
#pragma unroll
                for (int h = 0; h < C::NSPLIT; ++h) {
                    // MN-major no-swizzle: LBO = next 8 voxels (K), SBO = next 8 channels (M / N)
                    // (merged: B starts at the first block of all taps; else tap h
                    // is the window read h voxels further on)
                    const uint32_t boff = C::MERGE ? kk * 256 : (kk * 16 + h) * 16;
                    const uint64_t ad = nn_umma_sdesc(abase + kk * 256, 128, WG_BLOCK);
                    const uint64_t bd = nn_umma_sdesc(bbase + boff, 128, C::B_BSTRIDE);
                    nn_umma_bf16(tmem + h * C::NM, ad, bd, idesc, (j | kk) != 0);
                }
            nn_umma_commit(&done[q]);
            if (j + S < ntiles) {
                ok = nn_mbar_wait(&done[q], (uint32_t)((j / S) & 1), CONV_WAIT_LIMIT);
                if (!ok) break;
                issue(j + S);
            }
        }
        nn_umma_commit(&acc_bar);
        if (!ok) {
            abort_flag = 1;
            // let copies already in flight land before the CTA leaves
            for (int64_t j = consumed; j < issued; ++j)
                nn_mbar_wait(&full[j % S], (uint32_t)((j / S) & 1), CONV_WAIT_LIMIT);
        }
    }
    // lanes 1-31 of warp 0 wait here for lane 0's issue loop (spinning on
    // the mbarrier beside it would stall that loop at every wait); one thread
    // then waits for the accumulator and the block barrier releases the rest,
    // whose polls would otherwise take issue slots from the other CTAs
    __syncwarp();
    if (tid == 0 && !nn_mbar_wait(&acc_bar, 0, CONV_WAIT_LIMIT)) abort_flag = 1;
    __syncthreads();
    nn_tc_fence_after();
    if (abort_flag) {  // block-uniform: the TMEM loads below are warp-collective
        if (tid == 0) atomicExch(err, 1);
    } else if (ntiles > 0) {
        const int co = tid;  // TMEM lane == row == output channel
#pragma unroll
        for (int c0 = 0; c0 < C::N; c0 += 16) {
            float v[16];
            nn_tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + c0, v);
            if (co < COUT) {
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const int n = c0 + i, dx = n / CIN, ci = n - dx * CIN;
                    atomicAdd(dw + ((size_t)(st9 * 3 + dx) * CIN + ci) * COUT + co, v[i]);
                }
            }
        }
    }
    nn_tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        nn_tc_fence_after();
        nn_tmem_dealloc(tmem, C::TMEM_COLS);
    }
}

// db[c] += sum over voxels of gy(o, c)
__global__ void k_bias_grad(const uint4* __restrict__ gy, nn_act_geom g, int cout, float* db)
{
    __shared__ float part[64][8];
    const int gb = blockIdx.y;
    float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t o = g.o_first + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o <= g.o_last;
         o += (int64_t)gridDim.x * blockDim.x) {
        float v[8];
        unpack_bf16x8(gy[gb * g.S + g.GD + o], v);
#pragma unroll
        for (int i = 0; i < 8; ++i) s[i] += v[i];
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        float t = s[i];
        for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
        if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5][i] = t;
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        float t = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w][threadIdx.x];
        atomicAdd(&db[gb * 8 + threadIdx.x], t);
    }
    (void)cout;
}

// packed[(st, dx, kc, half, co, ci8)] from w[27][cin][cout] (or its adjoint)
__global__ void k_pack_weights(const float* w, int cin, int cout, int flip, __nv_bfloat16* out)
{
    // packed operator shape: ci_p x co_p
    const int ci_p = flip ? cout : cin, co_p = flip ? cin : cout;
    const int64_t total = 27LL * ci_p * co_p;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int tap = (int)(e / ((int64_t)ci_p * co_p));
        const int rem = (int)(e - (int64_t)tap * ci_p * co_p);
        const int ci = rem / co_p, co = rem - (rem / co_p) * co_p;
        const int st = tap / 3, dx = tap % 3;
        const float v = flip ? w[((size_t)(26 - tap) * cin + co) * cout + ci] : w[((size_t)tap * cin + ci) * cout + co];
        const size_t blk = (size_t)st * 3 * ci_p * co_p;
        const size_t idx = blk + (((size_t)(dx * (ci_p / 16) + ci / 16) * 2 + (ci % 16) / 8) * co_p + co) * 8 + ci % 8;
        out[idx] = __float2bfloat16_rn(v);
    }
}

__global__ void k_act_pack(const float* dense, nn_act_geom g, int C, uint4* act)
{
    const int64_t G = (int64_t)g.nz * g.ny * g.nx;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < G * (C / 8); e += (int64_t)gridDim.x * blockDim.x) {
        const int gb = (int)(e / G);
        const int64_t c = e - gb * G;
        const int x = (int)(c % g.nx), y = (int)((c / g.nx) % g.ny), z = (int)(c / ((int64_t)g.nx * g.ny));
        float f[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) f[i] = dense[(size_t)(gb * 8 + i) * G + c];
        const int64_t o = (int64_t)(z + 1) * g.P + (int64_t)(y + 1) * g.R + x + 1;
        act[gb * g.S + g.GD + o] = pack_bf16x8(f);
    }
}

__global__ void k_act_unpack(const uint4* act, nn_act_geom g, int C, float* dense)
{
    const int64_t G = (int64_t)g.nz * g.ny * g.nx;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < G * (C / 8); e += (int64_t)gridDim.x * blockDim.x) {
        const int gb = (int)(e / G);
        const int64_t c = e - gb * G;
        const int x = (int)(c % g.nx), y = (int)((c / g.nx) % g.ny), z = (int)(c / ((int64_t)g.nx * g.ny));
        const int64_t o = (int64_t)(z + 1) * g.P + (int64_t)(y + 1) * g.R + x + 1;
        float f[8];
        unpack_bf16x8(act[gb * g.S + g.GD + o], f);
#pragma unroll
        for (int i = 0; i < 8; ++i) dense[(size_t)(gb * 8 + i) * G + c] = f[i];
    }
}

// --------------------------------------------------------- dispatch --

template <int CIN, int COUT>
nn_status launch_fwd(nn_ctx* ctx, const ConvArgs& a)
{
    using C = ConvCfg<CIN, COUT>;
    static bool attr_set = false;  // per process; kernels are per device but the attribute is a function property
    if (!attr_set) {
        NN_CUDA(ctx, cudaFuncSetAttribute(k_conv3<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
        attr_set = true;
    }
    // small grids (at most four tiles per SM) are latency-bound: all their
    // stages in flight; large ones keep two and more CTAs per SM
    ConvArgs b = a;
    b.stages = a.g.tiles <= (int64_t)ctx->num_sms ? C::STAGES_BIG
                                                  : (a.g.tiles <= (int64_t)ctx->num_sms * 4 ? C::STAGES : 2);
    NN_CUDA(ctx, nn_launch_pdl(k_conv3<CIN, COUT>, dim3((unsigned)a.g.tiles), dim3(CONV_THREADS),
                               (size_t)C::smem(b.stages), ctx->stream, b));
    ctx->launches++;
    return NN_OK;
}

template <int CIN, int COUT>
nn_status launch_wgrad(nn_ctx* ctx, const nn_act_geom& g, const void* x, const void* gy, float* dw, int* err)
{
    using C = WgCfg<CIN, COUT>;
    static int per_sm = 0;  // resident CTAs per SM (per process, like the attribute)
    if (!per_sm) {
        NN_CUDA(ctx, cudaFuncSetAttribute(k_conv3_wgrad<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          C::SMEM));
        NN_CUDA(ctx, cudaFuncSetAttribute(k_conv3_wgrad<CIN, COUT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                          100));
        // CTAs that fit an SM's shared memory (1 KB reserved per CTA) and its
        // 512 tensor-memory columns; more would only wait for a slot
        int smem_sm = 0;
        NN_CUDA(ctx, cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device));
        per_sm = std::max(1, std::min(smem_sm / (C::SMEM + 1024), (int)(512 / C::TMEM_COLS)));
    }
    // one wave of persistent CTAs over the 9 (dz, dy) pairs
    const int64_t per_y = std::max<int64_t>(1, std::min<int64_t>(g.tiles, ((int64_t)ctx->num_sms * per_sm) / 9));
    dim3 grid((unsigned)per_y, 9);
    k_conv3_wgrad<CIN, COUT>
        <<<grid, WG_THREADS, C::SMEM, ctx->stream>>>((const uint4*)x, (const uint4*)gy, g, dw, err);
    NN_CHECK_LAUNCH(ctx, "k_conv3_wgrad");
    return NN_OK;
}

// The layer shapes of the 3-level, 16-base U-Net, forward and adjoint.
#define NN_CONV_SHAPES(X) \
    X(16, 16) X(16, 32) X(32, 32) X(32, 64) X(64, 64) X(96, 32) X(48, 16) X(32, 16) X(64, 32) X(32, 96) X(16, 48)
}  // namespace

bool nn_conv_supported(int cin, int cout)
{
#define NN_X(ci, co) if (cin == ci && cout == co) return true;
    NN_CONV_SHAPES(NN_X)
#undef NN_X
    return false;
}

size_t nn_conv_packed_weight_bytes(int cin, int cout) { return (size_t)27 * cin * cout * 2; }

nn_status nn_conv_forward(nn_ctx* ctx, const nn_act_geom& g, int cin, int cout, const void* x, const void* wpacked,
                          const float* bias, int relu, const void* mask, void* y, float* y32, int* err,
                          const double* y32_scale, void* up, const nn_act_geom* gup)
{
    ConvArgs a;
    a.y32_scale = y32_scale;
    a.up = (uint4*)up;
    if (up && gup) a.gu = *gup;
    a.x = (const uint4*)x;
    a.w = (const unsigned char*)wpacked;
    a.bias = bias;
    a.mask = (const uint4*)mask;
    a.y = (uint4*)y;
    a.y32 = y32;
    a.g = g;
    a.relu = relu;
    a.err = err;
    if (g.tiles <= 0) return NN_OK;
#define NN_X(ci, co) \
    if (cin == ci && cout == co) return launch_fwd<ci, co>(ctx, a);
    NN_CONV_SHAPES(NN_X)
#undef NN_X
    return nn_fail(ctx, NN_ERR_UNSUPPORTED, "conv3d %d -> %d channels is not instantiated", cin, cout);
}

nn_status nn_conv_wgrad(nn_ctx* ctx, const nn_act_geom& g, int cin, int cout, const void* x, const void* gy,
                        float* dw, float* db, int* err)
{
    if (g.tiles <= 0) return NN_OK;
    nn_status st = NN_ERR_UNSUPPORTED;
#define NN_X(ci, co) \
    if (st == NN_ERR_UNSUPPORTED && cin == ci && cout == co) st = launch_wgrad<ci, co>(ctx, g, x, gy, dw, err);
    NN_CONV_SHAPES(NN_X)
#undef NN_X
    if (st == NN_ERR_UNSUPPORTED) return nn_fail(ctx, st, "conv3d wgrad %d -> %d is not instantiated", cin, cout);
    if (st != NN_OK) return st;
    if (db) {
        dim3 grid((unsigned)std::min<int64_t>(g.tiles, (int64_t)ctx->num_sms * 4), cout / 8);
        k_bias_grad<<<grid, 256, 0, ctx->stream>>>((const uint4*)gy, g, cout, db);
        NN_CHECK_LAUNCH(ctx, "k_bias_grad");
    }
    return NN_OK;
}

nn_status nn_conv_pack(nn_ctx* ctx, int cin, int cout, const float* w, int flip, void* packed)
{
    const int64_t total = 27LL * cin * cout;
    k_pack_weights<<<nn_grid_for(ctx, total, 256, 4), 256, 0, ctx->stream>>>(w, cin, cout, flip,
                                                                             (__nv_bfloat16*)packed);
    NN_CHECK_LAUNCH(ctx, "k_pack_weights");
    return NN_OK;
}

nn_status nn_act_pack_dense(nn_ctx* ctx, const nn_act_geom& g, int C, const float* dense, void* act)
{
    const int64_t G = (int64_t)g.nz * g.ny * g.nx * (C / 8);
    k_act_pack<<<nn_grid_for(ctx, G, 256), 256, 0, ctx->stream>>>(dense, g, C, (uint4*)act);
    NN_CHECK_LAUNCH(ctx, "k_act_pack");
    return NN_OK;
}

nn_status nn_act_unpack_dense(nn_ctx* ctx, const nn_act_geom& g, int C, const void* act, float* dense)
{
    const int64_t G = (int64_t)g.nz * g.ny * g.nx * (C / 8);
    k_act_unpack<<<nn_grid_for(ctx, G, 256), 256, 0, ctx->stream>>>((const uint4*)act, g, C, dense);
    NN_CHECK_LAUNCH(ctx, "k_act_unpack");
    return NN_OK;
}

// ------------------------------------------------------------- C ABI --

extern "C" nn_status nn_act_layout(int nz, int ny, int nx, int channels, int64_t* block_stride, int64_t* guard,
                                   int64_t* bytes)
{
    if (nz < 1 || ny < 1 || nx < 1 || channels < 8 || channels % 8) return NN_ERR_INVALID_ARG;
    const nn_act_geom g = nn_act_geometry(nz, ny, nx);
    if (block_stride) *block_stride = g.S;
    if (guard) *guard = g.GD;
    if (bytes) *bytes = (int64_t)nn_act_bytes(g, channels);
    return NN_OK;
}

extern "C" nn_status nn_act_pack(nn_ctx* ctx, int nz, int ny, int nx, int channels, const float* d_dense, void* d_act)
{
    if (!ctx || !d_dense || !d_act || channels % 8 || channels < 8) return NN_ERR_INVALID_ARG;
    return nn_act_pack_dense(ctx, nn_act_geometry(nz, ny, nx), channels, d_dense, d_act);
}

extern "C" nn_status nn_act_unpack(nn_ctx* ctx, int nz, int ny, int nx, int channels, const void* d_act, float* d_dense)
{
    if (!ctx || !d_dense || !d_act || channels % 8 || channels < 8) return NN_ERR_INVALID_ARG;
    return nn_act_unpack_dense(ctx, nn_act_geometry(nz, ny, nx), channels, d_act, d_dense);
}

extern "C" nn_status nn_conv3d_pack_weights(nn_ctx* ctx, int cin, int cout, const float* d_w, int adjoint,
                                            void* d_packed)
{
    if (!ctx || !d_w || !d_packed) return NN_ERR_INVALID_ARG;
    if (!(adjoint ? nn_conv_supported(cout, cin) : nn_conv_supported(cin, cout))) return NN_ERR_UNSUPPORTED;
    return nn_conv_pack(ctx, cin, cout, d_w, adjoint, d_packed);
}

extern "C" nn_status nn_conv3d_forward(nn_ctx* ctx, int nz, int ny, int nx, int cin, int cout, const void* d_x,
                                       const void* d_wpacked, const float* d_bias, int relu, const void* d_mask,
                                       void* d_y, float* d_y32)
{
    if (!ctx || !d_x || !d_wpacked || !d_y || nz < 1 || ny < 1 || nx < 1) return NN_ERR_INVALID_ARG;
    if (!nn_conv_supported(cin, cout)) return nn_fail(ctx, NN_ERR_UNSUPPORTED, "conv3d %d -> %d", cin, cout);
    int* err = nullptr;
    NN_TRY(nn_alloc(ctx, &err, 1));
    nn_status st = nn_cuda_check(ctx, cudaMemsetAsync(err, 0, sizeof(int), ctx->stream), "memset");
    if (st == NN_OK)
        st = nn_conv_forward(ctx, nn_act_geometry(nz, ny, nx), cin, cout, d_x, d_wpacked, d_bias, relu, d_mask, d_y,
                             d_y32, err);
    int h_err = 0;
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost,
                                                             ctx->stream), "memcpy");
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "conv3d");
    nn_release(err);
    if (st == NN_OK && h_err) st = nn_fail(ctx, NN_ERR_TIMEOUT, "k_conv3: a pipeline wait timed out");
    return st;
}

extern "C" nn_status nn_conv3d_wgrad(nn_ctx* ctx, int nz, int ny, int nx, int cin, int cout, const void* d_x,
                                     const void* d_gy, float* d_dw, float* d_db)
{
    if (!ctx || !d_x || !d_gy || !d_dw) return NN_ERR_INVALID_ARG;
    if (!nn_conv_supported(cin, cout)) return nn_fail(ctx, NN_ERR_UNSUPPORTED, "conv3d wgrad %d -> %d", cin, cout);
    int* err = nullptr;
    NN_TRY(nn_alloc(ctx, &err, 1));
    nn_status st = nn_cuda_check(ctx, cudaMemsetAsync(err, 0, sizeof(int), ctx->stream), "memset");
    if (st == NN_OK) st = nn_conv_wgrad(ctx, nn_act_geometry(nz, ny, nx), cin, cout, d_x, d_gy, d_dw, d_db, err);
    int h_err = 0;
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost,
                                                             ctx->stream), "memcpy");
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "conv3d wgrad");
    nn_release(err);
    if (st == NN_OK && h_err) st = nn_fail(ctx, NN_ERR_TIMEOUT, "k_conv3_wgrad: a pipeline wait timed out");
    return st;
}
