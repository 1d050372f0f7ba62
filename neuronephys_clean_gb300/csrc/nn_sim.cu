// GB300 simulation step: RK4 Hodgkin-Huxley over SoA state, spike compaction
// fused into the neuron update, delayed weighted spike delivery (push scatter
// with red.global or deterministic pull gather over the CSC transpose) into an
// integer-delay ring buffer, and the paracrine field (spike deposit, 7-point
// backward-Euler Jacobi-PCG every `timescale` steps, gather to neurons).
//
// The step loop this replaces is _RunAndPrintSimulation's body
// (src/main.cu:166-181): coupling -> paracrine -> ephys, with a host
// synchronisation after every launch and the firing count read back every step.
// Here one step is two kernels with no host interaction:
//   k_hh_step      : ring slot t%D -> (ge, gi), RK4 with noise, spike test,
//                    warp-aggregated compaction, spike bitmap, voxel deposit
//   k_deliver_*    : spikes of step t -> ring slots (t+d)%D (push) or the
//                    whole input of step t+1 (pull); the last block to finish
//                    advances the device step counter.
// Periods of steps are captured once into a CUDA graph and replayed.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "nn_hh.cuh"
#include "nn_internal.cuh"
#include "nn_ptx.cuh"
#include "nn_step.cuh"

struct nn_pcg;
nn_status nn_pcg_run(nn_pcg* pc, const float* d_b, float* d_x, double rtol, int max_iter, int* iters, double* relres,
                     int* converged);

struct nn_sim {
    nn_ctx* ctx = nullptr;
    nn_sim_config cfg{};
    int n = 0, n_pad = 0, D = 0, words = 0;
    int npt = 2, tpb = 128;
    // neuron state (n_pad floats each)
    float* f[NN_F_COUNT] = {};
    float2* ring = nullptr;        // D * n_pad
    uint32_t* bitmap = nullptr;    // D * words (pull delivery)
    int* list = nullptr;           // 2 * n_pad
    int* counts = nullptr;         // [0], [1]: spikes of the step with that parity
    unsigned long long* step = nullptr;     // device step counter
    unsigned long long* total = nullptr;    // spikes so far
    unsigned long long* rcount = nullptr;   // raster entries written
    int2* raster = nullptr;        // (step, neuron)
    int* err = nullptr;
    uint8_t* is_inh = nullptr;
    // network
    int64_t nnz = 0;
    int64_t* row_ptr = nullptr;
    int32_t* col = nullptr;
    float* weight = nullptr;
    uint8_t* delay = nullptr;
    int64_t* col_ptr = nullptr;    // CSC
    uint32_t* csc_src = nullptr;   // source | inhibitory << 31
    float* csc_w = nullptr;
    uint8_t* csc_d = nullptr;
    // chunked CSC of the shared-memory pull (null when the network does not
    // qualify): entries ordered by (column block, delay, source bucket), cut
    // into chunks (see k_deliver_pull_sliced)
    int4* dsl_chunk = nullptr;     // {first entry, end entry, first bitmap word, words << 8 | delay}
    int32_t* dsl_cptr = nullptr;   // [block][j]: first chunk of the block with delay > j (j = 0: first chunk)
    uint32_t* dsl_ent = nullptr;   // entry words, chunk by chunk (each padded to a multiple of four)
    float* dsl_w = nullptr;        // their weights
    uint2* dsl_hits = nullptr;     // per block, from its first entry: the step's hits {entry word, weight bits}
    int dsl_cols = 0;              // columns per block of the sliced pull kernel
    int dsl_ring = 0;              // bitmap slots in shared memory
    int dsl_slotw = 0;             // words per slot
    int dsl_cmax = 0;              // most chunks of one block
    int dsl_dmax = 0;              // longest delay of the layout
    // paracrine
    int grid = 0;
    int64_t G = 0;
    int32_t* vox = nullptr;
    float* src = nullptr;
    float* u = nullptr;
    float* u_prev = nullptr;       // previous solve's solution (initial-guess extrapolation)
    bool have_prev = false;
    float* b = nullptr;
    nn_pcg* pcg = nullptr;
    // batch of independent networks: instance b owns neurons inst_off[b] ..
    // inst_off[b+1]-1 and (with a field) its own cubic grid of side inst_grid[b]
    int n_inst = 0;
    std::vector<int> h_inst_off, h_inst_grid;
    int* inst_off = nullptr;       // device [n_inst + 1]
    int* inst_grid = nullptr;      // device [n_inst]
    int64_t* inst_goff = nullptr;  // device [n_inst + 1] cell offsets
    nn_bpcg* bpcg = nullptr;
    std::vector<int> inst_iters;
    // overlapped field solve: with no feedback of the field into the neurons
    // (g_par == 0) a period's solve runs on its own stream while the next
    // period's steps run; the main stream waits for it only before the next
    // right-hand side is formed
    cudaStream_t par_stream = nullptr;
    cudaEvent_t ev_rhs = nullptr, ev_solved = nullptr;
    bool solve_pending = false;
    int iter_estimate = 64;
    nn_solve_stats stats{};
    // fused electrode recording (nn_sim_set_electrodes)
    uint2* el_group = nullptr;     // per 32-neuron group: member bits, members before it
    float* el_val = nullptr;       // [cap][members] potentials
    uint8_t* el_spk = nullptr;     // [cap][members] spike flags
    int el_every = 0, el_cap = 0, el_members = 0;
    int64_t el_first = 0;          // step of the first sample
    std::vector<int> el_roff, el_rpos;  // regions as lists of member positions
    // automatic delivery (NN_DELIVERY_AUTO): the mode of the periods being
    // enqueued (0 push, 1 pull), the ring rows' modes on the device, and the
    // spike totals read back after each period (pinned, asynchronous)
    int* rowflag = nullptr;        // [D]
    int cur_mode = 0;
    cudaGraphExec_t graph_pull = nullptr;
    static constexpr int TOT_Q = 4;
    unsigned long long* h_tot = nullptr;  // pinned [TOT_Q]
    cudaEvent_t ev_tot[TOT_Q] = {};
    int64_t tot_step[TOT_Q] = {};
    int tot_head = 0, tot_pending = 0;
    unsigned long long base_tot = 0;
    int64_t base_step = -1;        // step of base_tot (-1: none yet)
    float last_rate = -1.0f;       // spikes per neuron and step of the latest measured period
    std::vector<int8_t> mode_log;
    std::vector<float> rate_log;
    // host mirrors
    int64_t host_step = 0;
    bool gna_set = false;  // per-neuron gNa scale given (else the kernel skips the load)
    // graph of one period
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    // kernel timing: events before the neuron update, between it and the
    // delivery, and after the delivery, one triple per step of a period
    bool timing = false;
    std::vector<cudaEvent_t> ev_a, ev_b, ev_c;
    std::vector<char> ev_valid;
};

void nn_pcg_set_timing(nn_pcg* pc, bool on);
void nn_pcg_last_timing(const nn_pcg* pc, float* ms, int* iters);


namespace {

constexpr int DELIV_THREADS = 256;

// Advance the period's first step once all its launches are enqueued before it.
__global__ void k_advance(unsigned long long* base, int steps) { *base += (unsigned long long)steps; }

struct PullArgs {
    const int64_t* col_ptr;
    const uint32_t* csc_src;
    const float* csc_w;
    const uint8_t* csc_d;
    const uint32_t* bitmap;
    float* ring;
    const unsigned long long* base;
    int q;
    int n, n_pad, D, words;
    const int4* dsl_chunk;
    const int32_t* dsl_cptr;
    const uint32_t* dsl_ent;
    const float* dsl_w;
    uint2* dsl_hits;
    int dsl_cols, dsl_ring, dsl_slotw, dsl_cmax, dsl_dmax;
    // automatic delivery: only ring rows with rowflag set hold pull spikes
    // (the others were pushed), and the gather adds to the ring slot, which
    // pushed spikes may already have reached (null / 0: every row, overwrite)
    const int* rowflag;
    int add;
    int* err;
};

// Pull: a warp per postsynaptic neuron sums its CSC column against the spike
// bitmap of step t + 1 - delay and writes the complete input of step t + 1.
// Each lane takes four consecutive entries of a 128-entry window that starts
// on a multiple of four (one 16-byte load of source words, one 4-byte load of
// delays), so a column of up to 125 entries is a single pass; weights are read
// only for entries whose source fired.  The slot of step t + 1 - d is
// (s1 - d) mod D with s1 = (t + 1) mod D, in 32-bit arithmetic.
// Deterministic: each lane adds its entries in column order, then the warp
// tree reduction in a fixed order.
__global__ void __launch_bounds__(DELIV_THREADS) k_deliver_pull(PullArgs a)
{
    const uint64_t t1 = *a.base + (uint64_t)a.q + 1;
    const int s1 = (int)(t1 % (uint64_t)a.D);
    // delays longer than the elapsed steps reach back before step 0
    const int dlim = t1 < (uint64_t)a.D ? (int)t1 : a.D;
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * (DELIV_THREADS / 32) + (threadIdx.x >> 5);
    const int nwarps = gridDim.x * (DELIV_THREADS / 32);
    float* out = a.ring + (size_t)(t1 % (uint64_t)a.D) * a.n_pad * 2;
    for (int k = gw; k < a.n; k += nwarps) {
        const int64_t beg = a.col_ptr[k], end = a.col_ptr[k + 1];
        float acc_e = 0.0f, acc_i = 0.0f;
        for (int64_t e0 = (beg & ~(int64_t)3) + 4 * lane; e0 < end; e0 += 128) {
            const uint4 sv = *reinterpret_cast<const uint4*>(a.csc_src + e0);
            const uint32_t dv = *reinterpret_cast<const uint32_t*>(a.csc_d + e0);
            const uint32_t src[4] = {sv.x, sv.y, sv.z, sv.w};
            uint32_t hit = 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int d = (int)((dv >> (8 * j)) & 0xffu);
                const int64_t e = e0 + j;
                int hs = s1 - d;
                if (hs < 0) hs += a.D;
                if (e >= beg && e < end && d <= dlim && (!a.rowflag || a.rowflag[hs])) {
                    const uint32_t sid = src[j] & 0x7fffffffu;
                    const uint32_t word = a.bitmap[(size_t)hs * a.words + (sid >> 5)];
                    hit |= ((word >> (sid & 31)) & 1u) << j;
                }
            }
            if (hit) {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if ((hit >> j) & 1u) {
                        const float w = a.csc_w[e0 + j];
                        if (src[j] >> 31) acc_i += w;
                        else acc_e += w;
                    }
            }
        }
        acc_e = nn_warp_sumf(acc_e);
        acc_i = nn_warp_sumf(acc_i);
        if (lane == 0) {
            float2* o = reinterpret_cast<float2*>(out) + k;
            if (a.add) {
                const float2 v = *o;
                *o = make_float2(v.x + acc_e, v.y + acc_i);
            } else {
                *o = make_float2(acc_e, acc_i);
            }
        }
    }
}

// Pull through shared memory.  A block owns dsl_cols consecutive columns
// (postsynaptic neurons).  Its synapses are stored as one run per block,
// ordered by delay and, within a delay, by source bucket (DSL_BUCKET_WORDS
// bitmap words = 16,384 consecutive source neurons), and cut into chunks of
// at most DSL_CHUNK entries that span at most DSL_SPAN buckets.  An entry is
// one 32-bit word: the source's offset from the chunk's first bucket (18
// bits), the column offset within the block (13 bits) and the inhibitory bit.
// A chunk of delay d needs only its buckets' words of the spike bitmap of step
// t + 1 - d; two bulk copies stage those words (from L2) and the chunk's
// entries (from DRAM) into one of dsl_ring shared-memory slots, completing on
// the slot's "full" mbarrier.  Every consumer thread tests DSL_EPT entries of
// each chunk (16-byte reads; a warp reads consecutive words) against the
// staged bitmap, all lookups before any use.  Hits go to a per-warp queue of
// (entry, word) pairs in shared memory; a warp empties its queue when it could
// overflow and at the end into the block's hit list in global memory (room
// for every entry of the block), every lane loading all its weights before it
// stores any.  A warp done with a chunk arrives on the slot's "empty"
// mbarrier; one producer warp waits for it and refills the slot with the
// chunk dsl_ring places later.  Consumer warps drift apart by up to
// dsl_ring - 1 chunks, and no block-wide barrier separates the delays.  The
// sums are not held during the sweep, so the slots get all the shared memory
// (six at 1M neurons instead of three next to the sums): after the sweep the
// block adds its hit list into 64-bit fixed-point sums in the slots' bytes
// (weight x 2^32; integer addition does not depend on order, so the result is
// deterministic, and exact for weights >= 2^-8).  DRAM traffic per step: 4 B
// per synapse, per synapse whose source fired its weight and 16 B of hit
// list (written, then read back, mostly from L2), the ring slot written (8 B
// per neuron); the bitmap words come from L2.
// Every wait is bounded: a thread that gives up sets error bit 2 and the
// block's abort flag; the block then waits (bounded) for its copies in flight
// and leaves without writing its columns.
constexpr int DSL_THREADS = 512;                  // consumer threads (plus one producer warp)
constexpr int DSL_WARPS = DSL_THREADS / 32;
constexpr int DSL_EPT = 16;                       // entries per consumer thread and chunk
constexpr int DSL_CHUNK = DSL_EPT * DSL_THREADS;  // entries per chunk at most
constexpr int DSL_BUCKET_WORDS = 512;             // bitmap words per source bucket
constexpr int DSL_SPAN = 16;                      // buckets per chunk at most: source offsets below 2^18
constexpr int DSL_MAX_RING = 6;                   // slots at most
constexpr int DSL_HITCAP = 128;                   // hits a warp's queue holds
constexpr int DSL_MAX_COLS = 8192;                // 13-bit column offsets
constexpr int DSL_MAX_DELAY = 64;
constexpr double DSL_FIX = 4294967296.0;  // 2^32
constexpr uint32_t DSL_WAIT_LIMIT = 1u << 22;
static_assert(DSL_SPAN * DSL_BUCKET_WORDS * 32 <= (1 << 18), "source offsets take 18 bits");

// Stage chunk m = {first entry, entries, first word, words << 8 | delay}: its
// bitmap words of the row of step t + 1 - d, then its entries (a multiple of
// four words; the layout pads every chunk).
__device__ __forceinline__ void dsl_issue(const PullArgs& a, int s1, int4 m, uint32_t* dst, uint64_t* bar)
{
    int hs = s1 - (m.w & 255);
    if (hs < 0) hs += a.D;
    const uint32_t bw = (uint32_t)(m.w >> 8) * 4u;
    const uint32_t be = (uint32_t)((m.y + 3) & ~3) * 4u;
    nn_mbar_expect_tx(bar, bw + be);
    nn_bulk_g2s(dst, a.bitmap + (size_t)hs * a.words + m.z, bw, bar);
    nn_bulk_g2s(dst + a.dsl_slotw, a.dsl_ent + m.x, be, bar);
}

// Move a warp's queued hits {entry, word} to the block's hit list: each lane
// loads its weights, then stores {word, weight bits} pairs at out[0, cnt).
__device__ __forceinline__ void dsl_flush(const uint2* q, int cnt, int lane, const float* w, uint2* out)
{
    constexpr int PER = DSL_HITCAP / 32;
    uint32_t ew[PER];
    float wv[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int i = lane + 32 * k;
        ew[k] = 0u;
        wv[k] = 0.0f;
        if (i < cnt) {
            const uint2 h = q[i];
            ew[k] = h.y;
            wv[k] = w[h.x];
        }
    }
#pragma unroll
    for (int k = 0; k < PER; ++k)
        if (lane + 32 * k < cnt) out[lane + 32 * k] = make_uint2(ew[k], __float_as_uint(wv[k]));
}

__global__ void __launch_bounds__(DSL_THREADS + 32, 1) k_deliver_pull_sliced(PullArgs a)
{
    extern __shared__ __align__(128) unsigned char dsl_smem[];
    const int R = a.dsl_ring, SW = a.dsl_slotw, SL = a.dsl_slotw + DSL_CHUNK;  // slot: bitmap words, entries
    uint32_t* ring = reinterpret_cast<uint32_t*>(dsl_smem);
    // after the sweep the slots hold the sums
    unsigned long long* acc_e = reinterpret_cast<unsigned long long*>(dsl_smem);
    unsigned long long* acc_i = acc_e + a.dsl_cols;
    uint2* hitq = reinterpret_cast<uint2*>(
        dsl_smem + max((size_t)R * SL * 4, (size_t)a.dsl_cols * 16));  // [DSL_WARPS][DSL_HITCAP]
    int4* tab = reinterpret_cast<int4*>(hitq + DSL_WARPS * DSL_HITCAP);
    uint64_t* full = reinterpret_cast<uint64_t*>(tab + a.dsl_cmax);
    uint64_t* empty = full + R;
    int* last = reinterpret_cast<int*>(empty + R);  // last chunk issued into a slot
    __shared__ volatile int abort_flag;
    __shared__ int hit_count;  // entries of the block's hit list
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint64_t t1 = *a.base + (uint64_t)a.q + 1;
    const int s1 = (int)(t1 % (uint64_t)a.D);
    const int k0 = blockIdx.x * a.dsl_cols;
    const int k1 = min(a.n, k0 + a.dsl_cols);
    // delays beyond t + 1 reach before step 0
    const int dlast = min(t1 < (uint64_t)(a.D - 1) ? (int)t1 : a.D - 1, a.dsl_dmax);
    const int32_t* cp = a.dsl_cptr + (size_t)blockIdx.x * (a.dsl_dmax + 1);
    const int cfirst = cp[0];
    // the chunks of the live delays, in delay order: all of them, or with
    // rowflag given those whose source row was a pull step (warp 0 scans their
    // counts, two delays per lane)
    __shared__ int s_off[DSL_MAX_DELAY + 1], s_cp[DSL_MAX_DELAY + 1];
    int C = 0;
    if (!a.rowflag) {
        C = dlast >= 1 ? cp[dlast] - cfirst : 0;
        for (int c = tid; c < C; c += blockDim.x) tab[c] = a.dsl_chunk[cfirst + c];
    } else {
        if (warp == 0) {
            int len[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int d = lane + 1 + 32 * h;
                len[h] = 0;
                if (d <= dlast) {
                    int hs = s1 - d;
                    if (hs < 0) hs += a.D;
                    const int c0 = cp[d - 1];
                    s_cp[d] = c0;  // first chunk of delay d
                    if (a.rowflag[hs]) len[h] = cp[d] - c0;
                }
            }
            int run = 0;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                int v = len[h];
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int u = __shfl_up_sync(0xffffffffu, v, o);
                    if (lane >= o) v += u;
                }
                s_off[lane + 1 + 32 * h] = run + v;  // live chunks of delays <= lane + 1 + 32 h
                run += __shfl_sync(0xffffffffu, v, 31);
            }
            if (lane == 0) s_off[0] = 0;
        }
        __syncthreads();
        C = dlast >= 1 ? s_off[dlast] : 0;
        // one pass over the live chunks: live chunk c belongs to the delay d
        // with s_off[d - 1] <= c < s_off[d] (binary search)
        for (int c = tid; c < C; c += blockDim.x) {
            int lo = 1, hi = dlast;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (s_off[mid] > c) hi = mid;
                else lo = mid + 1;
            }
            tab[c] = a.dsl_chunk[s_cp[lo] + (c - s_off[lo - 1])];
        }
    }
    // the block's hit list starts at its first entry: it has room for every entry
    uint2* hits = a.dsl_hits + (C > 0 ? a.dsl_chunk[cfirst].x : 0);
    if (tid == 0) {
        abort_flag = 0;
        hit_count = 0;
        for (int r = 0; r < R; ++r) {
            nn_mbar_init(&full[r], 1);
            nn_mbar_init(&empty[r], DSL_WARPS);
            last[r] = -1;
        }
        nn_mbar_fence_init();
    }
    __syncthreads();
    if (warp == DSL_WARPS) {
        // producer: the first dsl_ring chunks, then chunk c once every
        // consumer warp is done with chunk c - dsl_ring
        if (lane == 0)
            for (int c = 0; c < C; ++c) {
                const int slot = c % R;
                if (c >= R) {
                    if (!nn_mbar_wait(&empty[slot], (uint32_t)((c / R - 1) & 1), DSL_WAIT_LIMIT)) {
                        abort_flag = 1;
                        break;
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                }
                last[slot] = c;
                dsl_issue(a, s1, tab[c], ring + (size_t)slot * SL, &full[slot]);
            }
    } else {
        uint2* hq = hitq + warp * DSL_HITCAP;
        int hcnt = 0;  // hits in this warp's queue (the same in every lane)
        int slot = 0;
        uint32_t phase = 0;
        for (int c = 0; c < C; ++c) {
            // (another warp's abort shows up here as a wait that runs out)
            const bool landed = __all_sync(0xffffffffu, nn_mbar_wait(&full[slot], phase, DSL_WAIT_LIMIT));
            if (!landed) {
                abort_flag = 1;
                break;
            }
            const int4 m = tab[c];
            const uint32_t* bm = ring + (size_t)slot * SL;
            const uint4* ent = reinterpret_cast<const uint4*>(bm + SW);
            uint32_t ew[DSL_EPT];
#pragma unroll
            for (int g = 0; g < DSL_EPT / 4; ++g) {
                const uint4 v = ent[tid + DSL_THREADS * g];
                ew[4 * g] = v.x;
                ew[4 * g + 1] = v.y;
                ew[4 * g + 2] = v.z;
                ew[4 * g + 3] = v.w;
            }
            // entry q of this thread: 4 (tid + DSL_THREADS (q / 4)) + q % 4.
            // Its source bit: word (offset >> 5) of the staged range, bit
            // (offset & 31) -- the low five bits of the entry word -- rotated
            // into bit q of hit.  In a partial chunk, words past its end
            // (padding, or left from an earlier chunk) are looked up at word 0
            // and masked.
            uint32_t hit = 0;
            if (m.y == DSL_CHUNK) {
#pragma unroll
                for (int q = 0; q < DSL_EPT; ++q) {
                    const uint32_t wv = bm[(ew[q] >> 5) & 0x1fffu];
                    hit |= __funnelshift_r(wv, wv, ew[q] - (uint32_t)q) & (1u << q);
                }
            } else {
#pragma unroll
                for (int q = 0; q < DSL_EPT; ++q) {
                    const int i = 4 * (tid + DSL_THREADS * (q / 4)) + (q % 4);
                    const bool in = i < m.y;
                    const uint32_t e = in ? ew[q] : 0u;
                    const uint32_t wv = bm[(e >> 5) & 0x1fffu];
                    hit |= __funnelshift_r(wv, wv, e - (uint32_t)q) & (in ? (1u << q) : 0u);
                }
            }
            // the slot's words are all read: release it to the producer
            __syncwarp();
            if (lane == 0) nn_mbar_arrive(&empty[slot]);
            if (__any_sync(0xffffffffu, hit != 0)) {
#pragma unroll
                for (int q = 0; q < DSL_EPT; ++q) {
                    const bool h = (hit >> q) & 1u;
                    const unsigned b = __ballot_sync(0xffffffffu, h);
                    if (!b) continue;
                    if (hcnt + __popc(b) > DSL_HITCAP) {
                        int hb = 0;
                        if (lane == 0) hb = atomicAdd(&hit_count, hcnt);
                        hb = __shfl_sync(0xffffffffu, hb, 0);
                        __syncwarp();
                        dsl_flush(hq, hcnt, lane, a.dsl_w, hits + hb);
                        __syncwarp();
                        hcnt = 0;
                    }
                    if (h) {
                        const int i = 4 * (tid + DSL_THREADS * (q / 4)) + (q % 4);
                        hq[hcnt + __popc(b & ((1u << lane) - 1u))] = make_uint2((uint32_t)(m.x + i), ew[q]);
                    }
                    hcnt += __popc(b);
                }
            }
            if (++slot == R) {
                slot = 0;
                phase ^= 1u;
            }
        }
        if (!abort_flag && hcnt > 0) {
            int hb = 0;
            if (lane == 0) hb = atomicAdd(&hit_count, hcnt);
            hb = __shfl_sync(0xffffffffu, hb, 0);
            __syncwarp();
            dsl_flush(hq, hcnt, lane, a.dsl_w, hits + hb);
        }
    }
    __syncthreads();
    if (abort_flag) {
        if (tid == 0) {
            atomicOr(a.err, 2);
            for (int r = 0; r < R; ++r)
                if (last[r] >= 0) nn_mbar_wait(&full[r], (uint32_t)((last[r] / R) & 1), DSL_WAIT_LIMIT);
        }
        return;
    }
    // every staged chunk was consumed, so no copy into the slots is pending:
    // sum the hit list (written by this block, read back through L2) into
    // the slots' bytes
    for (int k = tid; k < a.dsl_cols; k += blockDim.x) acc_e[k] = acc_i[k] = 0ull;
    __syncthreads();
    for (int i = tid; i < hit_count; i += blockDim.x) {
        const uint2 h = __ldcg(hits + i);
        atomicAdd(((h.x >> 31) ? acc_i : acc_e) + ((h.x >> 18) & 0x1fffu),
                  (unsigned long long)llrintf(__uint_as_float(h.y) * (float)DSL_FIX));
    }
    __syncthreads();
    float2* out = reinterpret_cast<float2*>(a.ring + (size_t)(t1 % (uint64_t)a.D) * a.n_pad * 2);
    for (int k = tid; k < k1 - k0; k += blockDim.x) {
        const float2 v = make_float2((float)((double)(long long)acc_e[k] / DSL_FIX),
                                     (float)((double)(long long)acc_i[k] / DSL_FIX));
        if (a.add) {
            const float2 o = out[k0 + k];
            out[k0 + k] = make_float2(o.x + v.x, o.y + v.y);
        } else {
            out[k0 + k] = v;
        }
    }
}

// Automatic delivery, return from pull to push at step T (the pull gather
// after step T - 1 delivered every arrival up to step T): the spikes of the
// pull rows among steps T - D .. T - 1 scatter their out-edges that arrive at
// step T + 1 or later, as the push would have.  Grid (word groups, D rows), a
// warp per bitmap word.
__global__ void __launch_bounds__(256) k_flush_pull(const uint32_t* bitmap, const int* rowflag, const int64_t* row_ptr,
                                                    const int32_t* col, const float* weight, const uint8_t* delay,
                                                    const uint8_t* is_inh, float* ring, int n, int n_pad, int D,
                                                    int words, long long T)
{
    const int r = blockIdx.y;
    if (!rowflag[r]) return;
    // the step row r holds: the latest step <= T - 1 congruent to r mod D
    const long long s = T - 1 - ((T - 1 - r) % D + D) % D;
    if (s < 0) return;
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (w >= words) return;
    uint32_t bits = bitmap[(size_t)r * words + w];
    while (bits) {
        const int j = 32 * w + __ffs(bits) - 1;
        bits &= bits - 1;
        if (j >= n) break;
        const int64_t beg = row_ptr[j], end = row_ptr[j + 1];
        const int chn = is_inh[j] ? 1 : 0;
        for (int64_t e = beg + lane; e < end; e += 32) {
            const long long arr = s + delay[e];
            if (arr >= T + 1) atomicAdd(ring + 2 * ((size_t)(arr % D) * n_pad + col[e]) + chn, weight[e]);
        }
    }
}

// Bounds for the fixed-point sums: the longest column and the largest |weight|.
__global__ void k_dsl_bounds(const int64_t* col_ptr, const float* csc_w, int n, unsigned int* out)
{
    unsigned int len = 0, wmax = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        len = max(len, (unsigned int)(col_ptr[k + 1] - col_ptr[k]));
        for (int64_t e = col_ptr[k]; e < col_ptr[k + 1]; ++e) wmax = max(wmax, __float_as_uint(fabsf(csc_w[e])));
    }
    atomicMax(out, len);
    atomicMax(out + 1, wmax);  // non-negative floats order like their bit patterns
}

// Chunked layout.  Entries counted per (column block, delay, source bucket), a
// thread per column ...
// (delays outside [1, dmax] cannot occur -- the network setters check them --
// and would be left out of both passes alike)
__device__ __forceinline__ size_t dsl_key(int k, int cols, int dmax, int nb, int d, uint32_t sw)
{
    const int bucket = (int)((sw & 0x7fffffffu) >> 5) / DSL_BUCKET_WORDS;
    return ((size_t)(k / cols) * dmax + (d - 1)) * nb + bucket;
}

__global__ void k_dsl_count(const int64_t* col_ptr, const uint32_t* csc_src, const uint8_t* csc_d, int n, int cols,
                            int dmax, int nb, unsigned int* cnt)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        for (int64_t e = col_ptr[k]; e < col_ptr[k + 1]; ++e) {
            const int d = csc_d[e];
            if (d >= 1 && d <= dmax) atomicAdd(&cnt[dsl_key(k, cols, dmax, nb, d, csc_src[e])], 1u);
        }
}

// ... placed at their bucket's cursor (first entry of the bucket, from the
// host's scan of the counts; the order inside a bucket is the order of the
// atomics and may differ between builds -- the fixed-point sums do not depend
// on it) ...
__global__ void k_dsl_fill(const int64_t* col_ptr, const uint32_t* csc_src, const float* csc_w, const uint8_t* csc_d,
                           int n, int cols, int dmax, int nb, unsigned int* cursor, uint32_t* out_src, float* out_w,
                           uint16_t* out_col)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        for (int64_t e = col_ptr[k]; e < col_ptr[k + 1]; ++e) {
            const int d = csc_d[e];
            if (d < 1 || d > dmax) continue;
            const uint32_t sw = csc_src[e];
            const unsigned int q = atomicAdd(&cursor[dsl_key(k, cols, dmax, nb, d, sw)], 1u);
            out_src[q] = sw;
            out_w[q] = csc_w[e];
            out_col[q] = (uint16_t)(k % cols);
        }
}

// ... and packed chunk by chunk into entry words (each chunk padded with
// zero entries to a multiple of four); ustart: the chunk's first entry in the
// bucketed arrays.  Within a chunk the entries are dealt to positions so that
// the 32 lanes of one lookup of k_deliver_pull_sliced read 32 different
// shared-memory banks: entries are ranked within their bank (bank = bitmap
// word & 31), the sequence "rank 0 of every bank, rank 1 of every bank, ..."
// is formed, and its element j goes to the j-th position in lookup order
// (dsl_lookup_rank).  While every bank still has entries, each lookup reads
// one word per bank.  A warp's lookup q reads positions
// 4 (32 h + lane) + c with h = warp + DSL_WARPS (q / 4), c = q % 4.  The
// order of entries does not change the fixed-point sums.
__device__ __forceinline__ int dsl_lookup_rank(int p, int n)
{
    const int h = p >> 7, c = p & 3;
    int r = 128 * h + ((p >> 2) & 31);
    for (int cc = 0; cc < c; ++cc) r += min(max((n - 128 * h - cc + 3) >> 2, 0), 32);
    return r;
}

constexpr int DSL_PACK_THREADS = 256;
constexpr int DSL_PACK_SMEM = DSL_CHUNK * 8;

__global__ void __launch_bounds__(DSL_PACK_THREADS) k_dsl_pack(const int4* chunk, const int32_t* ustart,
                                                               int nchunks, const uint32_t* src,
                                                               const uint16_t* col, const float* w,
                                                               uint32_t* ent, float* wout)
{
    constexpr int NW = DSL_PACK_THREADS / 32;
    // dynamic shared memory (DSL_PACK_SMEM bytes): the chunk's words, the rank
    // of each entry within its bank, the position of lookup-order index j
    extern __shared__ __align__(16) unsigned char pack_smem[];
    uint32_t* s_word = reinterpret_cast<uint32_t*>(pack_smem);
    uint16_t* s_rank = reinterpret_cast<uint16_t*>(s_word + DSL_CHUNK);
    uint16_t* s_pos = s_rank + DSL_CHUNK;
    __shared__ int s_cw[NW][32];            // per warp: entries per bank, then the warp's first rank
    __shared__ int s_cnt[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int4 m = chunk[c];
        const int us = ustart[c];
        const int n = m.y;
        const int padded = (n + 3) & ~3;
        for (int i = tid; i < n; i += DSL_PACK_THREADS) {
            const uint32_t sw = src[us + i];
            s_word[i] = ((sw & 0x7fffffffu) - (uint32_t)m.z * 32u) | ((uint32_t)col[us + i] << 18) |
                        (sw & 0x80000000u);
        }
        for (int p = tid; p < n; p += DSL_PACK_THREADS) s_pos[dsl_lookup_rank(p, n)] = (uint16_t)p;
        if (tid < NW * 32) s_cw[tid >> 5][tid & 31] = 0;
        __syncthreads();
        // rank within the bank: warp k ranks entries [k per, (k + 1) per) in
        // order, 32 at a time (peers with the same bank by __match_any_sync)
        const int per = ((n + NW - 1) / NW + 31) & ~31;
        for (int i0 = warp * per; i0 < min(n, (warp + 1) * per); i0 += 32) {
            const int i = i0 + lane;
            const uint32_t bank = i < n ? (s_word[i] >> 5) & 31u : 32u + (uint32_t)lane;
            const unsigned peers = __match_any_sync(0xffffffffu, bank);
            if (i < n) s_rank[i] = (uint16_t)(s_cw[warp][bank] + __popc(peers & ((1u << lane) - 1u)));
            __syncwarp();
            if (i < n && (__ffs(peers) - 1) == lane) s_cw[warp][bank] += __popc(peers);
            __syncwarp();
        }
        __syncthreads();
        if (tid < 32) {
            int acc = 0;
            for (int k = 0; k < NW; ++k) {
                const int t = s_cw[k][tid];
                s_cw[k][tid] = acc;
                acc += t;
            }
            s_cnt[tid] = acc;
        }
        __syncthreads();
        for (int i = tid; i < n; i += DSL_PACK_THREADS) {
            const uint32_t word = s_word[i];
            const int bank = (int)((word >> 5) & 31u);
            const int r = s_rank[i] + s_cw[i / per][bank];
            int j = 0;
#pragma unroll 8
            for (int b = 0; b < 32; ++b) {
                const int cb = s_cnt[b];
                j += min(cb, r) + (b < bank && cb > r ? 1 : 0);
            }
            const int p = s_pos[j];
            ent[m.x + p] = word;
            wout[m.x + p] = w[us + i];
        }
        for (int p = n + tid; p < padded; p += DSL_PACK_THREADS) {
            ent[m.x + p] = 0u;
            wout[m.x + p] = 0.0f;
        }
        __syncthreads();
    }
}

// Push delivery of an explicit spike list at the current step: the same
// scatter as the fused neuron update (a warp per spike, lanes over its
// out-edges, red.global.add into ring slot (t + d) % D), for callers that
// produce spikes elsewhere and for timing the delivery path on its own.
__global__ void __launch_bounds__(DELIV_THREADS) k_deliver_list(const int* list, int count, const int64_t* row_ptr,
                                                                const int32_t* col, const float* weight,
                                                                const uint8_t* delay, const uint8_t* is_inh,
                                                                float* ring, const unsigned long long* base,
                                                                int n_pad, int D)
{
    const int slot = (int)(*base % (uint64_t)D);
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * (DELIV_THREADS / 32) + (threadIdx.x >> 5);
    const int nwarps = gridDim.x * (DELIV_THREADS / 32);
    for (int q = gw; q < count; q += nwarps) {
        const int j = list[q];
        const int chn = is_inh[j] ? 1 : 0;
        const int64_t beg = row_ptr[j], end = row_ptr[j + 1];
        // PUSH_UNROLL edges per lane loaded before their reductions
        for (int64_t e0 = beg + lane; e0 < end; e0 += 32 * PUSH_UNROLL) {
            int tgt[PUSH_UNROLL], dl[PUSH_UNROLL];
            float w[PUSH_UNROLL];
#pragma unroll
            for (int u = 0; u < PUSH_UNROLL; ++u) {
                const int64_t e = e0 + 32 * u;
                if (e < end) {
                    tgt[u] = col[e];
                    w[u] = weight[e];
                    dl[u] = delay[e];
                }
            }
#pragma unroll
            for (int u = 0; u < PUSH_UNROLL; ++u) {
                if (e0 + 32 * u >= end) break;
                int sl = slot + dl[u];
                if (sl >= D) sl -= D;
                atomicAdd(ring + 2 * ((size_t)sl * n_pad + tgt[u]) + chn, w[u]);
            }
        }
    }
}

// spike bitmap of the current step from a list (pull delivery)
__global__ void k_list_bitmap(const int* list, int count, uint32_t* bitmap, const unsigned long long* base, int D,
                              int words)
{
    uint32_t* bm = bitmap + (size_t)(*base % (uint64_t)D) * words;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < count; q += gridDim.x * blockDim.x)
        atomicOr(bm + (list[q] >> 5), 1u << (list[q] & 31));
}

// paracrine: b = u + src ; src = 0 ; with u_prev: initial guess u <- 2u - u_prev
// (linear extrapolation in time of the slowly evolving field), u_prev <- u
__global__ void k_par_rhs(float* u, float* src, float* b, float* u_prev, int extrapolate, int64_t G)
{
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < G; q += (int64_t)gridDim.x * blockDim.x) {
        const float uq = u[q];
        b[q] = uq + src[q];
        src[q] = 0.0f;
        if (u_prev) {
            if (extrapolate) u[q] = 2.0f * uq - u_prev[q];
            u_prev[q] = uq;
        }
    }
}

__global__ void k_par_gather(const float* u, const int32_t* vox, float* upar, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) upar[i] = u[vox[i]];
}

// ------------------------------------------------------------ generators --

__global__ void k_fill_f(float* p, int64_t n, float v)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

// ER: edge i -> j (j != i) iff philox word < thr; counts per row.
// Instance of neuron i (binary search over the instance offsets; one instance
// when inst_off is null).
__device__ __forceinline__ int instance_of(const int* inst_off, int n_inst, int i)
{
    int lo = 0, hi = n_inst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (inst_off[mid] <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Erdos-Renyi rows by counter-based draws.  With instances (a batch), row i
// of instance b draws only among the instance's neurons, with the instance's
// threshold and the stream key seed + b over local indices, so each block of
// the block-diagonal network equals the single network of that size and seed.
struct ErRows {
    int n;
    uint32_t thr;
    uint64_t seed;
    const int* inst_off;   // null: one network
    const uint32_t* inst_thr;
    const float* inst_wmax;  // null: the network's w_max
    int n_inst;
};

__device__ __forceinline__ void er_row(const ErRows& g, int i, int& li, int& base, int& size, uint32_t& thr,
                                       uint64_t& key)
{
    if (g.inst_off) {
        const int b = instance_of(g.inst_off, g.n_inst, i);
        base = g.inst_off[b];
        size = g.inst_off[b + 1] - base;
        li = i - base;
        thr = g.inst_thr[b];
        key = g.seed + (uint64_t)b;
    } else {
        base = 0;
        size = g.n;
        li = i;
        thr = g.thr;
        key = g.seed;
    }
}

__global__ void k_er_count(ErRows g, int64_t* cnt)
{
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < g.n; i += nw) {
        int li, base, size;
        uint32_t thr;
        uint64_t key;
        er_row(g, i, li, base, size, thr, key);
        const int nb = (size + 3) >> 2;
        int c = 0;
        for (int jb = lane; jb < nb; jb += 32) {
            const nn_u4 r = nn_philox(key, (uint32_t)li, (uint32_t)jb, 0u, NN_P_ER);
            const uint32_t w[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int j = 4 * jb + q;
                c += (j < size && j != li && w[q] < thr) ? 1 : 0;
            }
        }
        c = __reduce_add_sync(0xffffffffu, c);
        if (lane == 0) cnt[i] = c;
    }
}

__global__ void k_er_fill(ErRows g, float wmax_all, const int64_t* row_ptr, int32_t* col, float* weight,
                          uint8_t* delay)
{
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < g.n; i += nw) {
        int li, base, size;
        uint32_t thr;
        uint64_t key;
        er_row(g, i, li, base, size, thr, key);
        const float wmax = g.inst_wmax ? g.inst_wmax[instance_of(g.inst_off, g.n_inst, i)] : wmax_all;
        const int nb = (size + 3) >> 2;
        int64_t pos = row_ptr[i];
        int e_run = 0;
        for (int jb0 = 0; jb0 < nb; jb0 += 32) {
            const int jb = jb0 + lane;
            uint32_t m = 0;
            if (jb < nb) {
                const nn_u4 r = nn_philox(key, (uint32_t)li, (uint32_t)jb, 0u, NN_P_ER);
                const uint32_t w[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int j = 4 * jb + q;
                    if (j < size && j != li && w[q] < thr) m |= 1u << q;
                }
            }
            const int c = __popc(m);
            int inc = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int tv = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += tv;
            }
            int e = e_run + inc - c;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (m & (1u << q)) {
                    const nn_u4 rw = nn_philox(key, (uint32_t)li, (uint32_t)e, 0u, NN_P_WEIGHT);
                    col[pos + e] = base + 4 * jb + q;
                    weight[pos + e] = __fmul_rn(wmax, nn_u01f(rw.x));
                    delay[pos + e] = 1;
                    ++e;
                }
            e_run += __shfl_sync(0xffffffffu, inc, 31);
        }
    }
}

__device__ __forceinline__ float lognormal_w(uint64_t seed, uint32_t i, uint32_t e, double mu, double sg, uint32_t* r2)
{
    const nn_u4 rw = nn_philox(seed, i, e, 0u, NN_P_WEIGHT);
    const double u1 = nn_u01d_open(rw.x), u2 = nn_u01d(rw.y);
    const double z = sqrt(-2.0 * log(u1)) * cos(6.283185307179586476925 * u2);
    *r2 = rw.z;
    return (float)exp(mu + sg * z);
}

// Gaussian distance-dependent: fixed out-degree k, lattice offsets drawn from
// the discretised Gaussian table, redrawn while outside the lattice, empty or
// the source itself (64 attempts, then the next neuron).
__global__ void k_gauss_fill(int n, int k, int L, const int16_t* table, uint64_t seed, double mu, double sg, int dmax,
                             int32_t* col, float* weight, uint8_t* delay)
{
    const int64_t total = (int64_t)n * k;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(q / k), e = (int)(q % k);
        const int cx = i % L, cy = (i / L) % L, cz = i / (L * L);
        int tgt = (i + 1) % n;
        for (int at = 0; at < 64; ++at) {
            const nn_u4 r = nn_philox(seed, (uint32_t)i, (uint32_t)e, (uint32_t)at, NN_P_GAUSS);
            const int tx = cx + table[r.x >> 20], ty = cy + table[r.y >> 20], tz = cz + table[r.z >> 20];
            if (tx < 0 || ty < 0 || tz < 0 || tx >= L || ty >= L || tz >= L) continue;
            const int64_t s = (int64_t)tx + (int64_t)L * ((int64_t)ty + (int64_t)L * tz);
            if (s >= n || s == i) continue;
            tgt = (int)s;
            break;
        }
        uint32_t r2;
        weight[q] = lognormal_w(seed, (uint32_t)i, (uint32_t)e, mu, sg, &r2);
        col[q] = tgt;
        delay[q] = (uint8_t)(1u + (uint32_t)(((uint64_t)r2 * (uint64_t)dmax) >> 32));
    }
}

// Region-block model: source region r, target region drawn from the row's
// cumulative 32-bit thresholds, target neuron uniform in the region, delay from
// the region-pair table.
__global__ void k_block_fill(int n, int k, int R, const int* region_of, const int* region_start,
                             const int* region_size, const uint32_t* cum, const uint8_t* pair_delay, uint64_t seed,
                             double mu, double sg, int32_t* col, float* weight, uint8_t* delay)
{
    const int64_t total = (int64_t)n * k;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(q / k), e = (int)(q % k);
        const int r = region_of[i];
        int tgt = (i + 1) % n, s = r;
        for (int at = 0; at < 64; ++at) {
            const nn_u4 u = nn_philox(seed, (uint32_t)i, (uint32_t)e, (uint32_t)at, NN_P_BLOCK);
            // first region whose cumulative threshold exceeds u.x
            int lo = 0, hi = R - 1;
            const uint32_t* row = cum + (size_t)r * R;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (row[mid] > u.x) hi = mid; else lo = mid + 1;
            }
            s = lo;
            const int off = (int)(((uint64_t)u.y * (uint64_t)region_size[s]) >> 32);
            const int cand = region_start[s] + off;
            if (cand == i) continue;
            tgt = cand;
            break;
        }
        uint32_t r2;
        weight[q] = lognormal_w(seed, (uint32_t)i, (uint32_t)e, mu, sg, &r2);
        col[q] = tgt;
        delay[q] = pair_delay[(size_t)r * R + s];
    }
}

__global__ void k_inh(int n, int random, double frac, uint64_t seed, uint8_t* is_inh)
{
    const int n_inh = (int)llround(frac * n);
    const double tf = floor(frac * 4294967296.0);
    const uint32_t thr = tf >= 4294967295.0 ? 0xffffffffu : (uint32_t)tf;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (random) is_inh[i] = nn_philox(seed, (uint32_t)i, 0u, 0u, NN_P_TYPE).x < thr ? 1 : 0;
        else is_inh[i] = i >= n - n_inh ? 1 : 0;
    }
}

// Initial state: V = v0, gates at their steady state, synapses 0, drive
// lo + (hi - lo) u, jittered-lattice positions and their voxels.
__global__ void k_init_state(StepArgs a, float v0, float m0, float h0, float n0, float lo, float hi, float* x, float* y,
                             float* z, float* gs, int L, int grid, int32_t* vox)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n_pad; i += gridDim.x * blockDim.x) {
        a.V[i] = v0; a.m[i] = m0; a.h[i] = h0; a.nn[i] = n0; a.ge[i] = 0.0f; a.gi[i] = 0.0f;
        gs[i] = 1.0f;
        if (i >= a.n) {
            const_cast<float*>(a.idrive)[i] = 0.0f;
            x[i] = y[i] = z[i] = 0.0f;
            continue;
        }
        const nn_u4 r = nn_philox(a.seed, (uint32_t)i, 0u, 0u, NN_P_DRIVE);
        const_cast<float*>(a.idrive)[i] = __fadd_rn(lo, __fmul_rn(__fsub_rn(hi, lo), nn_u01f(r.x)));
        const nn_u4 rp = nn_philox(a.seed, (uint32_t)i, 0u, 0u, NN_P_POS);
        const int cx = i % L, cy = (i / L) % L, cz = i / (L * L);
        x[i] = __fdiv_rn(__fadd_rn((float)cx, nn_u01f(rp.x)), (float)L);
        y[i] = __fdiv_rn(__fadd_rn((float)cy, nn_u01f(rp.y)), (float)L);
        z[i] = __fdiv_rn(__fadd_rn((float)cz, nn_u01f(rp.z)), (float)L);
        if (vox) {
            int ix = (int)__fmul_rn(x[i], (float)grid), iy = (int)__fmul_rn(y[i], (float)grid),
                iz = (int)__fmul_rn(z[i], (float)grid);
            ix = min(max(ix, 0), grid - 1); iy = min(max(iy, 0), grid - 1); iz = min(max(iz, 0), grid - 1);
            vox[i] = ix + grid * (iy + grid * iz);
        }
    }
}

// Batch: each instance on its own jittered lattice in the unit cube (local
// index, stream key seed + b), and voxels of its own grid (cell offset goff).
__global__ void k_inst_positions(int n, const int* inst_off, int n_inst, uint64_t seed, float* x, float* y, float* z)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int b = instance_of(inst_off, n_inst, i);
        const int li = i - inst_off[b];
        const int L = nn_lattice_side(inst_off[b + 1] - inst_off[b]);
        const nn_u4 rp = nn_philox(seed + (uint64_t)b, (uint32_t)li, 0u, 0u, NN_P_POS);
        const int cx = li % L, cy = (li / L) % L, cz = li / (L * L);
        x[i] = __fdiv_rn(__fadd_rn((float)cx, nn_u01f(rp.x)), (float)L);
        y[i] = __fdiv_rn(__fadd_rn((float)cy, nn_u01f(rp.y)), (float)L);
        z[i] = __fdiv_rn(__fadd_rn((float)cz, nn_u01f(rp.z)), (float)L);
    }
}

__global__ void k_inst_vox(const float* x, const float* y, const float* z, int n, const int* inst_off, int n_inst,
                           const int* inst_grid, const int64_t* inst_goff, int32_t* vox)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int b = instance_of(inst_off, n_inst, i);
        const int grid = inst_grid[b];
        int ix = (int)__fmul_rn(x[i], (float)grid), iy = (int)__fmul_rn(y[i], (float)grid),
            iz = (int)__fmul_rn(z[i], (float)grid);
        ix = min(max(ix, 0), grid - 1); iy = min(max(iy, 0), grid - 1); iz = min(max(iz, 0), grid - 1);
        vox[i] = (int32_t)(inst_goff[b] + ix + (int64_t)grid * (iy + (int64_t)grid * iz));
    }
}

__global__ void k_vox(const float* x, const float* y, const float* z, int n, int grid, int32_t* vox)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int ix = (int)__fmul_rn(x[i], (float)grid), iy = (int)__fmul_rn(y[i], (float)grid),
            iz = (int)__fmul_rn(z[i], (float)grid);
        ix = min(max(ix, 0), grid - 1); iy = min(max(iy, 0), grid - 1); iz = min(max(iz, 0), grid - 1);
        vox[i] = ix + grid * (iy + grid * iz);
    }
}

// CSC payload gather after the edge ids are ordered
__global__ void k_csc_gather(const uint32_t* edge_of, int64_t nnz, const int64_t* row_ptr, int n, const float* w,
                             const uint8_t* d, const uint8_t* is_inh, uint32_t* src, float* cw, uint8_t* cd)
{
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = edge_of[q];
        int lo = 0, hi = n - 1;  // row containing e: last lo with row_ptr[lo] <= e
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (row_ptr[mid] <= e) lo = mid; else hi = mid - 1;
        }
        src[q] = (uint32_t)lo | (is_inh[lo] ? 0x80000000u : 0u);
        cw[q] = w[e];
        cd[q] = d[e];
    }
}

}  // namespace

// ================================================================== API ====

extern "C" void nn_hh_params_standard(nn_hh_params* p)
{
    if (!p) return;
    p->C = 1.0f; p->gNa = 120.0f; p->gK = 36.0f; p->gL = 0.3f;
    p->ENa = 50.0f; p->EK = -77.0f; p->EL = -54.4f;
    p->E_exc = 0.0f; p->E_inh = -80.0f; p->tau_exc = 5.0f; p->tau_inh = 5.0f;
    p->v_thresh = -20.0f; p->noise_sigma = 1.0f; p->dt = 0.01f;
    p->g_par = 0.0f; p->E_par = 0.0f;
}

extern "C" void nn_sim_config_default(nn_sim_config* c, int n)
{
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->n = n;
    c->max_delay = 1;
    c->seed = 1;
    nn_hh_params_standard(&c->hp);
    c->delivery = NN_DELIVERY_PUSH;
    c->grid = 0;
    c->timescale = 100;
    c->par_D = 1.0f;
    c->par_decay = 0.0f;
    c->par_rtol = 1e-6;
    c->par_max_iter = 2000;
    c->par_extrapolate = 0;
    c->par_overlap = 1;
    c->pull_rate = 0.025f;
}

extern "C" void nn_net_spec_default(nn_net_spec* sp, int kind)
{
    if (!sp) return;
    std::memset(sp, 0, sizeof *sp);
    sp->kind = kind;
    sp->p = 0.01;
    sp->w_max = 0.5f;
    sp->k = 100;
    sp->sigma = 0.1;
    sp->w_mu = -1.0;
    sp->w_sigma = 1.0;
    sp->dmax = kind == NN_NET_ER ? 1 : 20;
    sp->inh_fraction = 0.2;
    sp->inh_random = kind == NN_NET_ER ? 0 : 1;
    sp->n_regions = 200;
    sp->region_size_sigma = 1.0;
    sp->density_sigma = 1.0;
    sp->block_dmax = 40;
}

// a paracrine field exists: one grid, or one grid per instance of a batch
static bool has_field(const nn_sim* s) { return s->grid > 0 || s->bpcg != nullptr; }

static StepArgs step_args(nn_sim* s, int q)
{
    StepArgs a;
    a.V = s->f[NN_F_V]; a.m = s->f[NN_F_M]; a.h = s->f[NN_F_H]; a.nn = s->f[NN_F_N];
    a.ge = s->f[NN_F_GE]; a.gi = s->f[NN_F_GI];
    a.idrive = s->f[NN_F_IDRIVE];
    a.gna_scale = s->gna_set ? s->f[NN_F_GNA_SCALE] : nullptr;  // all ones unless set
    a.upar = (s->cfg.hp.g_par != 0.0f && has_field(s)) ? s->f[NN_F_UPAR] : nullptr;
    a.ring = reinterpret_cast<float*>(s->ring);
    const bool autod = s->cfg.delivery == NN_DELIVERY_AUTO;
    // automatic delivery: push periods write no bitmap
    a.bitmap = autod && s->cur_mode == 0 ? nullptr : s->bitmap;
    a.rowflag = autod ? s->rowflag : nullptr;
    a.list = s->list;
    a.counts = s->counts;
    a.base = s->step;
    a.q = q;
    const bool push = s->cfg.delivery == NN_DELIVERY_PUSH || (autod && s->cur_mode == 0);
    a.row_ptr = push ? s->row_ptr : nullptr;
    a.col = s->col;
    a.weight = s->weight;
    a.delay = s->delay;
    a.is_inh = s->is_inh;
    a.total = s->total;
    a.rcount = s->rcount;
    a.raster = s->raster;
    a.rcap = s->cfg.raster_capacity;
    a.vox = s->vox;
    a.src = has_field(s) ? s->src : nullptr;
    a.el_group = s->el_group;
    a.el_val = s->el_val;
    a.el_spk = s->el_spk;
    a.el_every = s->el_every;
    a.el_cap = s->el_cap;
    a.el_members = s->el_members;
    a.err = s->err;
    a.n = s->n; a.n_pad = s->n_pad; a.D = s->D; a.words = s->words;
    a.zero_ring = push || autod;
    a.seed = s->cfg.seed;
    a.p = nn_hh_to_dev(s->cfg.hp);
    return a;
}

static PullArgs pull_args(nn_sim* s, int q, bool hybrid)
{
    PullArgs a;
    a.rowflag = hybrid ? s->rowflag : nullptr;
    a.add = hybrid ? 1 : 0;
    a.col_ptr = s->col_ptr; a.csc_src = s->csc_src; a.csc_w = s->csc_w; a.csc_d = s->csc_d;
    a.bitmap = s->bitmap;
    a.ring = reinterpret_cast<float*>(s->ring);
    a.base = s->step;
    a.q = q;
    a.n = s->n; a.n_pad = s->n_pad; a.D = s->D; a.words = s->words;
    a.dsl_chunk = s->dsl_chunk; a.dsl_cptr = s->dsl_cptr;
    a.dsl_ent = s->dsl_ent; a.dsl_w = s->dsl_w; a.dsl_hits = s->dsl_hits;
    a.dsl_cols = s->dsl_cols; a.dsl_ring = s->dsl_ring; a.dsl_slotw = s->dsl_slotw;
    a.dsl_cmax = s->dsl_cmax; a.dsl_dmax = s->dsl_dmax;
    a.err = s->err;
    return a;
}

// Dynamic shared memory of k_deliver_pull_sliced: the slots (slotw bitmap
// words and a chunk of entries each) during the sweep, the same bytes as two
// 64-bit sums per column after it; the warps' hit queues, the block's chunk
// table, and per slot two mbarriers (full, empty) and the last chunk issued.
static size_t dsl_smem_bytes(int ring, int slotw, int cols, int cmax)
{
    return std::max((size_t)ring * (slotw + DSL_CHUNK) * 4, (size_t)cols * 16) + (size_t)DSL_WARPS * DSL_HITCAP * 8 +
           (size_t)cmax * 16 + (size_t)ring * 20;
}

// The pull gather of one step: through shared memory when the chunked layout
// exists, else the warp-per-column kernel.
static nn_status launch_pull(nn_sim* s, const PullArgs& d, cudaStream_t cs)
{
    nn_ctx* ctx = s->ctx;
    if (s->dsl_chunk) {
        const int blocks = (s->n + s->dsl_cols - 1) / s->dsl_cols;
        k_deliver_pull_sliced<<<blocks, DSL_THREADS + 32,
                                dsl_smem_bytes(s->dsl_ring, s->dsl_slotw, s->dsl_cols, s->dsl_cmax), cs>>>(d);
        NN_CHECK_LAUNCH(ctx, "k_deliver_pull_sliced");
        return NN_OK;
    }
    k_deliver_pull<<<nn_grid_for(ctx, (int64_t)s->n * 32, DELIV_THREADS, 8), DELIV_THREADS, 0, cs>>>(d);
    NN_CHECK_LAUNCH(ctx, "k_deliver_pull");
    return NN_OK;
}

static void drop_graph(nn_sim* s)
{
    if (s->graph) cudaGraphExecDestroy(s->graph);
    if (s->graph_pull) cudaGraphExecDestroy(s->graph_pull);
    s->graph = nullptr;
    s->graph_pull = nullptr;
    s->graph_steps = 0;
}

extern "C" nn_status nn_sim_create(nn_ctx* ctx, const nn_sim_config* cfg, nn_sim** out)
{
    if (!ctx || !cfg || !out) return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_sim_create: NULL argument");
    if (cfg->n <= 0 || cfg->max_delay < 1 || cfg->max_delay > 254 ||
        (cfg->delivery != NN_DELIVERY_PUSH && cfg->delivery != NN_DELIVERY_PULL &&
         cfg->delivery != NN_DELIVERY_AUTO) || cfg->grid < 0 ||
        (cfg->grid > 0 && cfg->timescale < 1) || !(cfg->hp.dt > 0.0f) || cfg->raster_capacity < 0)
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_sim_create: invalid configuration");
    if (cfg->neurons_per_thread != 0 && cfg->neurons_per_thread != 1 && cfg->neurons_per_thread != 2 &&
        cfg->neurons_per_thread != 4)
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_sim_create: neurons_per_thread must be 1, 2 or 4");
    nn_sim* s = new nn_sim();
    s->ctx = ctx;
    nn_ctx_retain(ctx);
    s->cfg = *cfg;
    s->n = cfg->n;
    s->n_pad = (cfg->n + 127) / 128 * 128;
    s->D = cfg->max_delay + 1;
    s->words = s->n_pad / 32;
    s->npt = cfg->neurons_per_thread ? cfg->neurons_per_thread : 2;
    // 128 threads: 3 % faster than 256 on the 1M-neuron workload (smaller blocks
    // even out the last wave)
    s->tpb = cfg->threads_per_block ? cfg->threads_per_block : 128;
    if (s->tpb % 32 || s->tpb > 256 || s->tpb < 32) {
        nn_sim_destroy(s);
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_sim_create: threads_per_block must be a multiple of 32 <= 256");
    }
    s->grid = cfg->grid;
    s->G = (int64_t)cfg->grid * cfg->grid * cfg->grid;
    const size_t NP = (size_t)s->n_pad;
    nn_status st = NN_OK;
    for (int q = 0; q < NN_F_COUNT && st == NN_OK; ++q) st = nn_alloc(ctx, &s->f[q], NP);
    if (st == NN_OK) st = nn_alloc(ctx, &s->ring, (size_t)s->D * NP);
    const bool autod = cfg->delivery == NN_DELIVERY_AUTO;
    if (st == NN_OK && (cfg->delivery == NN_DELIVERY_PULL || autod))
        st = nn_alloc(ctx, &s->bitmap, (size_t)s->D * s->words);
    if (st == NN_OK && autod) {
        if (!(cfg->pull_rate >= 0.0f)) s->cfg.pull_rate = 0.025f;
        st = nn_alloc(ctx, &s->rowflag, (size_t)s->D);
        if (st == NN_OK)
            st = nn_cuda_check(ctx, cudaHostAlloc(&s->h_tot, sizeof(unsigned long long) * nn_sim::TOT_Q, 0),
                               "cudaHostAlloc");
        for (int k = 0; k < nn_sim::TOT_Q && st == NN_OK; ++k)
            st = nn_cuda_check(ctx, cudaEventCreateWithFlags(&s->ev_tot[k], cudaEventDisableTiming), "event");
    }
    if (st == NN_OK) st = nn_alloc(ctx, &s->list, 2 * NP);
    if (st == NN_OK) st = nn_alloc(ctx, &s->counts, 2);
    if (st == NN_OK) st = nn_alloc(ctx, &s->step, 1);
    if (st == NN_OK) st = nn_alloc(ctx, &s->total, 1);
    if (st == NN_OK) st = nn_alloc(ctx, &s->rcount, 1);
    if (st == NN_OK && cfg->raster_capacity > 0) st = nn_alloc(ctx, &s->raster, (size_t)cfg->raster_capacity);
    if (st == NN_OK) st = nn_alloc(ctx, &s->err, 1);
    if (st == NN_OK) st = nn_alloc(ctx, &s->is_inh, NP);
    if (st == NN_OK && s->grid > 0) {
        st = nn_alloc(ctx, &s->vox, NP);
        if (st == NN_OK) st = nn_alloc(ctx, &s->src, (size_t)s->G);
        if (st == NN_OK) st = nn_alloc(ctx, &s->u, (size_t)s->G);
        if (st == NN_OK && cfg->par_extrapolate) st = nn_alloc(ctx, &s->u_prev, (size_t)s->G);
        if (st == NN_OK) st = nn_alloc(ctx, &s->b, (size_t)s->G);
        if (st == NN_OK) {
            const double dt_s = (double)cfg->timescale * cfg->hp.dt * 1e-3;
            const double alpha = dt_s * cfg->par_D * (double)cfg->grid * cfg->grid;
            const double beta = dt_s * cfg->par_decay;
            st = nn_pcg_create(ctx, cfg->grid, cfg->grid, cfg->grid, alpha, beta, nullptr, &s->pcg);
        }
    }
    if (st != NN_OK) {
        nn_sim_destroy(s);
        return st;
    }
    cudaStream_t cs = ctx->stream;
    for (int q = 0; q < NN_F_COUNT; ++q) cudaMemsetAsync(s->f[q], 0, NP * sizeof(float), cs);
    k_fill_f<<<nn_grid_for(ctx, (int64_t)NP, 256), 256, 0, cs>>>(s->f[NN_F_GNA_SCALE], (int64_t)NP, 1.0f);
    ctx->launches++;
    cudaMemsetAsync(s->ring, 0, (size_t)s->D * NP * sizeof(float2), cs);
    if (s->bitmap) cudaMemsetAsync(s->bitmap, 0, (size_t)s->D * s->words * sizeof(uint32_t), cs);
    if (s->rowflag) cudaMemsetAsync(s->rowflag, 0, (size_t)s->D * sizeof(int), cs);
    cudaMemsetAsync(s->list, 0, 2 * NP * sizeof(int), cs);
    cudaMemsetAsync(s->counts, 0, 2 * sizeof(int), cs);
    cudaMemsetAsync(s->step, 0, sizeof(unsigned long long), cs);
    cudaMemsetAsync(s->total, 0, sizeof(unsigned long long), cs);
    cudaMemsetAsync(s->rcount, 0, sizeof(unsigned long long), cs);
    cudaMemsetAsync(s->err, 0, sizeof(int), cs);
    cudaMemsetAsync(s->is_inh, 0, NP, cs);
    if (s->grid > 0) {
        cudaMemsetAsync(s->vox, 0, NP * sizeof(int32_t), cs);
        cudaMemsetAsync(s->src, 0, (size_t)s->G * sizeof(float), cs);
        cudaMemsetAsync(s->u, 0, (size_t)s->G * sizeof(float), cs);
    }
    st = nn_cuda_check(ctx, cudaStreamSynchronize(cs), "nn_sim_create");
    if (st != NN_OK) {
        nn_sim_destroy(s);
        return st;
    }
    *out = s;
    return NN_OK;
}

static void free_network(nn_sim* s)
{
    nn_release(s->row_ptr); nn_release(s->col); nn_release(s->weight); nn_release(s->delay);
    nn_release(s->col_ptr); nn_release(s->csc_src); nn_release(s->csc_w); nn_release(s->csc_d);
    nn_release(s->dsl_chunk); nn_release(s->dsl_cptr); nn_release(s->dsl_ent); nn_release(s->dsl_w); nn_release(s->dsl_hits);
    s->nnz = 0;
}

extern "C" nn_status nn_sim_destroy(nn_sim* s)
{
    if (!s) return NN_OK;
    if (s->par_stream) cudaStreamSynchronize(s->par_stream);
    if (s->ctx) cudaStreamSynchronize(s->ctx->stream);
    drop_graph(s);
    for (int q = 0; q < NN_F_COUNT; ++q) nn_release(s->f[q]);
    nn_release(s->ring); nn_release(s->bitmap); nn_release(s->list); nn_release(s->counts); nn_release(s->step);
    nn_release(s->rowflag);
    if (s->h_tot) cudaFreeHost(s->h_tot);
    for (auto e : s->ev_tot)
        if (e) cudaEventDestroy(e);
    nn_release(s->el_group); nn_release(s->el_val); nn_release(s->el_spk);
    nn_release(s->total); nn_release(s->rcount); nn_release(s->raster); nn_release(s->err);
    nn_release(s->is_inh); nn_release(s->vox); nn_release(s->src); nn_release(s->u); nn_release(s->u_prev); nn_release(s->b);
    free_network(s);
    if (s->pcg) nn_pcg_destroy(s->pcg);
    if (s->bpcg) nn_bpcg_destroy(s->bpcg);
    nn_release(s->inst_off); nn_release(s->inst_grid); nn_release(s->inst_goff);
    if (s->par_stream) cudaStreamDestroy(s->par_stream);
    if (s->ev_rhs) cudaEventDestroy(s->ev_rhs);
    if (s->ev_solved) cudaEventDestroy(s->ev_solved);
    for (auto e : s->ev_a) cudaEventDestroy(e);
    for (auto e : s->ev_b) cudaEventDestroy(e);
    for (auto e : s->ev_c) cudaEventDestroy(e);
    nn_ctx* ctx = s->ctx;
    delete s;
    nn_ctx_release(ctx);
    return NN_OK;
}

// Chunked copy of the CSC for the shared-memory pull kernel (see
// k_deliver_pull_sliced), built when the block's sums, chunk table and at
// least two slots fit in a block's shared memory, a block has at most
// DSL_MAX_COLS columns, delays stay within DSL_MAX_DELAY, entry offsets within
// 32 bits and the fixed-point sums below 2^31 (longest column x largest
// |weight|).  The host cuts each (block, delay) run into chunks from the
// bucket counts; the entries are first placed by bucket, then packed chunk by
// chunk.  NN_PULL_UNSLICED=1 keeps the warp-per-column kernel (for
// comparisons); NN_PULL_RING=r caps the slots at r (2 .. DSL_MAX_RING).
static nn_status build_sliced(nn_sim* s)
{
    nn_ctx* ctx = s->ctx;
    const char* env = std::getenv("NN_PULL_UNSLICED");
    if (env && env[0] == '1') return NN_OK;
    int smem_max = 0;
    NN_CUDA(ctx, cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    const int cols = (s->n + ctx->num_sms - 1) / ctx->num_sms;
    const int nblk = (s->n + cols - 1) / cols;
    const int dmax = s->D - 1;
    const int nb = (s->words + DSL_BUCKET_WORDS - 1) / DSL_BUCKET_WORDS;
    const int slotw = std::min(s->words, DSL_SPAN * DSL_BUCKET_WORDS);
    if (s->nnz <= 0 || dsl_smem_bytes(2, slotw, cols, 0) > (size_t)smem_max || cols > DSL_MAX_COLS || dmax < 1 ||
        dmax > DSL_MAX_DELAY || s->nnz >= INT32_MAX / 2 || (s->words % 4))
        return NN_OK;
    // fixed-point range: |sum| <= longest column x largest |weight| < 2^31
    unsigned int* bnd = nullptr;
    NN_TRY(nn_alloc(ctx, &bnd, 2));
    NN_CUDA(ctx, nn_zero_async(ctx, bnd, 2 * sizeof(unsigned int)));
    k_dsl_bounds<<<nn_grid_for(ctx, s->n, 256, 8), 256, 0, ctx->stream>>>(s->col_ptr, s->csc_w, s->n, bnd);
    NN_CHECK_LAUNCH(ctx, "k_dsl_bounds");
    unsigned int hb[2] = {0, 0};
    const cudaError_t ce = nn_copy_sync(ctx, hb, bnd, sizeof hb, cudaMemcpyDeviceToHost);
    cudaFree(bnd);
    NN_CUDA(ctx, ce);
    float wmax;
    std::memcpy(&wmax, &hb[1], sizeof wmax);
    if (!(std::isfinite(wmax)) || (double)hb[0] * (double)wmax >= 2147483648.0) return NN_OK;
    // entries per (block, delay, bucket)
    const size_t nkeys = (size_t)nblk * dmax * nb;
    unsigned int* cnt = nullptr;
    NN_TRY(nn_alloc(ctx, &cnt, nkeys));
    std::vector<unsigned int> h(nkeys);
    nn_status st = nn_cuda_check(ctx, nn_zero_async(ctx, cnt, sizeof(unsigned int) * nkeys), "build_sliced");
    if (st == NN_OK) {
        k_dsl_count<<<nn_grid_for(ctx, s->n, 256, 8), 256, 0, ctx->stream>>>(s->col_ptr, s->csc_src, s->csc_d, s->n,
                                                                            cols, dmax, nb, cnt);
        st = nn_cuda_check(ctx, cudaGetLastError(), "k_dsl_count");
    }
    if (st == NN_OK)
        st = nn_cuda_check(ctx, nn_copy_sync(ctx, h.data(), cnt, sizeof(unsigned int) * nkeys, cudaMemcpyDeviceToHost),
                           "build_sliced");
    // bucket offsets (block-major), chunks and their padded starts
    std::vector<int4> chunks;         // {padded first entry, entries, first word, words << 8 | delay}
    std::vector<int32_t> ustart;      // first entry in the bucketed arrays
    std::vector<int32_t> cptr((size_t)nblk * (dmax + 1));
    int cmax = 0;
    int64_t pos = 0, ppos = 0;
    if (st == NN_OK) {
        for (int b = 0; b < nblk; ++b) {
            const size_t c_b = chunks.size();
            cptr[(size_t)b * (dmax + 1)] = (int32_t)c_b;
            for (int d = 1; d <= dmax; ++d) {
                bool open = false;
                int64_t start = 0;
                int len = 0, b0 = 0, b1 = 0;
                auto close = [&]() {
                    const int w0 = b0 * DSL_BUCKET_WORDS;
                    const int w1 = std::min((b1 + 1) * DSL_BUCKET_WORDS, s->words);
                    chunks.push_back(make_int4((int)ppos, len, w0, ((w1 - w0) << 8) | d));
                    ustart.push_back((int32_t)start);
                    ppos += (len + 3) & ~3;
                    open = false;
                };
                for (int bk = 0; bk < nb; ++bk) {
                    const size_t key = ((size_t)b * dmax + (d - 1)) * nb + bk;
                    int64_t left = h[key];
                    h[key] = (unsigned int)pos;
                    while (left > 0) {
                        if (open && (len == DSL_CHUNK || bk - b0 >= DSL_SPAN)) close();
                        if (!open) {
                            open = true;
                            start = pos;
                            len = 0;
                            b0 = bk;
                        }
                        const int take = (int)std::min<int64_t>(left, DSL_CHUNK - len);
                        len += take;
                        pos += take;
                        left -= take;
                        b1 = bk;
                    }
                }
                if (open) close();
                cptr[(size_t)b * (dmax + 1) + d] = (int32_t)chunks.size();
            }
            cmax = std::max(cmax, (int)(chunks.size() - c_b));
        }
    }
    // slots: as many as fit, up to DSL_MAX_RING (at least two)
    int ring = DSL_MAX_RING;
    if (const char* r = std::getenv("NN_PULL_RING")) ring = std::max(2, std::min(DSL_MAX_RING, std::atoi(r)));
    while (ring >= 2 && dsl_smem_bytes(ring, slotw, cols, cmax) > (size_t)smem_max) --ring;
    if (st != NN_OK || pos > s->nnz || ppos >= INT32_MAX || chunks.empty() || ring < 2) {
        cudaFree(cnt);
        return st;
    }
    // place by bucket into temporary arrays, then pack chunk by chunk
    uint32_t* t_src = nullptr;
    uint16_t* t_col = nullptr;
    float* t_w = nullptr;
    int32_t* d_ustart = nullptr;
    const size_t E = (size_t)std::max<int64_t>(pos, 1);
    st = nn_cuda_check(ctx, nn_copy_sync(ctx, cnt, h.data(), sizeof(unsigned int) * nkeys, cudaMemcpyHostToDevice),
                       "build_sliced");
    if (st == NN_OK) st = nn_alloc(ctx, &t_src, E);
    if (st == NN_OK) st = nn_alloc(ctx, &t_col, E);
    if (st == NN_OK) st = nn_alloc(ctx, &t_w, E);
    if (st == NN_OK) st = nn_alloc(ctx, &d_ustart, ustart.size());
    if (st == NN_OK) st = nn_alloc(ctx, &s->dsl_chunk, chunks.size());
    if (st == NN_OK) st = nn_alloc(ctx, &s->dsl_cptr, cptr.size());
    if (st == NN_OK) st = nn_alloc(ctx, &s->dsl_ent, (size_t)ppos);
    if (st == NN_OK) st = nn_alloc(ctx, &s->dsl_w, (size_t)ppos);
    if (st == NN_OK) st = nn_alloc(ctx, &s->dsl_hits, (size_t)ppos);
    if (st == NN_OK)
        st = nn_cuda_check(ctx, nn_copy_sync(ctx, s->dsl_chunk, chunks.data(), sizeof(int4) * chunks.size(),
                                             cudaMemcpyHostToDevice), "build_sliced");
    if (st == NN_OK)
        st = nn_cuda_check(ctx, nn_copy_sync(ctx, s->dsl_cptr, cptr.data(), sizeof(int32_t) * cptr.size(),
                                             cudaMemcpyHostToDevice), "build_sliced");
    if (st == NN_OK)
        st = nn_cuda_check(ctx, nn_copy_sync(ctx, d_ustart, ustart.data(), sizeof(int32_t) * ustart.size(),
                                             cudaMemcpyHostToDevice), "build_sliced");
    if (st == NN_OK) {
        k_dsl_fill<<<nn_grid_for(ctx, s->n, 128, 8), 128, 0, ctx->stream>>>(
            s->col_ptr, s->csc_src, s->csc_w, s->csc_d, s->n, cols, dmax, nb, cnt, t_src, t_w, t_col);
        st = nn_cuda_check(ctx, cudaGetLastError(), "k_dsl_fill");
    }
    if (st == NN_OK) {
        st = nn_cuda_check(ctx, cudaFuncSetAttribute(k_dsl_pack, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     DSL_PACK_SMEM), "cudaFuncSetAttribute");
    }
    if (st == NN_OK) {
        const int nc = (int)chunks.size();
        k_dsl_pack<<<std::min(nc, ctx->num_sms * 8), DSL_PACK_THREADS, DSL_PACK_SMEM, ctx->stream>>>(
            s->dsl_chunk, d_ustart, nc, t_src, t_col, t_w, s->dsl_ent, s->dsl_w);
        st = nn_cuda_check(ctx, cudaGetLastError(), "k_dsl_pack");
    }
    const size_t smem = dsl_smem_bytes(ring, slotw, cols, cmax);
    if (st == NN_OK)
        st = nn_cuda_check(ctx, cudaFuncSetAttribute(k_deliver_pull_sliced,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                           "cudaFuncSetAttribute");
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "build_sliced");
    cudaFree(cnt);
    cudaFree(t_src);
    cudaFree(t_col);
    cudaFree(t_w);
    cudaFree(d_ustart);
    if (st != NN_OK) {
        nn_release(s->dsl_chunk); nn_release(s->dsl_cptr); nn_release(s->dsl_ent); nn_release(s->dsl_w); nn_release(s->dsl_hits);
        return st;
    }
    s->dsl_cols = cols;
    s->dsl_ring = ring;
    s->dsl_slotw = slotw;
    s->dsl_cmax = cmax;
    s->dsl_dmax = dmax;
    return NN_OK;
}

static nn_status build_csc(nn_sim* s)
{
    nn_ctx* ctx = s->ctx;
    if (s->col_ptr) return NN_OK;
    NN_TRY(nn_alloc(ctx, &s->col_ptr, (size_t)s->n + 1));
    uint32_t* edge_of = nullptr;
    NN_TRY(nn_alloc(ctx, &edge_of, (size_t)std::max<int64_t>(s->nnz, 1)));
    NN_TRY(nn_build_csc(ctx, s->n, s->nnz, s->row_ptr, s->col, s->col_ptr, edge_of));
    // the pull kernel reads whole groups of four entries: pad to a multiple
    // of four (the padding is never summed)
    const size_t E = ((size_t)std::max<int64_t>(s->nnz, 1) + 3) & ~(size_t)3;
    NN_TRY(nn_alloc(ctx, &s->csc_src, E));
    NN_TRY(nn_alloc(ctx, &s->csc_w, E));
    NN_TRY(nn_alloc(ctx, &s->csc_d, E));
    NN_CUDA(ctx, nn_zero_async(ctx, s->csc_src, E * sizeof(uint32_t)));
    NN_CUDA(ctx, nn_zero_async(ctx, s->csc_w, E * sizeof(float)));
    NN_CUDA(ctx, nn_zero_async(ctx, s->csc_d, E));
    if (s->nnz > 0) {
        k_csc_gather<<<nn_grid_for(ctx, s->nnz, 256, 16), 256, 0, ctx->stream>>>(
            edge_of, s->nnz, s->row_ptr, s->n, s->weight, s->delay, s->is_inh, s->csc_src, s->csc_w, s->csc_d);
        NN_CHECK_LAUNCH(ctx, "k_csc_gather");
    }
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFree(edge_of);
    return build_sliced(s);
}

static nn_status after_network(nn_sim* s)
{
    drop_graph(s);
    nn_release(s->col_ptr); nn_release(s->csc_src); nn_release(s->csc_w); nn_release(s->csc_d);
    nn_release(s->dsl_chunk); nn_release(s->dsl_cptr); nn_release(s->dsl_ent); nn_release(s->dsl_w); nn_release(s->dsl_hits);
    if (s->cfg.delivery == NN_DELIVERY_PULL || s->cfg.delivery == NN_DELIVERY_AUTO) NN_TRY(build_csc(s));
    return NN_OK;
}

extern "C" nn_status nn_sim_set_network(nn_sim* s, const int64_t* h_row_ptr, const int32_t* h_col,
                                        const float* h_weight, const uint8_t* h_delay, int64_t nnz,
                                        const uint8_t* h_is_inh)
{
    if (!s || !h_row_ptr || nnz < 0 || (nnz && (!h_col || !h_weight || !h_delay)))
        return nn_fail(s ? s->ctx : nullptr, NN_ERR_INVALID_ARG, "nn_sim_set_network: bad argument");
    nn_ctx* ctx = s->ctx;
    const int n = s->n;
    if (h_row_ptr[0] != 0 || h_row_ptr[n] != nnz) return nn_fail(ctx, NN_ERR_INVALID_ARG, "row_ptr must span [0, nnz]");
    for (int i = 0; i < n; ++i)
        if (h_row_ptr[i + 1] < h_row_ptr[i]) return nn_fail(ctx, NN_ERR_INVALID_ARG, "row_ptr is not monotone at %d", i);
    for (int64_t e = 0; e < nnz; ++e) {
        if (h_col[e] < 0 || h_col[e] >= n) return nn_fail(ctx, NN_ERR_INVALID_ARG, "col[%lld] = %d out of range", (long long)e, h_col[e]);
        if (h_delay[e] < 1 || h_delay[e] > s->cfg.max_delay)
            return nn_fail(ctx, NN_ERR_INVALID_ARG, "delay[%lld] = %d outside [1, %d]", (long long)e, h_delay[e], s->cfg.max_delay);
        if (!std::isfinite(h_weight[e])) return nn_fail(ctx, NN_ERR_INVALID_ARG, "weight[%lld] is not finite", (long long)e);
    }
    free_network(s);
    s->nnz = nnz;
    const size_t E = (size_t)std::max<int64_t>(nnz, 1);
    NN_TRY(nn_alloc(ctx, &s->row_ptr, (size_t)n + 1));
    NN_TRY(nn_alloc(ctx, &s->col, E));
    NN_TRY(nn_alloc(ctx, &s->weight, E));
    NN_TRY(nn_alloc(ctx, &s->delay, E));
    cudaStream_t cs = ctx->stream;
    NN_CUDA(ctx, cudaMemcpyAsync(s->row_ptr, h_row_ptr, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyHostToDevice, cs));
    if (nnz) {
        NN_CUDA(ctx, cudaMemcpyAsync(s->col, h_col, sizeof(int32_t) * (size_t)nnz, cudaMemcpyHostToDevice, cs));
        NN_CUDA(ctx, cudaMemcpyAsync(s->weight, h_weight, sizeof(float) * (size_t)nnz, cudaMemcpyHostToDevice, cs));
        NN_CUDA(ctx, cudaMemcpyAsync(s->delay, h_delay, (size_t)nnz, cudaMemcpyHostToDevice, cs));
    }
    NN_CUDA(ctx, cudaMemsetAsync(s->is_inh, 0, (size_t)s->n_pad, cs));
    if (h_is_inh) NN_CUDA(ctx, cudaMemcpyAsync(s->is_inh, h_is_inh, (size_t)n, cudaMemcpyHostToDevice, cs));
    NN_CUDA(ctx, cudaStreamSynchronize(cs));
    return after_network(s);
}

// Host-side tables of the region-block model (shared by the oracle's
// restatement): lognormal region sizes (largest-remainder rounding), uniform
// centroids, lognormal block densities turned into per-row cumulative 32-bit
// thresholds weighted by target size, delays 1..dmax by centroid distance.
static void block_tables(int n, const nn_net_spec* sp, uint64_t seed, std::vector<int>& start, std::vector<int>& size,
                         std::vector<uint32_t>& cum, std::vector<uint8_t>& pdelay)
{
    const int R = sp->n_regions;
    std::vector<double> w(R), cx(R), cy(R), cz(R);
    double sw = 0.0;
    for (int r = 0; r < R; ++r) {
        const nn_u4 u = nn_philox(seed, (uint32_t)r, 0u, 0u, NN_P_REGION);
        const double u1 = nn_u01d_open(u.x), u2 = nn_u01d(u.y);
        const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586476925 * u2);
        w[r] = std::exp(sp->region_size_sigma * z);
        sw += w[r];
        cx[r] = nn_u01d(u.z);
        const nn_u4 v = nn_philox(seed, (uint32_t)r, 1u, 0u, NN_P_REGION);
        cy[r] = nn_u01d(v.x);
        cz[r] = nn_u01d(v.y);
    }
    // every region gets at least one neuron, the rest by largest remainder
    size.assign(R, 1);
    int left = n - R;
    std::vector<double> fr(R);
    std::vector<int> order(R);
    int assigned = 0;
    for (int r = 0; r < R; ++r) {
        const double want = left * w[r] / sw;
        const int fl = (int)std::floor(want);
        size[r] += fl;
        assigned += fl;
        fr[r] = want - fl;
        order[r] = r;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return fr[a] > fr[b]; });
    for (int q = 0; q < left - assigned; ++q) size[order[q]] += 1;
    start.assign(R, 0);
    for (int r = 1; r < R; ++r) start[r] = start[r - 1] + size[r - 1];
    // block densities
    cum.assign((size_t)R * R, 0);
    pdelay.assign((size_t)R * R, 1);
    double dmax_dist = 0.0;
    for (int r = 0; r < R; ++r)
        for (int t = 0; t < R; ++t)
            dmax_dist = std::max(dmax_dist, std::sqrt((cx[r] - cx[t]) * (cx[r] - cx[t]) + (cy[r] - cy[t]) * (cy[r] - cy[t]) +
                                                      (cz[r] - cz[t]) * (cz[r] - cz[t])));
    std::vector<double> row(R);
    for (int r = 0; r < R; ++r) {
        double s = 0.0;
        for (int t = 0; t < R; ++t) {
            const nn_u4 u = nn_philox(seed, (uint32_t)r, (uint32_t)t, 0u, NN_P_BLOCK + 16u);
            const double u1 = nn_u01d_open(u.x), u2 = nn_u01d(u.y);
            const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586476925 * u2);
            row[t] = std::exp(sp->density_sigma * z) * (double)size[t];
            s += row[t];
            const double dist = std::sqrt((cx[r] - cx[t]) * (cx[r] - cx[t]) + (cy[r] - cy[t]) * (cy[r] - cy[t]) +
                                          (cz[r] - cz[t]) * (cz[r] - cz[t]));
            const double dd = dmax_dist > 0 ? 1.0 + (sp->block_dmax - 1) * dist / dmax_dist : 1.0;
            pdelay[(size_t)r * R + t] = (uint8_t)std::min<long>(sp->block_dmax, std::max<long>(1, std::lround(dd)));
        }
        double acc = 0.0;
        for (int t = 0; t < R; ++t) {
            acc += row[t];
            const double th = std::floor(acc / s * 4294967296.0);
            cum[(size_t)r * R + t] = t == R - 1 ? 0xffffffffu : (uint32_t)std::min(th, 4294967295.0);
        }
    }
}

static void free_instances(nn_sim* s)
{
    nn_release(s->inst_off);
    nn_release(s->inst_grid);
    nn_release(s->inst_goff);
    if (s->bpcg) {
        nn_bpcg_destroy(s->bpcg);
        s->bpcg = nullptr;
        nn_release(s->vox);
        nn_release(s->src);
        nn_release(s->u);
        nn_release(s->b);
        s->G = 0;
    }
    s->n_inst = 0;
    s->h_inst_off.clear();
    s->h_inst_grid.clear();
}

extern "C" nn_status nn_sim_set_instances(nn_sim* s, int n_inst, const int* h_offsets, const int* h_grid_sides)
{
    if (!s || n_inst < 1 || !h_offsets) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    if (h_offsets[0] != 0 || h_offsets[n_inst] != s->n)
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "instance offsets must run from 0 to n = %d", s->n);
    for (int b = 0; b < n_inst; ++b)
        if (h_offsets[b + 1] <= h_offsets[b])
            return nn_fail(ctx, NN_ERR_INVALID_ARG, "instance %d is empty", b);
    if (h_grid_sides) {
        if (s->grid > 0)
            return nn_fail(ctx, NN_ERR_INVALID_ARG, "per-instance grids need a simulation created with grid = 0");
        for (int b = 0; b < n_inst; ++b)
            if (h_grid_sides[b] < 1) return nn_fail(ctx, NN_ERR_INVALID_ARG, "instance %d: grid side < 1", b);
    }
    drop_graph(s);
    free_instances(s);
    s->n_inst = n_inst;
    s->h_inst_off.assign(h_offsets, h_offsets + n_inst + 1);
    NN_TRY(nn_alloc(ctx, &s->inst_off, (size_t)n_inst + 1));
    NN_CUDA(ctx, nn_copy_sync(ctx, s->inst_off, h_offsets, sizeof(int) * (n_inst + 1), cudaMemcpyHostToDevice));
    if (h_grid_sides) {
        s->h_inst_grid.assign(h_grid_sides, h_grid_sides + n_inst);
        const double dt_s = (double)s->cfg.timescale * s->cfg.hp.dt * 1e-3;
        NN_TRY(nn_bpcg_create(ctx, n_inst, h_grid_sides, dt_s * s->cfg.par_D, dt_s * s->cfg.par_decay, &s->bpcg));
        s->G = nn_bpcg_cells(s->bpcg);
        NN_TRY(nn_alloc(ctx, &s->inst_grid, (size_t)n_inst));
        NN_TRY(nn_alloc(ctx, &s->inst_goff, (size_t)n_inst + 1));
        NN_CUDA(ctx, nn_copy_sync(ctx, s->inst_grid, h_grid_sides, sizeof(int) * n_inst, cudaMemcpyHostToDevice));
        NN_CUDA(ctx, nn_copy_sync(ctx, s->inst_goff, nn_bpcg_offsets(s->bpcg), sizeof(int64_t) * (n_inst + 1),
                                cudaMemcpyHostToDevice));
        NN_TRY(nn_alloc(ctx, &s->vox, (size_t)s->n_pad));
        NN_TRY(nn_alloc(ctx, &s->src, (size_t)s->G));
        NN_TRY(nn_alloc(ctx, &s->u, (size_t)s->G));
        NN_TRY(nn_alloc(ctx, &s->b, (size_t)s->G));
        NN_CUDA(ctx, nn_zero_async(ctx, s->vox, sizeof(int32_t) * s->n_pad));
        NN_CUDA(ctx, nn_zero_async(ctx, s->src, sizeof(float) * s->G));
        NN_CUDA(ctx, nn_zero_async(ctx, s->u, sizeof(float) * s->G));
    }
    return NN_OK;
}

extern "C" nn_status nn_sim_get_vox(nn_sim* s, int32_t* h_vox)
{
    if (!s || !h_vox || !s->vox) return NN_ERR_INVALID_ARG;
    NN_CUDA(s->ctx, cudaStreamSynchronize(s->ctx->stream));
    NN_CUDA(s->ctx, nn_copy_sync(s->ctx, h_vox, s->vox, sizeof(int32_t) * s->n, cudaMemcpyDeviceToHost));
    return NN_OK;
}

extern "C" nn_status nn_sim_field_cells(nn_sim* s, int64_t* cells)
{
    if (!s || !cells) return NN_ERR_INVALID_ARG;
    *cells = has_field(s) ? s->G : 0;
    return NN_OK;
}

extern "C" nn_status nn_sim_instance_iterations(nn_sim* s, int* h_iters)
{
    if (!s || !h_iters || s->n_inst < 1) return NN_ERR_INVALID_ARG;
    for (int b = 0; b < s->n_inst; ++b) h_iters[b] = b < (int)s->inst_iters.size() ? s->inst_iters[(size_t)b] : 0;
    return NN_OK;
}

extern "C" nn_status nn_sim_generate_network(nn_sim* s, const nn_net_spec* sp)
{
    if (!s || !sp) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    cudaStream_t cs = ctx->stream;
    const int n = s->n;
    const uint64_t seed = s->cfg.seed;
    free_network(s);
    NN_TRY(nn_alloc(ctx, &s->row_ptr, (size_t)n + 1));
    if (sp->kind == NN_NET_ER) {
        if (!(sp->p >= 0.0 && sp->p <= 1.0)) return nn_fail(ctx, NN_ERR_INVALID_ARG, "ER p outside [0,1]");
        const double tf = std::floor(sp->p * 4294967296.0);
        const uint32_t thr = tf >= 4294967295.0 ? 0xffffffffu : (uint32_t)tf;
        int64_t* cnt = nullptr;
        NN_TRY(nn_alloc(ctx, &cnt, (size_t)n + 1));
        NN_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(int64_t) * ((size_t)n + 1), cs));
        ErRows g{n, thr, seed, nullptr, nullptr, nullptr, 0};
        uint32_t* d_thr = nullptr;
        float* d_wmax = nullptr;
        if (s->n_inst > 0 && sp->inst_p) {
            // a batch: the instances' own probabilities
            std::vector<uint32_t> th((size_t)s->n_inst);
            for (int b = 0; b < s->n_inst; ++b) {
                if (!(sp->inst_p[b] >= 0.0 && sp->inst_p[b] <= 1.0))
                    return nn_fail(ctx, NN_ERR_INVALID_ARG, "instance %d: ER p outside [0,1]", b);
                const double t = std::floor(sp->inst_p[b] * 4294967296.0);
                th[(size_t)b] = t >= 4294967295.0 ? 0xffffffffu : (uint32_t)t;
            }
            NN_TRY(nn_alloc(ctx, &d_thr, th.size()));
            NN_CUDA(ctx, cudaMemcpyAsync(d_thr, th.data(), sizeof(uint32_t) * th.size(), cudaMemcpyHostToDevice, cs));
            g.inst_off = s->inst_off;
            g.inst_thr = d_thr;
            g.n_inst = s->n_inst;
            if (sp->inst_w_max) {
                NN_TRY(nn_alloc(ctx, &d_wmax, (size_t)s->n_inst));
                NN_CUDA(ctx, cudaMemcpyAsync(d_wmax, sp->inst_w_max, sizeof(float) * s->n_inst, cudaMemcpyHostToDevice,
                                             cs));
                g.inst_wmax = d_wmax;
            }
        }
        k_er_count<<<nn_grid_for(ctx, (int64_t)n * 32, 256, 16), 256, 0, cs>>>(g, cnt);
        NN_CHECK_LAUNCH(ctx, "k_er_count");
        NN_TRY(nn_scan_exclusive_i64(ctx, cnt, s->row_ptr, (int64_t)n + 1));
        cudaFree(cnt);
        NN_CUDA(ctx, cudaMemcpyAsync(&s->nnz, s->row_ptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, cs));
        NN_CUDA(ctx, cudaStreamSynchronize(cs));
        const size_t E = (size_t)std::max<int64_t>(s->nnz, 1);
        NN_TRY(nn_alloc(ctx, &s->col, E));
        NN_TRY(nn_alloc(ctx, &s->weight, E));
        NN_TRY(nn_alloc(ctx, &s->delay, E));
        k_er_fill<<<nn_grid_for(ctx, (int64_t)n * 32, 256, 16), 256, 0, cs>>>(g, sp->w_max, s->row_ptr, s->col,
                                                                               s->weight, s->delay);
        NN_CHECK_LAUNCH(ctx, "k_er_fill");
        NN_CUDA(ctx, cudaStreamSynchronize(cs));
        if (d_thr) cudaFree(d_thr);
        if (d_wmax) cudaFree(d_wmax);
    } else if (sp->kind == NN_NET_GAUSS || sp->kind == NN_NET_BLOCK) {
        if (sp->k < 0 || (int64_t)n * sp->k >= ((int64_t)1 << 32))
            return nn_fail(ctx, NN_ERR_INVALID_ARG, "out-degree k out of range");
        s->nnz = (int64_t)n * sp->k;
        std::vector<int64_t> rp((size_t)n + 1);
        for (int i = 0; i <= n; ++i) rp[(size_t)i] = (int64_t)i * sp->k;
        NN_CUDA(ctx, cudaMemcpyAsync(s->row_ptr, rp.data(), sizeof(int64_t) * rp.size(), cudaMemcpyHostToDevice, cs));
        const size_t E = (size_t)std::max<int64_t>(s->nnz, 1);
        NN_TRY(nn_alloc(ctx, &s->col, E));
        NN_TRY(nn_alloc(ctx, &s->weight, E));
        NN_TRY(nn_alloc(ctx, &s->delay, E));
        if (sp->kind == NN_NET_GAUSS) {
            if (sp->dmax < 1 || sp->dmax > s->cfg.max_delay)
                return nn_fail(ctx, NN_ERR_INVALID_ARG, "dmax %d outside [1, max_delay=%d]", sp->dmax, s->cfg.max_delay);
            const int L = nn_lattice_side(n);
            int16_t table[4096];
            nn_host_gauss_table(sp->sigma * (double)L, table);
            int16_t* d_table = nullptr;
            NN_TRY(nn_alloc(ctx, &d_table, 4096));
            NN_CUDA(ctx, cudaMemcpyAsync(d_table, table, sizeof table, cudaMemcpyHostToDevice, cs));
            if (s->nnz)
                k_gauss_fill<<<nn_grid_for(ctx, s->nnz, 256, 16), 256, 0, cs>>>(n, sp->k, L, d_table, seed, sp->w_mu,
                                                                                 sp->w_sigma, sp->dmax, s->col,
                                                                                 s->weight, s->delay);
            NN_CHECK_LAUNCH(ctx, "k_gauss_fill");
            NN_CUDA(ctx, cudaStreamSynchronize(cs));
            cudaFree(d_table);
        } else {
            const int R = sp->n_regions;
            if (R < 1 || R > n || sp->block_dmax < 1 || sp->block_dmax > s->cfg.max_delay)
                return nn_fail(ctx, NN_ERR_INVALID_ARG, "block model: bad region count or delay range");
            std::vector<int> start, size;
            std::vector<uint32_t> cum;
            std::vector<uint8_t> pdel;
            block_tables(n, sp, seed, start, size, cum, pdel);
            std::vector<int> region_of((size_t)n);
            for (int r = 0; r < R; ++r)
                for (int q = 0; q < size[(size_t)r]; ++q) region_of[(size_t)(start[(size_t)r] + q)] = r;
            int *d_rof = nullptr, *d_start = nullptr, *d_size = nullptr;
            uint32_t* d_cum = nullptr;
            uint8_t* d_pd = nullptr;
            NN_TRY(nn_alloc(ctx, &d_rof, (size_t)n));
            NN_TRY(nn_alloc(ctx, &d_start, (size_t)R));
            NN_TRY(nn_alloc(ctx, &d_size, (size_t)R));
            NN_TRY(nn_alloc(ctx, &d_cum, (size_t)R * R));
            NN_TRY(nn_alloc(ctx, &d_pd, (size_t)R * R));
            NN_CUDA(ctx, cudaMemcpyAsync(d_rof, region_of.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, cs));
            NN_CUDA(ctx, cudaMemcpyAsync(d_start, start.data(), sizeof(int) * (size_t)R, cudaMemcpyHostToDevice, cs));
            NN_CUDA(ctx, cudaMemcpyAsync(d_size, size.data(), sizeof(int) * (size_t)R, cudaMemcpyHostToDevice, cs));
            NN_CUDA(ctx, cudaMemcpyAsync(d_cum, cum.data(), sizeof(uint32_t) * cum.size(), cudaMemcpyHostToDevice, cs));
            NN_CUDA(ctx, cudaMemcpyAsync(d_pd, pdel.data(), pdel.size(), cudaMemcpyHostToDevice, cs));
            if (s->nnz)
                k_block_fill<<<nn_grid_for(ctx, s->nnz, 256, 16), 256, 0, cs>>>(n, sp->k, R, d_rof, d_start, d_size,
                                                                                 d_cum, d_pd, seed, sp->w_mu,
                                                                                 sp->w_sigma, s->col, s->weight,
                                                                                 s->delay);
            NN_CHECK_LAUNCH(ctx, "k_block_fill");
            NN_CUDA(ctx, cudaStreamSynchronize(cs));
            cudaFree(d_rof); cudaFree(d_start); cudaFree(d_size); cudaFree(d_cum); cudaFree(d_pd);
        }
    } else {
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "unknown network kind %d", sp->kind);
    }
    NN_CUDA(ctx, cudaMemsetAsync(s->is_inh, 0, (size_t)s->n_pad, cs));
    k_inh<<<nn_grid_for(ctx, n, 256, 16), 256, 0, cs>>>(n, sp->inh_random, sp->inh_fraction, seed, s->is_inh);
    NN_CHECK_LAUNCH(ctx, "k_inh");
    NN_CUDA(ctx, cudaStreamSynchronize(cs));
    return after_network(s);
}

extern "C" nn_status nn_sim_network_size(nn_sim* s, int64_t* nnz)
{
    if (!s || !nnz) return NN_ERR_INVALID_ARG;
    *nnz = s->nnz;
    return NN_OK;
}

extern "C" nn_status nn_sim_get_network(nn_sim* s, int64_t* h_row_ptr, int32_t* h_col, float* h_weight,
                                        uint8_t* h_delay, uint8_t* h_is_inh)
{
    if (!s) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    cudaStream_t cs = ctx->stream;
    if (!s->row_ptr) return nn_fail(ctx, NN_ERR_INVALID_ARG, "no network set");
    if (h_row_ptr) NN_CUDA(ctx, cudaMemcpyAsync(h_row_ptr, s->row_ptr, sizeof(int64_t) * ((size_t)s->n + 1), cudaMemcpyDeviceToHost, cs));
    if (s->nnz) {
        if (h_col) NN_CUDA(ctx, cudaMemcpyAsync(h_col, s->col, sizeof(int32_t) * (size_t)s->nnz, cudaMemcpyDeviceToHost, cs));
        if (h_weight) NN_CUDA(ctx, cudaMemcpyAsync(h_weight, s->weight, sizeof(float) * (size_t)s->nnz, cudaMemcpyDeviceToHost, cs));
        if (h_delay) NN_CUDA(ctx, cudaMemcpyAsync(h_delay, s->delay, (size_t)s->nnz, cudaMemcpyDeviceToHost, cs));
    }
    if (h_is_inh) NN_CUDA(ctx, cudaMemcpyAsync(h_is_inh, s->is_inh, (size_t)s->n, cudaMemcpyDeviceToHost, cs));
    NN_CUDA(ctx, cudaStreamSynchronize(cs));
    return NN_OK;
}

extern "C" nn_status nn_sim_get_csc(nn_sim* s, int64_t* h_col_ptr, int32_t* h_src, float* h_weight, uint8_t* h_delay)
{
    if (!s) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    if (!s->row_ptr) return nn_fail(ctx, NN_ERR_INVALID_ARG, "no network set");
    NN_TRY(build_csc(s));
    cudaStream_t cs = ctx->stream;
    if (h_col_ptr) NN_CUDA(ctx, cudaMemcpyAsync(h_col_ptr, s->col_ptr, sizeof(int64_t) * ((size_t)s->n + 1), cudaMemcpyDeviceToHost, cs));
    if (s->nnz) {
        if (h_src) NN_CUDA(ctx, cudaMemcpyAsync(h_src, s->csc_src, sizeof(uint32_t) * (size_t)s->nnz, cudaMemcpyDeviceToHost, cs));
        if (h_weight) NN_CUDA(ctx, cudaMemcpyAsync(h_weight, s->csc_w, sizeof(float) * (size_t)s->nnz, cudaMemcpyDeviceToHost, cs));
        if (h_delay) NN_CUDA(ctx, cudaMemcpyAsync(h_delay, s->csc_d, (size_t)s->nnz, cudaMemcpyDeviceToHost, cs));
    }
    NN_CUDA(ctx, cudaStreamSynchronize(cs));
    if (h_src)
        for (int64_t e = 0; e < s->nnz; ++e) h_src[e] &= 0x7fffffff;
    return NN_OK;
}

extern "C" float* nn_sim_field_ptr(nn_sim* s, int field)
{
    if (!s || field < 0 || field >= NN_F_COUNT) return nullptr;
    return s->f[field];
}

extern "C" nn_status nn_sim_set_field(nn_sim* s, int field, const float* h)
{
    if (!s || !h || field < 0 || field >= NN_F_COUNT) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    NN_CUDA(ctx, cudaMemcpyAsync(s->f[field], h, sizeof(float) * (size_t)s->n, cudaMemcpyHostToDevice, ctx->stream));
    if (field == NN_F_GNA_SCALE && !s->gna_set) {
        s->gna_set = true;
        drop_graph(s);  // the captured kernels' arguments change
    }
    if ((field == NN_F_X || field == NN_F_Y || field == NN_F_Z) && s->bpcg) {
        k_inst_vox<<<nn_grid_for(ctx, s->n, 256, 16), 256, 0, ctx->stream>>>(
            s->f[NN_F_X], s->f[NN_F_Y], s->f[NN_F_Z], s->n, s->inst_off, s->n_inst, s->inst_grid, s->inst_goff, s->vox);
        NN_CHECK_LAUNCH(ctx, "k_inst_vox");
    }
    if ((field == NN_F_X || field == NN_F_Y || field == NN_F_Z) && s->grid > 0) {
        k_vox<<<nn_grid_for(ctx, s->n, 256, 16), 256, 0, ctx->stream>>>(s->f[NN_F_X], s->f[NN_F_Y], s->f[NN_F_Z], s->n,
                                                                         s->grid, s->vox);
        NN_CHECK_LAUNCH(ctx, "k_vox");
    }
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return NN_OK;
}

static nn_status check_err(nn_sim* s)
{
    int e = 0;
    NN_CUDA(s->ctx, cudaMemcpyAsync(&e, s->err, sizeof(int), cudaMemcpyDeviceToHost, s->ctx->stream));
    NN_CUDA(s->ctx, cudaStreamSynchronize(s->ctx->stream));
    if (e & 2) return nn_fail(s->ctx, NN_ERR_TIMEOUT, "pull delivery: a bitmap-copy wait gave up");
    if (e) return nn_fail(s->ctx, NN_ERR_NUMERIC, "non-finite membrane potential detected");
    return NN_OK;
}

extern "C" nn_status nn_sim_get_field(nn_sim* s, int field, float* h)
{
    if (!s || !h || field < 0 || field >= NN_F_COUNT) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    NN_CUDA(ctx, cudaMemcpyAsync(h, s->f[field], sizeof(float) * (size_t)s->n, cudaMemcpyDeviceToHost, ctx->stream));
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return check_err(s);
}

extern "C" nn_status nn_sim_init_state(nn_sim* s, float v0, float i_lo, float i_hi)
{
    if (!s) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    // steady-state gates at v0 (double precision on the host)
    auto xr = [](double u) { return std::fabs(u) < 1e-4 ? 1.0 + 0.5 * u + u * u / 12.0 : u / (-std::expm1(-u)); };
    const double V = v0;
    const double am = xr((V + 40.0) / 10.0), bm = 4.0 * std::exp(-(V + 65.0) / 18.0);
    const double ah = 0.07 * std::exp(-(V + 65.0) / 20.0), bh = 1.0 / (1.0 + std::exp(-(V + 35.0) / 10.0));
    const double an = 0.1 * xr((V + 55.0) / 10.0), bn = 0.125 * std::exp(-(V + 65.0) / 80.0);
    StepArgs a = step_args(s, 0);
    const int L = nn_lattice_side(s->n);
    k_init_state<<<nn_grid_for(ctx, s->n_pad, 256, 16), 256, 0, ctx->stream>>>(
        a, v0, (float)(am / (am + bm)), (float)(ah / (ah + bh)), (float)(an / (an + bn)), i_lo, i_hi, s->f[NN_F_X],
        s->f[NN_F_Y], s->f[NN_F_Z], s->f[NN_F_GNA_SCALE], L, s->grid, s->grid > 0 ? s->vox : nullptr);
    NN_CHECK_LAUNCH(ctx, "k_init_state");
    if (s->n_inst > 0) {
        k_inst_positions<<<nn_grid_for(ctx, s->n, 256, 16), 256, 0, ctx->stream>>>(
            s->n, s->inst_off, s->n_inst, s->cfg.seed, s->f[NN_F_X], s->f[NN_F_Y], s->f[NN_F_Z]);
        NN_CHECK_LAUNCH(ctx, "k_inst_positions");
        if (s->bpcg) {
            k_inst_vox<<<nn_grid_for(ctx, s->n, 256, 16), 256, 0, ctx->stream>>>(
                s->f[NN_F_X], s->f[NN_F_Y], s->f[NN_F_Z], s->n, s->inst_off, s->n_inst, s->inst_grid, s->inst_goff,
                s->vox);
            NN_CHECK_LAUNCH(ctx, "k_inst_vox");
        }
    }
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return NN_OK;
}

// Enqueue one step: the neuron update (with push delivery inline), plus the
// pull gather in pull mode.  qk: the step's offset from the device step base;
// qe: its timing-event slot.
static nn_status enqueue_step(nn_sim* s, int qk, int qe)
{
    nn_ctx* ctx = s->ctx;
    cudaStream_t cs = ctx->stream;
    const bool tm = s->timing && qe >= 0 && qe < (int)s->ev_a.size();
    if (tm) NN_CUDA(ctx, cudaEventRecordWithFlags(s->ev_a[qe], cs, cudaEventRecordExternal));
    StepArgs a = step_args(s, qk);
    const int warps_needed = s->n_pad / (32 * s->npt);
    const int blocks = std::max(1, std::min((warps_needed * 32 + s->tpb - 1) / s->tpb, ctx->num_sms * 16));
    NN_CUDA(ctx, nn_launch_hh_step(a, s->npt, blocks, s->tpb, cs));
    NN_CHECK_LAUNCH(ctx, "k_hh_step");
    if (tm) NN_CUDA(ctx, cudaEventRecordWithFlags(s->ev_b[qe], cs, cudaEventRecordExternal));
    if (s->cfg.delivery == NN_DELIVERY_PULL) {
        NN_TRY(launch_pull(s, pull_args(s, qk, false), cs));
    } else if (s->cfg.delivery == NN_DELIVERY_AUTO && s->cur_mode == 1) {
        NN_TRY(launch_pull(s, pull_args(s, qk, true), cs));
    }
    if (tm) {
        NN_CUDA(ctx, cudaEventRecordWithFlags(s->ev_c[qe], cs, cudaEventRecordExternal));
        s->ev_valid[qe] = 1;
    }
    return NN_OK;
}

static int launches_per_step(const nn_sim* s)
{
    return s->cfg.delivery == NN_DELIVERY_PULL || (s->cfg.delivery == NN_DELIVERY_AUTO && s->cur_mode == 1) ? 2 : 1;
}

static nn_status enqueue_advance(nn_sim* s, int steps)
{
    k_advance<<<1, 1, 0, s->ctx->stream>>>(s->step, steps);
    NN_CHECK_LAUNCH(s->ctx, "k_advance");
    return NN_OK;
}

extern "C" nn_status nn_sim_set_kernel_timing(nn_sim* s, int enable)
{
    if (!s) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    const int P = has_field(s) ? s->cfg.timescale : 50;
    drop_graph(s);
    s->timing = enable != 0;
    if (s->timing && (int)s->ev_a.size() < P) {
        while ((int)s->ev_a.size() < P) {
            cudaEvent_t a, b, c;
            NN_CUDA(ctx, cudaEventCreate(&a));
            NN_CUDA(ctx, cudaEventCreate(&b));
            NN_CUDA(ctx, cudaEventCreate(&c));
            s->ev_a.push_back(a);
            s->ev_b.push_back(b);
            s->ev_c.push_back(c);
        }
    }
    s->ev_valid.assign(s->ev_a.size(), 0);
    if (s->pcg) nn_pcg_set_timing(s->pcg, s->timing);
    if (s->bpcg) nn_bpcg_set_timing(s->bpcg, s->timing);
    return NN_OK;
}

extern "C" nn_status nn_sim_kernel_times(nn_sim* s, nn_kernel_times* out)
{
    if (!s || !out) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double hh = 0.0, dl = 0.0;
    int cnt = 0;
    std::vector<float> hv, dv;
    for (size_t q = 0; q < s->ev_valid.size(); ++q) {
        if (!s->ev_valid[q]) continue;
        float a = 0.0f, b = 0.0f;
        NN_CUDA(ctx, cudaEventElapsedTime(&a, s->ev_a[q], s->ev_b[q]));
        NN_CUDA(ctx, cudaEventElapsedTime(&b, s->ev_b[q], s->ev_c[q]));
        hh += a;
        dl += b;
        hv.push_back(a);
        dv.push_back(b);
        ++cnt;
    }
    out->hh_step_ms = cnt ? (float)(hh / cnt) : 0.0f;
    out->deliver_ms = cnt ? (float)(dl / cnt) : 0.0f;
    out->samples = cnt;
    auto median = [](std::vector<float>& v) {
        if (v.empty()) return 0.0f;
        std::nth_element(v.begin(), v.begin() + v.size() / 2, v.end());
        return v[v.size() / 2];
    };
    out->hh_step_median_ms = median(hv);
    out->deliver_median_ms = median(dv);
    out->solve_ms = 0.0f;
    out->solve_iterations = 0;
    if (s->pcg) nn_pcg_last_timing(s->pcg, &out->solve_ms, &out->solve_iterations);
    if (s->bpcg) nn_bpcg_last_timing(s->bpcg, &out->solve_ms, &out->solve_iterations);
    return NN_OK;
}

// The field solve overlaps the next period's steps when the field does not
// feed back into the neurons -- except while kernel timing is on, so that
// each kernel is timed alone.
static bool overlap_solve(const nn_sim* s)
{
    return s->cfg.par_overlap && s->cfg.hp.g_par == 0.0f && !s->timing &&
           (s->bpcg != nullptr || (s->pcg && nn_pcg_async_supported(s->pcg)));
}

// Complete an overlapped solve: wait for its stream, finish it if the
// enqueued iterations were not enough, record its statistics.
static nn_status finish_solve(nn_sim* s)
{
    if (!s->solve_pending) return NN_OK;
    s->solve_pending = false;
    int it = 0, conv = 0;
    double rel = 0.0;
    if (s->bpcg) {
        int unconv = 0;
        s->inst_iters.assign((size_t)s->n_inst, 0);
        NN_TRY(nn_bpcg_async_finish(s->bpcg, s->inst_iters.data(), &it, &unconv));
        conv = unconv == 0;
        s->iter_estimate = it + 2;  // the batch stops with its slowest instance
    } else {
        NN_TRY(nn_pcg_async_finish(s->pcg, &it, &rel, &conv));
        s->iter_estimate = it + 8;
    }
    s->stats.iterations = it;
    s->stats.relres = rel;
    s->stats.converged = conv;
    return NN_OK;
}

static nn_status paracrine_solve(nn_sim* s)
{
    nn_ctx* ctx = s->ctx;
    cudaStream_t cs = ctx->stream;
    const bool overlap = overlap_solve(s);
    if (overlap) {
        // the previous overlapped solve must be complete before b and u are reused
        NN_TRY(finish_solve(s));
        if (!s->par_stream) {
            NN_CUDA(ctx, cudaStreamCreateWithFlags(&s->par_stream, cudaStreamNonBlocking));
            NN_CUDA(ctx, cudaEventCreateWithFlags(&s->ev_rhs, cudaEventDisableTiming));
            NN_CUDA(ctx, cudaEventCreateWithFlags(&s->ev_solved, cudaEventDisableTiming));
        }
        NN_CUDA(ctx, cudaStreamWaitEvent(cs, s->ev_solved, 0));
    }
    k_par_rhs<<<nn_grid_for(ctx, s->G, 256, 8), 256, 0, cs>>>(s->u, s->src, s->b, s->u_prev, s->have_prev ? 1 : 0,
                                                               s->G);
    s->have_prev = s->u_prev != nullptr;
    NN_CHECK_LAUNCH(ctx, "k_par_rhs");
    if (overlap) {
        NN_CUDA(ctx, cudaEventRecord(s->ev_rhs, cs));
        NN_CUDA(ctx, cudaStreamWaitEvent(s->par_stream, s->ev_rhs, 0));
        if (s->bpcg)
            NN_TRY(nn_bpcg_async_begin(s->bpcg, s->b, s->u, s->cfg.par_rtol, s->cfg.par_max_iter, s->iter_estimate,
                                       s->par_stream));
        else
            NN_TRY(nn_pcg_async_begin(s->pcg, s->b, s->u, s->cfg.par_rtol, s->cfg.par_max_iter, s->iter_estimate,
                                      s->par_stream));
        NN_CUDA(ctx, cudaEventRecord(s->ev_solved, s->par_stream));
        s->solve_pending = true;
        s->stats.solves += 1;
        return NN_OK;
    }
    int it = 0, conv = 0;
    double rel = 0.0;
    if (s->bpcg) {
        int unconv = 0;
        s->inst_iters.assign((size_t)s->n_inst, 0);
        NN_TRY(nn_bpcg_solve(s->bpcg, s->b, s->u, s->cfg.par_rtol, s->cfg.par_max_iter, s->inst_iters.data(), &it,
                             &unconv));
        conv = unconv == 0;
    } else {
        NN_TRY(nn_pcg_run_best(s->pcg, s->b, s->u, s->cfg.par_rtol, s->cfg.par_max_iter, &it, &rel, &conv));
    }
    s->stats.iterations = it;
    s->stats.relres = rel;
    s->stats.converged = conv;
    s->stats.solves += 1;
    if (s->cfg.hp.g_par != 0.0f) {
        k_par_gather<<<nn_grid_for(ctx, s->n, 256, 16), 256, 0, cs>>>(s->u, s->vox, s->f[NN_F_UPAR], s->n);
        NN_CHECK_LAUNCH(ctx, "k_par_gather");
    }
    return NN_OK;
}

// Steps per captured graph: one paracrine period, or 50 steps without a field.
static int period_steps(const nn_sim* s) { return has_field(s) ? s->cfg.timescale : 50; }

static nn_status ensure_graph(nn_sim* s)
{
    cudaGraphExec_t* slot = s->cur_mode == 1 ? &s->graph_pull : &s->graph;
    if (*slot) return NN_OK;
    nn_ctx* ctx = s->ctx;
    cudaStream_t cs = ctx->stream;
    const int P = period_steps(s);
    const int64_t launches0 = ctx->launches;
    NN_CUDA(ctx, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    nn_status st = NN_OK;
    for (int q = 0; q < P && st == NN_OK; ++q) st = enqueue_step(s, q, q);
    if (st == NN_OK) st = enqueue_advance(s, P);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(cs, &g);
    ctx->launches = launches0;
    if (st != NN_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return nn_cuda_check(ctx, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(slot, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        *slot = nullptr;
        return nn_cuda_check(ctx, e, "cudaGraphInstantiate");
    }
    s->graph_steps = P;
    return NN_OK;
}

// Launch-shape autotuner for the neuron update: time trial steps of every
// (threads per block, neurons per thread) candidate on this simulation's own
// network and state, keep the fastest, and restore the state the trials
// changed (neuron fields, delay ring, spike counters and lists, bitmap,
// deposits).  The step counter is restored too, so the trials leave no trace.
// Copy of every device buffer that steps of the simulation write (neuron
// fields, delay ring, bitmap and row flags, spike lists and counters, step
// counter, deposits, the field and its right-hand side, electrode samples),
// for trials that must leave no trace.
struct SimSnapshot {
    struct Buf { void* dst; const void* src; size_t bytes; };
    std::vector<Buf> keep;
};

static nn_status snapshot_take(nn_sim* s, SimSnapshot& snap)
{
    nn_ctx* ctx = s->ctx;
    cudaStream_t cs = ctx->stream;
    const size_t NP = (size_t)s->n_pad;
    auto save = [&](const void* p, size_t bytes) -> nn_status {
        if (!p || !bytes) return NN_OK;
        unsigned char* d = nullptr;
        NN_TRY(nn_alloc(ctx, &d, bytes));
        snap.keep.push_back({d, p, bytes});
        NN_CUDA(ctx, cudaMemcpyAsync(d, p, bytes, cudaMemcpyDeviceToDevice, cs));
        return NN_OK;
    };
    nn_status st = NN_OK;
    for (int q = 0; q < NN_F_COUNT && st == NN_OK; ++q) st = save(s->f[q], NP * sizeof(float));
    if (st == NN_OK) st = save(s->ring, (size_t)s->D * NP * sizeof(float2));
    if (st == NN_OK) st = save(s->bitmap, s->bitmap ? (size_t)s->D * s->words * sizeof(uint32_t) : 0);
    if (st == NN_OK) st = save(s->rowflag, s->rowflag ? (size_t)s->D * sizeof(int) : 0);
    if (st == NN_OK) st = save(s->list, 2 * NP * sizeof(int));
    if (st == NN_OK) st = save(s->counts, 2 * sizeof(int));
    if (st == NN_OK) st = save(s->step, sizeof(unsigned long long));
    if (st == NN_OK) st = save(s->total, sizeof(unsigned long long));
    if (st == NN_OK) st = save(s->rcount, sizeof(unsigned long long));
    if (st == NN_OK) st = save(s->src, has_field(s) ? (size_t)s->G * sizeof(float) : 0);
    if (st == NN_OK) st = save(s->u, s->u ? (size_t)s->G * sizeof(float) : 0);
    if (st == NN_OK) st = save(s->u_prev, s->u_prev ? (size_t)s->G * sizeof(float) : 0);
    if (st == NN_OK) st = save(s->b, s->b ? (size_t)s->G * sizeof(float) : 0);
    if (st == NN_OK) st = save(s->el_val, (size_t)s->el_cap * s->el_members * sizeof(float));
    if (st == NN_OK) st = save(s->el_spk, (size_t)s->el_cap * s->el_members);
    return st;
}

static nn_status snapshot_restore(nn_sim* s, const SimSnapshot& snap)
{
    for (const auto& b : snap.keep)
        NN_CUDA(s->ctx, cudaMemcpyAsync((void*)b.src, b.dst, b.bytes, cudaMemcpyDeviceToDevice, s->ctx->stream));
    return NN_OK;
}

static void snapshot_free(SimSnapshot& snap)
{
    for (const auto& b : snap.keep) cudaFree(b.dst);
    snap.keep.clear();
}

extern "C" nn_status nn_sim_autotune(nn_sim* s, int trial_steps, int* best_tpb, int* best_npt, float* best_ms)
{
    if (!s || trial_steps < 1) return NN_ERR_INVALID_ARG;
    if (!s->row_ptr) return nn_fail(s->ctx, NN_ERR_INVALID_ARG, "nn_sim_autotune: no network set");
    nn_ctx* ctx = s->ctx;
    cudaStream_t cs = ctx->stream;
    // a pending overlapped solve writes the field the snapshot holds
    NN_TRY(finish_solve(s));
    if (s->ev_solved) NN_CUDA(ctx, cudaStreamWaitEvent(cs, s->ev_solved, 0));
    SimSnapshot snap;
    nn_status st = snapshot_take(s, snap);
    const int old_tpb = s->tpb, old_npt = s->npt;
    const bool old_timing = s->timing;
    s->timing = false;
    float best = 1e30f;
    int btpb = old_tpb, bnpt = old_npt;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventCreate(&e0), "event");
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventCreate(&e1), "event");
    for (int npt : {1, 2, 4}) {
        for (int tpb : {64, 128, 256}) {
            if (st != NN_OK) break;
            s->tpb = tpb;
            s->npt = npt;
            // restore, warm once, then time
            if (st == NN_OK) st = snapshot_restore(s, snap);
            if (st == NN_OK) st = enqueue_step(s, 0, -1);
            if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventRecord(e0, cs), "event");
            for (int q = 0; q < trial_steps && st == NN_OK; ++q) st = enqueue_step(s, 0, -1);
            if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventRecord(e1, cs), "event");
            float ms = 0.0f;
            if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventSynchronize(e1), "event");
            if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventElapsedTime(&ms, e0, e1), "event");
            ms /= trial_steps;
            if (st == NN_OK && ms < best) {
                best = ms;
                btpb = tpb;
                bnpt = npt;
            }
        }
    }
    if (st == NN_OK) st = snapshot_restore(s, snap);
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaStreamSynchronize(cs), "nn_sim_autotune");
    snapshot_free(snap);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    s->timing = old_timing;
    s->tpb = st == NN_OK ? btpb : old_tpb;
    s->npt = st == NN_OK ? bnpt : old_npt;
    drop_graph(s);
    if (best_tpb) *best_tpb = s->tpb;
    if (best_npt) *best_npt = s->npt;
    if (best_ms) *best_ms = best;
    return st;
}

// Automatic delivery.  After each period the spike total is copied to
// pinned memory behind an event; the periods whose events have completed
// give the measured rate (spikes per neuron and step), without waiting for
// the device unless TOT_Q periods are outstanding.
// Fold the completed spike-total measurements into the measured rate, oldest
// first (all of them once the stream is synchronised).
static nn_status fold_totals(nn_sim* s)
{
    while (s->tot_pending > 0) {
        const int k = s->tot_head;
        const cudaError_t q = cudaEventQuery(s->ev_tot[k]);
        if (q == cudaErrorNotReady) break;
        NN_CUDA(s->ctx, q);
        const unsigned long long tot = s->h_tot[k];
        if (s->base_step >= 0 && s->tot_step[k] > s->base_step)
            s->last_rate = (float)((double)(tot - s->base_tot) / ((double)(s->tot_step[k] - s->base_step) * s->n));
        s->base_tot = tot;
        s->base_step = s->tot_step[k];
        s->tot_head = (k + 1) % nn_sim::TOT_Q;
        --s->tot_pending;
    }
    return NN_OK;
}

static nn_status record_total(nn_sim* s)
{
    nn_ctx* ctx = s->ctx;
    if (s->tot_pending == nn_sim::TOT_Q) {
        NN_CUDA(ctx, cudaEventSynchronize(s->ev_tot[s->tot_head]));
    }
    NN_TRY(fold_totals(s));
    const int k = (s->tot_head + s->tot_pending) % nn_sim::TOT_Q;
    NN_CUDA(ctx, cudaMemcpyAsync(&s->h_tot[k], s->total, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    NN_CUDA(ctx, cudaEventRecord(s->ev_tot[k], ctx->stream));
    s->tot_step[k] = s->host_step;
    ++s->tot_pending;
    return NN_OK;
}

// The next period's mode from the latest measured rate.  Leaving pull
// delivery scatters the pull spikes still in flight (k_flush_pull) and clears
// the row flags; entering it needs nothing (the pull gather skips the rows of
// pushed steps).
static nn_status choose_delivery(nn_sim* s)
{
    nn_ctx* ctx = s->ctx;
    cudaStream_t cs = ctx->stream;
    const int want = s->last_rate >= 0.0f && s->last_rate >= s->cfg.pull_rate ? 1 : 0;
    if (s->cur_mode == 1 && want == 0) {
        const dim3 grid((unsigned)((s->words + 7) / 8), (unsigned)s->D);
        k_flush_pull<<<grid, 256, 0, cs>>>(s->bitmap, s->rowflag, s->row_ptr, s->col, s->weight, s->delay, s->is_inh,
                                          reinterpret_cast<float*>(s->ring), s->n, s->n_pad, s->D, s->words,
                                          (long long)s->host_step);
        NN_CHECK_LAUNCH(ctx, "k_flush_pull");
        NN_CUDA(ctx, cudaMemsetAsync(s->rowflag, 0, (size_t)s->D * sizeof(int), cs));
    }
    s->cur_mode = want;
    s->mode_log.push_back((int8_t)want);
    s->rate_log.push_back(s->last_rate);
    return NN_OK;
}

extern "C" nn_status nn_sim_delivery_log(nn_sim* s, int8_t* h_modes, float* h_rates, int cap, int* count, int reset)
{
    if (!s || !count || cap < 0) return NN_ERR_INVALID_ARG;
    const int m = (int)s->mode_log.size();
    for (int i = 0; i < std::min(cap, m); ++i) {
        if (h_modes) h_modes[i] = s->mode_log[(size_t)i];
        if (h_rates) h_rates[i] = s->rate_log[(size_t)i];
    }
    *count = m;
    if (reset) {
        s->mode_log.clear();
        s->rate_log.clear();
    }
    return NN_OK;
}

// Block shape of the overlapped field solve (a single grid's tile depth, a
// batch's cells per block), chosen by the time of whole periods: the solve
// shares the GPU with the next period's neuron updates, so the shape fastest
// alone need not be fastest beside them.  Each candidate runs six periods
// from the same snapshot of the simulation (restored after each, and at the
// end, with the step counters and the delivery bookkeeping).
static nn_status autotune_overlapped_tiles(nn_sim* s, int* shape, float* ms_per_step)
{
    const bool batch = s->bpcg != nullptr;
    nn_ctx* ctx = s->ctx;
    cudaStream_t cs = ctx->stream;
    // fold the pending spike totals, so the automatic delivery's state is all on the host
    NN_CUDA(ctx, cudaStreamSynchronize(cs));
    NN_TRY(fold_totals(s));
    SimSnapshot snap;
    nn_status st = snapshot_take(s, snap);
    const int64_t host_step = s->host_step;
    const int cur_mode = s->cur_mode, tot_head = s->tot_head, iter_estimate = s->iter_estimate;
    const float last_rate = s->last_rate;
    const unsigned long long base_tot = s->base_tot;
    const int64_t base_step = s->base_step;
    const size_t nlog = s->mode_log.size();
    const nn_solve_stats stats = s->stats;
    const bool have_prev = s->have_prev;
    auto restore_host = [&]() {
        s->host_step = host_step;
        s->cur_mode = cur_mode;
        s->tot_head = tot_head;
        s->tot_pending = 0;
        s->last_rate = last_rate;
        s->base_tot = base_tot;
        s->base_step = base_step;
        s->mode_log.resize(nlog);
        s->rate_log.resize(nlog);
        s->stats = stats;
        s->iter_estimate = iter_estimate;
        s->have_prev = have_prev;
    };
    const int P = period_steps(s);
    const int zc0 = batch ? nn_bpcg_cells_per_block(s->bpcg) : nn_pcg_tile_depth(s->pcg);
    auto set_shape = [&](int v) -> nn_status {
        if (batch) return nn_bpcg_set_cells_per_block(s->bpcg, v);
        nn_pcg_set_tile_depth(s->pcg, v);
        return NN_OK;
    };
    int best_zc = zc0;
    float best = 1e30f;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventCreate(&e0), "event");
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventCreate(&e1), "event");
    std::vector<int> cands;
    if (batch) {
        cands = {512, 1024, 2048, 4096};
    } else {
        int nz = 0, d0 = 0, d1 = 0;
        nn_ctx* c_ = nullptr;
        const float* i_ = nullptr;
        const float* D_ = nullptr;
        float ic_ = 0.0f;
        nn_pcg_info(s->pcg, &c_, &d0, &d1, &nz, &i_, &ic_, &D_);
        int prev = 0;
        for (int zc : {4, 6, 8, 12, 16, 24, 32}) {
            if (prev >= nz) break;  // deeper tiles than the grid change nothing
            prev = zc;
            cands.push_back(zc);
        }
    }
    for (int zc : cands) {
        if (st != NN_OK) break;
        st = set_shape(zc);
        if (st == NN_OK) st = snapshot_restore(s, snap);
        restore_host();
        if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventRecord(e0, cs), "event");
        if (st == NN_OK) st = nn_sim_step(s, 6 * P);  // returns with its last solve finished
        if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventRecord(e1, cs), "event");
        float ms = 0.0f;
        if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventSynchronize(e1), "event");
        if (st == NN_OK) st = nn_cuda_check(ctx, cudaEventElapsedTime(&ms, e0, e1), "event");
        if (st == NN_OK) st = nn_cuda_check(ctx, cudaStreamSynchronize(cs), "sync");
        // fold the trial's spike totals away before the next restore
        while (s->tot_pending > 0) {
            s->tot_head = (s->tot_head + 1) % nn_sim::TOT_Q;
            --s->tot_pending;
        }
        if (st == NN_OK && ms < best) {
            best = ms;
            best_zc = zc;
        }
    }
    const nn_status st3 = set_shape(st == NN_OK ? best_zc : zc0);
    if (st == NN_OK) st = st3;
    const nn_status st2 = snapshot_restore(s, snap);
    restore_host();
    if (st == NN_OK) st = st2;
    if (st == NN_OK) st = nn_cuda_check(ctx, cudaStreamSynchronize(cs), "autotune_overlapped_tiles");
    snapshot_free(snap);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (shape) *shape = batch ? nn_bpcg_cells_per_block(s->bpcg) : nn_pcg_tile_depth(s->pcg);
    if (ms_per_step) *ms_per_step = best < 1e30f ? best / (6.0f * P) : 0.0f;
    return st;
}

extern "C" nn_status nn_sim_autotune_solver(nn_sim* s, int trial_iters, int* shape, float* ms_per_iter)
{
    if (!s || trial_iters < 1) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    if (!s->pcg && !s->bpcg) return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_sim_autotune_solver: no paracrine field");
    // a pending overlapped solve owns the solver's work vectors
    NN_TRY(finish_solve(s));
    if (s->ev_solved) NN_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, s->ev_solved, 0));
    if (s->pcg) {
        if (!s->row_ptr || !overlap_solve(s) || nn_pcg_tile_depth(s->pcg) == 0)
            return nn_pcg_autotune_tiles(s->pcg, trial_iters, shape, ms_per_iter);
        return autotune_overlapped_tiles(s, shape, ms_per_iter);
    }
    if (s->row_ptr && overlap_solve(s)) return autotune_overlapped_tiles(s, shape, ms_per_iter);
    float *b = nullptr, *x = nullptr;
    const int64_t G = s->G;
    NN_TRY(nn_alloc(ctx, &b, (size_t)G));
    nn_status st = nn_alloc(ctx, &x, (size_t)G);
    if (st == NN_OK) {
        k_fill_f<<<nn_grid_for(ctx, G, 256), 256, 0, ctx->stream>>>(b, G, 1.0f);
        st = nn_cuda_check(ctx, cudaPeekAtLastError(), "k_fill_f");
    }
    if (st == NN_OK) st = nn_bpcg_autotune(s->bpcg, b, x, trial_iters, shape, ms_per_iter);
    cudaStreamSynchronize(ctx->stream);
    nn_release(b);
    nn_release(x);
    return st;
}

extern "C" nn_status nn_sim_set_pull_rate(nn_sim* s, float pull_rate)
{
    if (!s || !(pull_rate >= 0.0f)) return NN_ERR_INVALID_ARG;
    if (s->cfg.delivery != NN_DELIVERY_AUTO)
        return nn_fail(s->ctx, NN_ERR_INVALID_ARG, "nn_sim_set_pull_rate: the simulation is not in automatic delivery");
    s->cfg.pull_rate = pull_rate;
    return NN_OK;
}

extern "C" nn_status nn_sim_step(nn_sim* s, int nsteps)
{
    if (!s || nsteps < 0) return NN_ERR_INVALID_ARG;
    if (!s->row_ptr) return nn_fail(s->ctx, NN_ERR_INVALID_ARG, "nn_sim_step: no network set");
    nn_ctx* ctx = s->ctx;
    const int P = period_steps(s);
    int left = nsteps;
    const bool autod = s->cfg.delivery == NN_DELIVERY_AUTO;
    while (left > 0) {
        const bool aligned = (s->host_step % P) == 0;
        if (aligned && left >= P) {
            if (autod) NN_TRY(choose_delivery(s));
            NN_TRY(ensure_graph(s));
            NN_CUDA(ctx, cudaGraphLaunch(s->cur_mode == 1 ? s->graph_pull : s->graph, ctx->stream));
            ctx->launches += (int64_t)launches_per_step(s) * P + 1;
            s->host_step += P;
            left -= P;
            if (autod) NN_TRY(record_total(s));
        } else {
            NN_TRY(enqueue_step(s, 0, (int)(s->host_step % P)));
            NN_TRY(enqueue_advance(s, 1));
            s->host_step += 1;
            left -= 1;
        }
        if (has_field(s) && (s->host_step % s->cfg.timescale) == 0) NN_TRY(paracrine_solve(s));
    }
    // the call's last overlapped solve completes before it returns, and the
    // main stream is ordered after it
    if (s->solve_pending) {
        NN_TRY(finish_solve(s));
        NN_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, s->ev_solved, 0));
    }
    return NN_OK;
}

extern "C" nn_status nn_sim_pull_info(nn_sim* s, int* sliced, int* cols)
{
    if (!s || !sliced || !cols) return NN_ERR_INVALID_ARG;
    *sliced = s->dsl_chunk ? 1 : 0;
    *cols = s->dsl_chunk ? s->dsl_cols : 0;
    return NN_OK;
}

extern "C" nn_status nn_sim_deliver_spikes(nn_sim* s, const int* d_list, int count, int mode)
{
    if (!s || (count > 0 && !d_list) || count < 0 || count > s->n) return NN_ERR_INVALID_ARG;
    if (!s->row_ptr) return nn_fail(s->ctx, NN_ERR_INVALID_ARG, "nn_sim_deliver_spikes: no network");
    nn_ctx* ctx = s->ctx;
    cudaStream_t cs = ctx->stream;
    if (mode == NN_DELIVERY_PUSH) {
        if (count == 0) return NN_OK;
        k_deliver_list<<<nn_grid_for(ctx, (int64_t)count * 32, DELIV_THREADS, 16), DELIV_THREADS, 0, cs>>>(
            d_list, count, s->row_ptr, s->col, s->weight, s->delay, s->is_inh, reinterpret_cast<float*>(s->ring),
            s->step, s->n_pad, s->D);
        NN_CHECK_LAUNCH(ctx, "k_deliver_list");
        return NN_OK;
    }
    if (mode != NN_DELIVERY_PULL) return NN_ERR_INVALID_ARG;
    if (!s->bitmap || !s->col_ptr)
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_sim_deliver_spikes: pull needs a simulation in pull mode");
    NN_CUDA(ctx, cudaMemsetAsync(s->bitmap, 0, sizeof(uint32_t) * (size_t)s->D * s->words, cs));
    if (count > 0) {
        k_list_bitmap<<<nn_grid_for(ctx, count, 256, 4), 256, 0, cs>>>(d_list, count, s->bitmap, s->step, s->D,
                                                                       s->words);
        NN_CHECK_LAUNCH(ctx, "k_list_bitmap");
    }
    return launch_pull(s, pull_args(s, 0, false), cs);
}

extern "C" nn_status nn_sim_pull_gather(nn_sim* s)
{
    if (!s) return NN_ERR_INVALID_ARG;
    if (!s->bitmap || !s->col_ptr)
        return nn_fail(s->ctx, NN_ERR_INVALID_ARG, "nn_sim_pull_gather: needs a simulation with pull delivery");
    return launch_pull(s, pull_args(s, 0, false), s->ctx->stream);
}

extern "C" nn_status nn_sim_run_host(nn_sim* s, const float* h_in, int nsteps, float* h_out, int64_t* h_spikes)
{
    if (!s || !h_in || !h_out || nsteps < 0) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    cudaStream_t cs = ctx->stream;
    const size_t bytes = sizeof(float) * (size_t)s->n;
    const int planes[6] = {NN_F_V, NN_F_M, NN_F_H, NN_F_N, NN_F_GE, NN_F_GI};
    unsigned long long t0 = 0;
    NN_CUDA(ctx, cudaMemcpyAsync(&t0, s->total, sizeof t0, cudaMemcpyDeviceToHost, cs));
    for (int q = 0; q < 6; ++q)
        NN_CUDA(ctx, cudaMemcpyAsync(s->f[planes[q]], h_in + (size_t)q * s->n, bytes, cudaMemcpyHostToDevice, cs));
    NN_TRY(nn_sim_step(s, nsteps));
    for (int q = 0; q < 6; ++q)
        NN_CUDA(ctx, cudaMemcpyAsync(h_out + (size_t)q * s->n, s->f[planes[q]], bytes, cudaMemcpyDeviceToHost, cs));
    unsigned long long t1 = 0;
    NN_CUDA(ctx, cudaMemcpyAsync(&t1, s->total, sizeof t1, cudaMemcpyDeviceToHost, cs));
    NN_CUDA(ctx, cudaStreamSynchronize(cs));
    if (h_spikes) *h_spikes = (int64_t)(t1 - t0);
    return check_err(s);
}

extern "C" nn_status nn_sim_counters(nn_sim* s, int64_t* step, int64_t* total_spikes)
{
    if (!s) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    unsigned long long v[2];
    NN_CUDA(ctx, cudaMemcpyAsync(&v[0], s->step, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    NN_CUDA(ctx, cudaMemcpyAsync(&v[1], s->total, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (step) *step = (int64_t)v[0];
    if (total_spikes) *total_spikes = (int64_t)v[1];
    return check_err(s);
}

extern "C" nn_status nn_sim_set_electrodes(nn_sim* s, const int* h_indices, const int* h_offsets, int n_regions,
                                           int every, int capacity)
{
    if (!s || n_regions < 0 || every < 0) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    drop_graph(s);  // the captured launches carry the recording's arguments
    nn_release(s->el_group); nn_release(s->el_val); nn_release(s->el_spk);
    s->el_every = s->el_cap = s->el_members = 0;
    s->el_roff.clear();
    s->el_rpos.clear();
    if (every == 0 || n_regions == 0) return NN_OK;
    if (!h_indices || !h_offsets || capacity < 1)
        return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_sim_set_electrodes: regions and a capacity >= 1 needed");
    if (h_offsets[0] != 0) return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_sim_set_electrodes: offsets[0] must be 0");
    const int n = s->n;
    // member positions in ascending neuron order; regions as lists of positions
    std::vector<int> pos((size_t)n, -1);
    for (int r = 0; r < n_regions; ++r) {
        if (h_offsets[r + 1] < h_offsets[r])
            return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_sim_set_electrodes: offsets not monotone at %d", r);
        for (int k = h_offsets[r]; k < h_offsets[r + 1]; ++k) {
            const int i = h_indices[k];
            if (i < 0 || i >= n) return nn_fail(ctx, NN_ERR_INVALID_ARG, "nn_sim_set_electrodes: index %d out of range", i);
            pos[(size_t)i] = 0;
        }
    }
    int members = 0;
    std::vector<uint2> grp((size_t)s->n_pad / 32, make_uint2(0u, 0u));
    for (int i = 0; i < n; ++i) {
        if ((i & 31) == 0) grp[(size_t)i >> 5].y = (unsigned)members;
        if (pos[(size_t)i] == 0) {
            pos[(size_t)i] = members++;
            grp[(size_t)i >> 5].x |= 1u << (i & 31);
        }
    }
    s->el_roff.assign(h_offsets, h_offsets + n_regions + 1);
    s->el_rpos.resize((size_t)h_offsets[n_regions]);
    for (int k = 0; k < h_offsets[n_regions]; ++k) s->el_rpos[(size_t)k] = pos[(size_t)h_indices[k]];
    const size_t cells = (size_t)capacity * members;
    NN_TRY(nn_alloc(ctx, &s->el_group, grp.size()));
    NN_TRY(nn_alloc(ctx, &s->el_val, cells));
    NN_TRY(nn_alloc(ctx, &s->el_spk, cells));
    NN_CUDA(ctx, nn_copy_sync(ctx, s->el_group, grp.data(), sizeof(uint2) * grp.size(), cudaMemcpyHostToDevice));
    s->el_every = every;
    s->el_cap = capacity;
    s->el_members = members;
    s->el_first = (s->host_step + every - 1) / every * every;
    return NN_OK;
}

extern "C" nn_status nn_sim_read_electrodes(nn_sim* s, float* h_avg, int* h_firing, int64_t* first_step,
                                            int* n_samples)
{
    if (!s || !n_samples) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    *n_samples = 0;
    if (first_step) *first_step = s->el_first;
    if (s->el_every == 0) return NN_OK;
    const int64_t E = s->el_every, M = s->el_members;
    const int R = (int)s->el_roff.size() - 1;
    const int64_t count = s->host_step > s->el_first ? (s->host_step - s->el_first - 1) / E + 1 : 0;
    const int64_t kept = std::min<int64_t>(count, s->el_cap);
    std::vector<float> val((size_t)s->el_cap * M);
    std::vector<uint8_t> spk((size_t)s->el_cap * M);
    NN_CUDA(ctx, cudaMemcpyAsync(val.data(), s->el_val, sizeof(float) * val.size(), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    NN_CUDA(ctx, cudaMemcpyAsync(spk.data(), s->el_spk, spk.size(), cudaMemcpyDeviceToHost, ctx->stream));
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const int64_t first_smp = s->el_first / E + (count - kept);
    for (int64_t k = 0; k < kept; ++k) {
        const size_t base = (size_t)((first_smp + k) % s->el_cap) * (size_t)M;
        for (int r = 0; r < R; ++r) {
            double v = 0.0;
            int f = 0;
            for (int q = s->el_roff[(size_t)r]; q < s->el_roff[(size_t)r + 1]; ++q) {
                v += val[base + (size_t)s->el_rpos[(size_t)q]];
                f += spk[base + (size_t)s->el_rpos[(size_t)q]];
            }
            const int sz = s->el_roff[(size_t)r + 1] - s->el_roff[(size_t)r];
            if (h_avg) h_avg[k * R + r] = sz ? (float)(v / sz) : 0.0f;
            if (h_firing) h_firing[k * R + r] = f;
        }
    }
    if (first_step) *first_step = first_smp * E;
    *n_samples = (int)kept;
    return check_err(s);
}

extern "C" nn_status nn_sim_get_ring(nn_sim* s, float* h_ring)
{
    if (!s || !h_ring) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    // device rows are n_pad pairs long, host rows n
    NN_CUDA(ctx, cudaMemcpy2DAsync(h_ring, sizeof(float2) * (size_t)s->n, s->ring, sizeof(float2) * (size_t)s->n_pad,
                                   sizeof(float2) * (size_t)s->n, (size_t)s->D, cudaMemcpyDeviceToHost, ctx->stream));
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return check_err(s);
}

extern "C" nn_status nn_sim_reset_raster(nn_sim* s)
{
    if (!s) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    NN_CUDA(ctx, cudaMemsetAsync(s->rcount, 0, sizeof(unsigned long long), ctx->stream));
    return NN_OK;
}

extern "C" nn_status nn_sim_get_raster(nn_sim* s, int64_t cap, int32_t* h_step, int32_t* h_neuron, int64_t* count)
{
    if (!s || !count || cap < 0) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    unsigned long long rc = 0;
    NN_CUDA(ctx, cudaMemcpyAsync(&rc, s->rcount, sizeof rc, cudaMemcpyDeviceToHost, ctx->stream));
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *count = (int64_t)rc;
    const int64_t m = std::min<int64_t>(cap, (int64_t)rc);
    if (m > 0 && s->raster) {
        std::vector<int2> tmp((size_t)m);
        NN_CUDA(ctx, cudaMemcpyAsync(tmp.data(), s->raster, sizeof(int2) * (size_t)m, cudaMemcpyDeviceToHost, ctx->stream));
        NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        std::sort(tmp.begin(), tmp.end(), [](const int2& a, const int2& b) { return a.x != b.x ? a.x < b.x : a.y < b.y; });
        for (int64_t q = 0; q < m; ++q) {
            if (h_step) h_step[q] = tmp[(size_t)q].x;
            if (h_neuron) h_neuron[q] = tmp[(size_t)q].y;
        }
    }
    return NN_OK;
}

extern "C" nn_status nn_sim_get_density(nn_sim* s, float* h_u)
{
    if (!s || !h_u || !has_field(s)) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    NN_CUDA(ctx, cudaMemcpyAsync(h_u, s->u, sizeof(float) * (size_t)s->G, cudaMemcpyDeviceToHost, ctx->stream));
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return NN_OK;
}

extern "C" nn_status nn_sim_set_density(nn_sim* s, const float* h_u)
{
    if (!s || !h_u || !has_field(s)) return NN_ERR_INVALID_ARG;
    nn_ctx* ctx = s->ctx;
    NN_CUDA(ctx, cudaMemcpyAsync(s->u, h_u, sizeof(float) * (size_t)s->G, cudaMemcpyHostToDevice, ctx->stream));
    NN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    s->have_prev = false;
    return NN_OK;
}

extern "C" nn_status nn_sim_solve_stats(nn_sim* s, nn_solve_stats* st)
{
    if (!s || !st) return NN_ERR_INVALID_ARG;
    *st = s->stats;
    return NN_OK;
}
