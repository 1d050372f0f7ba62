// The neuron update: one RK4 step of every neuron with threshold detection,
// compaction and push delivery (see the kernel comment).
#include "nn_step.cuh"

namespace {

// One simulation step, NPT consecutive neurons per lane:
//   ring slot t%D -> (ge, gi) jump, RK4 with noise, upward threshold crossing,
//   warp-aggregated compaction (one atomic per warp with spikes), spike bitmap
//   (pull), voxel deposit, raster, and -- in push mode -- the delivery itself:
//   the warp that found the spikes scatters their out-edges into ring slots
//   (t+d)%D with red.global.add (d >= 1, so never the slot this launch reads).
// Loop trip counts are warp-uniform so the warp collectives stay converged.
// Registers the neuron update is compiled for: 3 blocks of 256 threads per
// SM (at most 85 registers; 80 used, with a few spilled words in the spike
// path) is faster than 2 blocks without spills (21.3 vs 18.1 us per
// 1M-neuron step) and than 4.
#ifndef NN_HH_MIN_BLOCKS
#define NN_HH_MIN_BLOCKS 3
#endif
// UNI: no per-neuron gNa scale and no paracrine feedback (the common case),
// so the step's constant current terms are launch constants
// (nn_hh_drive_uniform) rather than registers.
// EL: electrode recording compiled in (nn_sim_set_electrodes); without it
// the update carries none of that code.
template <int NPT, bool UNI, bool EL>
__global__ void __launch_bounds__(256, NN_HH_MIN_BLOCKS) k_hh_step(StepArgs a)
{
    const uint64_t t = *a.base + (uint64_t)a.q;
    const int slot = (int)(t % (uint64_t)a.D);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.counts[(t + 1) & 1] = 0;  // next step's count
        if (a.rowflag) a.rowflag[slot] = a.bitmap != nullptr;
    }
    // electrode sample slot of this step (-1: no sample)
    const int s_el =
        (EL && t % (uint64_t)a.el_every == 0) ? (int)((t / (uint64_t)a.el_every) % (uint64_t)a.el_cap) : -1;
    float* ring_slot = a.ring + (size_t)slot * a.n_pad * 2;
    int* list = a.list + (size_t)(t & 1) * a.n_pad;
    int* cnt = a.counts + (t & 1);
    uint32_t* bm = a.bitmap ? a.bitmap + (size_t)slot * a.words : nullptr;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int chunk = 32 * NPT;
    // electrode sample of this step (nullptr: none)
    float* el_v = EL && s_el >= 0 ? a.el_val + (size_t)s_el * a.el_members : nullptr;
    uint8_t* el_s = EL && s_el >= 0 ? a.el_spk + (size_t)s_el * a.el_members : nullptr;
    const int nchunks = a.n_pad / chunk;
    for (int ch = warp; ch < nchunks; ch += nwarps) {
        const int i0 = ch * chunk + lane * NPT;
        float V[NPT], M[NPT], H[NPT], N[NPT], GE[NPT], GI[NPT], ID[NPT];
        vload<NPT>(a.V, i0, V);
        vload<NPT>(a.m, i0, M);
        vload<NPT>(a.h, i0, H);
        vload<NPT>(a.nn, i0, N);
        vload<NPT>(a.ge, i0, GE);
        vload<NPT>(a.gi, i0, GI);
        vload<NPT>(a.idrive, i0, ID);
        float RG[2 * NPT];
        if (NPT == 1) {
            const float2 v = *reinterpret_cast<const float2*>(ring_slot + 2 * i0);
            RG[0] = v.x; RG[1] = v.y;
        } else {
#pragma unroll
            for (int q = 0; q < NPT / 2; ++q) {
                const float4 v = *reinterpret_cast<const float4*>(ring_slot + 2 * i0 + 4 * q);
                RG[4 * q] = v.x; RG[4 * q + 1] = v.y; RG[4 * q + 2] = v.z; RG[4 * q + 3] = v.w;
            }
        }
        float GS[NPT], UP[NPT];
        if (a.gna_scale) vload<NPT>(a.gna_scale, i0, GS);
        else {
#pragma unroll
            for (int q = 0; q < NPT; ++q) GS[q] = 1.0f;
        }
        if (a.upar) vload<NPT>(a.upar, i0, UP);
        else {
#pragma unroll
            for (int q = 0; q < NPT; ++q) UP[q] = 0.0f;
        }
        // noise: one Philox draw and one Box-Muller per neuron pair
        float Z[NPT];
        if (NPT == 1) {
            Z[0] = nn_normal(a.seed, (uint32_t)i0, t);
        } else {
#pragma unroll
            for (int q = 0; q < NPT; q += 2) nn_normal_pair(a.seed, (uint32_t)(i0 + q) >> 1, t, Z[q], Z[q + 1]);
        }
        uint32_t mask = 0;
        bool bad = false;
        bool any_in = false;
        // RK4 on neuron pairs through packed two-lane arithmetic (one lane
        // when NPT = 1; the results are the same bits either way)
        constexpr int W = NPT >= 2 ? 2 : 1;
#pragma unroll
        for (int p0 = 0; p0 < NPT; p0 += W) {
            nn_hh_state<W> y;
            nn_vf<W> ngna, iext, ngpu;
#pragma unroll
            for (int l = 0; l < W; ++l) {
                const int q = p0 + l;
                y.V.v[l] = V[q]; y.m.v[l] = M[q]; y.h.v[l] = H[q]; y.n.v[l] = N[q];
                y.ge.v[l] = __fadd_rn(GE[q], RG[2 * q]);
                y.gi.v[l] = __fadd_rn(GI[q], RG[2 * q + 1]);
                any_in |= (RG[2 * q] != 0.0f) | (RG[2 * q + 1] != 0.0f);
                iext.v[l] = __fmaf_rn(a.p.noise_sigma, Z[q], ID[q]);
                ngna.v[l] = -__fmul_rn(a.p.gNa, GS[q]);
                ngpu.v[l] = -__fmul_rn(a.p.g_par, UP[q]);
            }
            if (UNI) nn_hh_rk4<W>(a.p, nn_hh_make_drive_uniform<W>(a.p, iext), y);
            else nn_hh_rk4<W>(a.p, nn_hh_make_drive<W>(a.p, ngna, iext, ngpu), y);
#pragma unroll
            for (int l = 0; l < W; ++l) {
                const int q = p0 + l;
                const bool valid = i0 + q < a.n;
                const float vn = y.V.v[l];
                if (valid && V[q] < a.p.v_thresh && vn >= a.p.v_thresh) mask |= 1u << q;
                if (valid && !isfinite(vn)) bad = true;
                V[q] = vn; M[q] = y.m.v[l]; H[q] = y.h.v[l]; N[q] = y.n.v[l]; GE[q] = y.ge.v[l]; GI[q] = y.gi.v[l];
            }
        }
        vstore<NPT>(a.V, i0, V);
        vstore<NPT>(a.m, i0, M);
        vstore<NPT>(a.h, i0, H);
        vstore<NPT>(a.nn, i0, N);
        vstore<NPT>(a.ge, i0, GE);
        vstore<NPT>(a.gi, i0, GI);
        if (a.zero_ring && any_in) {
            if (NPT == 1) {
                *reinterpret_cast<float2*>(ring_slot + 2 * i0) = make_float2(0.0f, 0.0f);
            } else {
#pragma unroll
                for (int q = 0; q < NPT / 2; ++q)
                    *reinterpret_cast<float4*>(ring_slot + 2 * i0 + 4 * q) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
        }
        if (bad) atomicOr(a.err, 1);
        // ElectrodeNet::DoElectrodeMeasurements fused: member neurons record
        // their potential and spike.  A lane's NPT neurons lie in one 32-neuron
        // group; its member bits and count of earlier members give the
        // position (most groups hold no member).
        if (EL && el_v) {
            const uint2 gm = a.el_group[i0 >> 5];
            if (gm.x) {
#pragma unroll
                for (int q = 0; q < NPT; ++q) {
                    const int b = (i0 + q) & 31;
                    if ((gm.x >> b) & 1u) {
                        const int pos = (int)gm.y + __popc(gm.x & ((1u << b) - 1u));
                        el_v[pos] = V[q];
                        el_s[pos] = (mask >> q) & 1u;
                    }
                }
            }
        }
        // spike bitmap word of 32 consecutive neurons (pull delivery)
        if (bm) {
            uint32_t bits = mask << ((lane * NPT) & 31);
#pragma unroll
            for (int o = 1; o < 32 / NPT; o <<= 1) bits |= __shfl_xor_sync(0xffffffffu, bits, o);
            if ((lane % (32 / NPT)) == 0) bm[(ch * chunk + lane * NPT) >> 5] = bits;
        }
        const int c = __popc(mask);
        if (!__any_sync(0xffffffffu, c != 0)) continue;
        // warp-aggregated compaction, totals and raster: one atomic each per warp
        int inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int tv = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += tv;
        }
        const int tot = __shfl_sync(0xffffffffu, inc, 31);
        int base = 0;
        unsigned long long rbase = 0;
        if (lane == 31) {
            base = atomicAdd(cnt, tot);
            atomicAdd(a.total, (unsigned long long)tot);
            if (a.raster) rbase = atomicAdd(a.rcount, (unsigned long long)tot);
        }
        base = __shfl_sync(0xffffffffu, base, 31);
        rbase = __shfl_sync(0xffffffffu, rbase, 31);
        int pos = base + inc - c;
        unsigned long long rpos = rbase + (unsigned long long)(inc - c);
#pragma unroll
        for (int q = 0; q < NPT; ++q)
            if (mask & (1u << q)) {
                list[pos++] = i0 + q;
                if (a.src) atomicAdd(a.src + a.vox[i0 + q], 1.0f);
                if (a.raster && rpos < (unsigned long long)a.rcap) a.raster[rpos] = make_int2((int)t, i0 + q);
                ++rpos;
            }
        // push delivery of this warp's spikes: every spiking lane loads its
        // own rows' bounds and types at once, then all lanes scatter each
        // spike's out-edges (nn_push_row)
        if (a.row_ptr) {
            int64_t rb[NPT], re[NPT];
            int rc[NPT];
#pragma unroll
            for (int q = 0; q < NPT; ++q) {
                rb[q] = re[q] = 0;
                rc[q] = 0;
                if (mask & (1u << q)) {
                    const int j = i0 + q;
                    rb[q] = a.row_ptr[j];
                    re[q] = a.row_ptr[j + 1];
                    rc[q] = a.is_inh[j] ? 1 : 0;
                }
            }
            unsigned who = __ballot_sync(0xffffffffu, mask != 0);
            while (who) {
                const int sl_lane = __ffs(who) - 1;
                who &= who - 1;
                const uint32_t m = __shfl_sync(0xffffffffu, mask, sl_lane);
#pragma unroll
                for (int q = 0; q < NPT; ++q) {
                    if (!(m & (1u << q))) continue;
                    const int64_t beg = __shfl_sync(0xffffffffu, rb[q], sl_lane);
                    const int64_t end = __shfl_sync(0xffffffffu, re[q], sl_lane);
                    const int chn = __shfl_sync(0xffffffffu, rc[q], sl_lane);
                    nn_push_row(a, beg, end, chn, slot, lane);
                }
            }
        }
    }
}

}  // namespace

cudaError_t nn_launch_hh_step(const StepArgs& a, int npt, int blocks, int tpb, cudaStream_t cs)
{
    // uniform when no per-neuron gNa scale is loaded and the field does not
    // feed back (g_par = 0 or no density input): then ngna = -gNa and
    // ngpu = 0 (or -0) for every neuron, as the general form computes them
    const bool uni = !a.gna_scale && (!a.upar || a.p.g_par == 0.0f);
    const bool el = a.el_every > 0;
    switch (npt * 4 + (uni ? 2 : 0) + (el ? 1 : 0)) {
        case 4: k_hh_step<1, false, false><<<blocks, tpb, 0, cs>>>(a); break;
        case 5: k_hh_step<1, false, true><<<blocks, tpb, 0, cs>>>(a); break;
        case 6: k_hh_step<1, true, false><<<blocks, tpb, 0, cs>>>(a); break;
        case 7: k_hh_step<1, true, true><<<blocks, tpb, 0, cs>>>(a); break;
        case 8: k_hh_step<2, false, false><<<blocks, tpb, 0, cs>>>(a); break;
        case 9: k_hh_step<2, false, true><<<blocks, tpb, 0, cs>>>(a); break;
        case 10: k_hh_step<2, true, false><<<blocks, tpb, 0, cs>>>(a); break;
        case 11: k_hh_step<2, true, true><<<blocks, tpb, 0, cs>>>(a); break;
        case 16: k_hh_step<4, false, false><<<blocks, tpb, 0, cs>>>(a); break;
        case 17: k_hh_step<4, false, true><<<blocks, tpb, 0, cs>>>(a); break;
        case 18: k_hh_step<4, true, false><<<blocks, tpb, 0, cs>>>(a); break;
        default: k_hh_step<4, true, true><<<blocks, tpb, 0, cs>>>(a); break;
    }
    return cudaPeekAtLastError();
}
