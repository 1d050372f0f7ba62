// The neuron update's launch arguments and its launcher (the kernel is in
// nn_step.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "nn_hh.cuh"

struct StepArgs {
    float *V, *m, *h, *nn, *ge, *gi;
    const float* idrive;
    const float* gna_scale;
    const float* upar;
    float* ring;            // float2 (E, I) per neuron, D slots
    uint32_t* bitmap;       // pull delivery: spike bitmap of the last D steps
    int* list;              // spikes of the step (by step parity)
    int* counts;
    const unsigned long long* base;  // first step of the current period
    int q;                  // this launch's step within the period
    // push delivery (row_ptr == nullptr: pull delivery runs as its own kernel)
    const int64_t* row_ptr;
    const int32_t* col;
    const float* weight;
    const uint8_t* delay;
    const uint8_t* is_inh;
    unsigned long long* total;
    unsigned long long* rcount;
    int2* raster;
    long long rcap;
    const int32_t* vox;
    float* src;
    // fused electrode recording (el_every > 0): on steps t with t % el_every
    // == 0 each member neuron (a neuron of some region) writes its new
    // potential and its spike flag to its member position (members in
    // ascending neuron order) of sample slot
    // (t / el_every) % el_cap; the host forms the region means and counts
    const uint2* el_group;    // per 32-neuron group g (neurons 32g .. 32g+31): {member bits, members before g}
    float* el_val;            // [el_cap][el_members]
    uint8_t* el_spk;          // [el_cap][el_members]
    int el_every, el_cap, el_members;
    // automatic delivery: rowflag[t % D] = 1 when step t's spikes go to the
    // bitmap for the pull gather, 0 when they are pushed (null otherwise)
    int* rowflag;
    int* err;
    int n, n_pad, D, words;
    int zero_ring;
    uint64_t seed;
    nn_hh_dev p;
};

template <int NPT> struct VecT;
template <> struct VecT<1> { using type = float; };
template <> struct VecT<2> { using type = float2; };
template <> struct VecT<4> { using type = float4; };

template <int NPT>
__device__ __forceinline__ void vload(const float* base, int i0, float (&out)[NPT])
{
    using V = typename VecT<NPT>::type;
    const V v = *reinterpret_cast<const V*>(base + i0);
    const float* pv = reinterpret_cast<const float*>(&v);
#pragma unroll
    for (int q = 0; q < NPT; ++q) out[q] = pv[q];
}

template <int NPT>
__device__ __forceinline__ void vstore(float* base, int i0, const float (&in)[NPT])
{
    using V = typename VecT<NPT>::type;
    V v;
    float* pv = reinterpret_cast<float*>(&v);
#pragma unroll
    for (int q = 0; q < NPT; ++q) pv[q] = in[q];
    *reinterpret_cast<V*>(base + i0) = v;
}

// Scatter one spike's out-edges [beg, end) into the delay ring (all 32 lanes
// of the warp): each lane loads PUSH_UNROLL edges (target, weight, delay)
// before issuing their reductions, so a row of up to 32 * PUSH_UNROLL edges
// costs one load round trip.  slot: the current step's ring slot; chn: 0
// excitatory, 1 inhibitory.
constexpr int PUSH_UNROLL = 4;

__device__ __forceinline__ void nn_push_row(const StepArgs& a, int64_t beg, int64_t end, int chn, int slot, int lane)
{
    for (int64_t e0 = beg + lane; e0 < end; e0 += 32 * PUSH_UNROLL) {
        int tgt[PUSH_UNROLL], dl[PUSH_UNROLL];
        float w[PUSH_UNROLL];
#pragma unroll
        for (int u = 0; u < PUSH_UNROLL; ++u) {
            const int64_t e = e0 + 32 * u;
            if (e < end) {
                tgt[u] = a.col[e];
                w[u] = a.weight[e];
                dl[u] = a.delay[e];
            }
        }
#pragma unroll
        for (int u = 0; u < PUSH_UNROLL; ++u) {
            if (e0 + 32 * u >= end) break;
            int sl = slot + dl[u];
            if (sl >= a.D) sl -= a.D;
            atomicAdd(a.ring + 2 * ((size_t)sl * a.n_pad + tgt[u]) + chn, w[u]);
        }
    }
}

// One step of every neuron on stream cs (NPT neurons per thread: 1, 2 or 4).
cudaError_t nn_launch_hh_step(const StepArgs& a, int npt, int blocks, int tpb, cudaStream_t cs);
