// The reference's hh_benchmark step loop (src/main.cu:307-424, loop body
// src/main.cu:166-181) written against the C++ adaptors: two uniform random
// networks (excitatory / inhibitory) turned into chunked adjacency lists, two
// AtomicCouplings and the HH leapfrog step on the 17-slot SoA table.
// Usage: hh_loop <N> <steps>; prints "N steps total_firing mean_V".
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "neuronephys.hpp"

using namespace neuronephys;

int main(int argc, char** argv)
{
    const int N = argc > 1 ? std::atoi(argv[1]) : 2000;
    const int steps = argc > 2 ? std::atoi(argv[2]) : 50;
    nn_ctx* c = ctx().get();
    std::vector<void*> sim_vars_cpu(NN_HH_NUM_VARS);
    std::vector<float> host((size_t)N, 0.0f);
    for (auto& p : sim_vars_cpu) {
        ctx().check(nn_malloc(c, sizeof(float) * N, &p), "nn_malloc");
        ctx().check(nn_memset_d(c, p, 0, sizeof(float) * N), "memset");
    }
    // V spread over [-80, -30] mV (deterministic), gates and synapses at 0
    for (int i = 0; i < N; ++i) host[(size_t)i] = -80.0f + 50.0f * (float)((i * 7919) % N) / (float)N;
    ctx().check(nn_memcpy_h2d(c, sim_vars_cpu[NN_HH_V], host.data(), sizeof(float) * N), "h2d");
    void* d_table = nullptr;
    ctx().check(nn_malloc(c, sizeof(void*) * NN_HH_NUM_VARS, &d_table), "nn_malloc");
    ctx().check(nn_memcpy_h2d(c, d_table, sim_vars_cpu.data(), sizeof(void*) * NN_HH_NUM_VARS), "h2d");

    HHEphys ephys(N);
    AtomicCoupling e_coupling(N), i_coupling(N);
    UniformRandomNetwork e_net(8), i_net(2);
    e_net.Generate(N);
    i_net.Generate(N);
    Float* ecount = (Float*)sim_vars_cpu[NN_HH_ECOUNT];
    Float* icount = (Float*)sim_vars_cpu[NN_HH_ICOUNT];
    ChunkedAdjacencyList e_list = e_net.ToChunkedAdjacencyList(ecount);
    ChunkedAdjacencyList i_list = i_net.ToChunkedAdjacencyList(icount);
    long long total = 0;
    for (int t = 0; t < steps; ++t) {
        total += e_coupling(e_list, (Float*)sim_vars_cpu[NN_HH_EIN], (Float*)sim_vars_cpu[NN_HH_EOUTPUT]);
        total += i_coupling(i_list, (Float*)sim_vars_cpu[NN_HH_IIN], (Float*)sim_vars_cpu[NN_HH_IOUTPUT]);
        ephys.SimulateEphys((Float**)d_table);
    }
    ctx().check(nn_memcpy_d2h(c, host.data(), sim_vars_cpu[NN_HH_V], sizeof(float) * N), "d2h");
    double mean = 0.0;
    for (float v : host) mean += v;
    std::printf("%d %d %lld %.6f\n", N, steps, total, mean / N);
    for (auto p : sim_vars_cpu) nn_free(c, p);
    nn_free(c, d_table);
    return 0;
}
