/* Driver that runs the reference's own host-side connectivity construction
 * (UniformRandomNetwork::Generate, Network::ToAdjacencyList,
 * Network::ToChunkedAdjacencyList from src/network_factory.cu) and dumps the
 * results as raw int32/float32 files, to pin the oracle's restatement.
 * Usage: ref_netgen <outdir> */
#include "network_factory.cuh"
#include <cstdio>
#include <string>
#include <vector>

static void dump(std::string const& dir, std::string const& name, void const* p, size_t bytes)
{
    FILE* f = std::fopen((dir + "/" + name).c_str(), "wb");
    if (!f) { std::perror(name.c_str()); std::exit(2); }
    std::fwrite(p, 1, bytes, f);
    std::fclose(f);
}

template <class V> static void dump_vec(std::string const& dir, std::string const& name, V const& v)
{
    std::vector<typename V::value_type> h(v.begin(), v.end());
    dump(dir, name, h.data(), h.size() * sizeof(typename V::value_type));
}

int main(int argc, char** argv)
{
    if (argc < 2) return 1;
    std::string dir = argv[1];
    /* Case A: the hh_benchmark pattern (src/main.cu:381-385): two networks
     * drawn from the one shared unseeded engine, then their in-degrees. */
    int const NA = 1000;
    UniformRandomNetwork e_net(8), i_net(2);
    e_net.Generate(NA);
    i_net.Generate(NA);
    std::vector<Float> tc_e(NA), tc_i(NA);
    Float* pe = tc_e.data();
    Float* pi = tc_i.data();
    AdjacencyList le = e_net.ToAdjacencyList(pe);
    AdjacencyList li = i_net.ToAdjacencyList(pi);
    dump_vec(dir, "A_e_indices.i32", le.indices);
    dump_vec(dir, "A_e_offsets.i32", le.offset_in_indices);
    dump_vec(dir, "A_i_indices.i32", li.indices);
    dump_vec(dir, "A_i_offsets.i32", li.offset_in_indices);
    dump(dir, "A_e_tcount.f32", tc_e.data(), NA * sizeof(Float));
    dump(dir, "A_i_tcount.f32", tc_i.data(), NA * sizeof(Float));
    /* Case B: the chunked list at the SCN size the chunking is built for
     * (NCHUNKS * N_PER_CHUNK, src/defines.cuh:83-84), continuing the engine. */
    int const NB = NCHUNKS * N_PER_CHUNK;
    UniformRandomNetwork c_net(3);
    c_net.Generate(NB);
    std::vector<Float> tc_c(NB);
    Float* pc = tc_c.data();
    ChunkedAdjacencyList lc = c_net.ToChunkedAdjacencyList(pc);
    dump_vec(dir, "B_indices.i32", c_net.GetCpuIndices());
    dump_vec(dir, "B_offsets.i32", c_net.GetCpuOffsetsIntoIndices());
    dump(dir, "B_tcount.f32", tc_c.data(), NB * sizeof(Float));
    std::vector<int*> ci(lc.indices_chunks.begin(), lc.indices_chunks.end());
    std::vector<int*> co(lc.offset_in_indices_chunks.begin(), lc.offset_in_indices_chunks.end());
    for (int c = 0; c < NCHUNKS; ++c) {
        int nnz_c = co[c][NB];
        dump(dir, "B_chunk" + std::to_string(c) + "_indices.i32", ci[c], nnz_c * sizeof(int));
        dump(dir, "B_chunk" + std::to_string(c) + "_offsets.i32", co[c], (NB + 1) * sizeof(int));
    }
    return 0;
}
