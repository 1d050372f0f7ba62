// neuronephys.hpp -- C++ adaptors with the reference's class names and
// signatures, implemented on the C ABI of neuronephys.h.
//
// A step loop written against the reference (src/main.cu:112-182) compiles
// against these classes unchanged apart from the include:
//
//   UniformRandomNetwork e_net(800);  e_net.Generate(N);
//   ChunkedAdjacencyList e_list = e_net.ToChunkedAdjacencyList(sim_vars_cpu[SIM_PARAMS_ECOUNT]);
//   AtomicCoupling e_coupling(N);
//   HHEphys ephys(N);
//   for (...) { e_coupling(e_list, ein, eout); ephys.SimulateEphys(d_sim_vars); }
//
// Differences from the reference, all deliberate:
// * errors throw neuronephys::Error (the reference prints and exit()s);
// * every call returns after its device work has finished, as the reference's
//   cudaDeviceSynchronize after each launch did (set_synchronous(false) lets
//   calls run ahead on the library's stream);
// * the device buffers the reference kept in thrust::device_vector are owned
//   by these objects and released in their destructors.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "neuronephys.h"

namespace neuronephys {

typedef float Float;  // src/defines.cuh:50-55 (USE_DOUBLE_PRECISION 0)

class Error : public std::runtime_error {
public:
    Error(nn_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    nn_status status;
};

// One library context per thread (device 0 unless select_device was called).
class Context {
public:
    static Context& thread_default()
    {
        thread_local Context c;
        return c;
    }
    static void select_device(int d) { device_() = d; }
    nn_ctx* get()
    {
        if (!ctx_) check(nn_ctx_create(device_(), &ctx_), "nn_ctx_create");
        return ctx_;
    }
    void check(nn_status s, const char* what)
    {
        if (s == NN_OK) return;
        std::string msg = std::string(what) + ": " + nn_status_string(s);
        if (ctx_ && *nn_ctx_last_error(ctx_)) msg += std::string(" (") + nn_ctx_last_error(ctx_) + ")";
        throw Error(s, msg);
    }
    void finish(const char* what)
    {
        if (synchronous_) check(nn_ctx_synchronize(get()), what);
    }
    void set_synchronous(bool on) { synchronous_ = on; }
    ~Context()
    {
        if (ctx_) nn_ctx_destroy(ctx_);
    }

private:
    Context() = default;
    static int& device_()
    {
        static int d = 0;
        return d;
    }
    nn_ctx* ctx_ = nullptr;
    bool synchronous_ = true;
};

inline Context& ctx() { return Context::thread_default(); }

// ------------------------------------------------------------------ ephys --
// Ephys / HHEphys (src/ephys.cuh:6-31).
class Ephys {
public:
    explicit Ephys(int N_) : N(N_) {}
    virtual ~Ephys() = default;
    // sim_vars: device array of NUM_SIM_PARAMS device pointers (the reference's
    // thrust::raw_pointer_cast(sim_vars.data())).
    virtual void SimulateEphys(Float** sim_vars) = 0;

protected:
    int const N;
};

class HHEphys : public Ephys {
public:
    // variant 0: the src/ constants, 1: the src_wholebrain/ constants.
    explicit HHEphys(int const N_, int variant = 0, uint64_t seed = 0, Float dt = 0.4f)
        : Ephys(N_), seed_(seed), dt_(dt)
    {
        nn_leapfrog_params_reference(&params_, variant);
    }
    void SimulateEphys(Float** sim_vars) override
    {
        // the 17 device pointers are read from the device table once per table
        if (sim_vars != table_dev_) {
            ctx().check(nn_memcpy_d2h(ctx().get(), table_, sim_vars, sizeof table_), "SimulateEphys");
            table_dev_ = sim_vars;
        }
        ctx().check(nn_hh_leapfrog_step(ctx().get(), table_, N, dt_, &params_, seed_, step_++), "SimulateEphys");
        ctx().finish("SimulateEphys");
    }
    nn_leapfrog_params& params() { return params_; }

private:
    nn_leapfrog_params params_{};
    uint64_t seed_ = 0, step_ = 0;
    Float dt_ = 0.4f;
    Float** table_dev_ = nullptr;
    float* table_[NN_HH_NUM_VARS] = {};
};

// --------------------------------------------------------------- coupling --
// AdjacencyList / ChunkedAdjacencyList (src/coupling.cuh:4-14): device CSR,
// row = presynaptic neuron, owned by the list.
struct DeviceBuffer {
    void* p = nullptr;
    DeviceBuffer() = default;
    explicit DeviceBuffer(size_t bytes) { ctx().check(nn_malloc(ctx().get(), bytes ? bytes : 1, &p), "nn_malloc"); }
    DeviceBuffer(DeviceBuffer&& o) noexcept : p(o.p) { o.p = nullptr; }
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept
    {
        std::swap(p, o.p);
        return *this;
    }
    DeviceBuffer(const DeviceBuffer&) = delete;
    ~DeviceBuffer()
    {
        if (p) nn_free(ctx().get(), p);
    }
};

struct AdjacencyList {
    int n = 0;
    int64_t nnz = 0;
    DeviceBuffer indices_buf, offsets_buf;
    const int* indices() const { return (const int*)indices_buf.p; }
    const int* offset_in_indices() const { return (const int*)offsets_buf.p; }
};

struct ChunkedAdjacencyList {
    int n = 0, n_per_chunk = 0;
    std::vector<DeviceBuffer> indices_chunks, offset_in_indices_chunks;
    std::vector<int64_t> chunk_nnz;
};

class AtomicCoupling {
public:
    explicit AtomicCoupling(int const N_, int signal_mode = NN_SIGNAL_COUNT) : N(N_), mode_(signal_mode)
    {
        ctx().check(nn_coupling_create(ctx().get(), N, &c_), "AtomicCoupling");
    }
    ~AtomicCoupling()
    {
        if (c_) nn_coupling_destroy(c_);
    }
    AtomicCoupling(const AtomicCoupling&) = delete;
    AtomicCoupling& operator=(const AtomicCoupling&) = delete;

    // src/coupling.cu:111-141
    int operator()(AdjacencyList const& connectivity, Float* spikes, Float const* neuron_outputs)
    {
        int nf = 0;
        ctx().check(nn_coupling_run(c_, connectivity.indices(), connectivity.offset_in_indices(), spikes,
                                    neuron_outputs, mode_, &nf),
                    "AtomicCoupling()");
        return nf;
    }
    // src/coupling.cu:143-178
    int operator()(ChunkedAdjacencyList const& connectivity, Float* spikes, Float const* neuron_outputs)
    {
        std::vector<const int*> ci, co;
        for (auto& b : connectivity.indices_chunks) ci.push_back((const int*)b.p);
        for (auto& b : connectivity.offset_in_indices_chunks) co.push_back((const int*)b.p);
        int nf = 0;
        ctx().check(nn_coupling_run_chunked(c_, (int)ci.size(), connectivity.n_per_chunk, ci.data(), co.data(),
                                            spikes, neuron_outputs, &nf),
                    "AtomicCoupling()");
        return nf;
    }
    // src/coupling.cuh:37 (device pointer to the n-entry buffer)
    const int* GetFiringNeurons() const { return nn_coupling_firing_list(c_); }
    nn_coupling* handle() const { return c_; }

private:
    int N;
    int mode_;
    nn_coupling* c_ = nullptr;
};

// --------------------------------------------------------------- network --
// Network / UniformRandomNetwork (src/network_factory.cuh:6-67).
class Network {
public:
    virtual ~Network() = default;
    virtual bool Generate(int const N) = 0;

    // src/network_factory.cu:5-27: upload the CSR, write the in-degree into Tcount (device)
    AdjacencyList ToAdjacencyList(Float*& Tcount) const
    {
        AdjacencyList l;
        l.n = (int)offset_in_indices.size() - 1;
        l.nnz = (int64_t)indices.size();
        if (l.n < 0) return l;
        l.indices_buf = DeviceBuffer(indices.size() * sizeof(int));
        l.offsets_buf = DeviceBuffer(offset_in_indices.size() * sizeof(int));
        ctx().check(nn_memcpy_h2d(ctx().get(), l.indices_buf.p, indices.data(), indices.size() * sizeof(int)), "h2d");
        ctx().check(nn_memcpy_h2d(ctx().get(), l.offsets_buf.p, offset_in_indices.data(),
                                  offset_in_indices.size() * sizeof(int)),
                    "h2d");
        ctx().check(nn_net_tcount(ctx().get(), l.indices(), l.nnz, l.n, Tcount), "ToAdjacencyList");
        ctx().finish("ToAdjacencyList");
        return l;
    }

    // src/network_factory.cu:29-85 (NCHUNKS = 2, N_PER_CHUNK = 7319 in the reference)
    ChunkedAdjacencyList ToChunkedAdjacencyList(Float*& Tcount, int nchunks = 2, int n_per_chunk = 7319) const
    {
        AdjacencyList flat = ToAdjacencyList(Tcount);
        ChunkedAdjacencyList c;
        c.n = flat.n;
        c.n_per_chunk = n_per_chunk;
        std::vector<int*> ci, co;
        for (int k = 0; k < nchunks; ++k) {
            c.indices_chunks.emplace_back(std::max<size_t>(indices.size(), 1) * sizeof(int));
            c.offset_in_indices_chunks.emplace_back((size_t)(flat.n + 1) * sizeof(int));
            ci.push_back((int*)c.indices_chunks.back().p);
            co.push_back((int*)c.offset_in_indices_chunks.back().p);
        }
        c.chunk_nnz.assign((size_t)nchunks, 0);
        ctx().check(nn_net_to_chunked(ctx().get(), flat.indices(), flat.offset_in_indices(), flat.n, nchunks,
                                      n_per_chunk, ci.data(), co.data(), c.chunk_nnz.data()),
                    "ToChunkedAdjacencyList");
        return c;
    }
    std::vector<int> const& GetCpuIndices() const { return indices; }
    std::vector<int> const& GetCpuOffsetsIntoIndices() const { return offset_in_indices; }

protected:
    std::vector<int> indices;
    std::vector<int> offset_in_indices;
};

class UniformRandomNetwork : public Network {
public:
    explicit UniformRandomNetwork(int Ncouple_) : Ncouple(Ncouple_) {}
    // src/network_factory.cu:96-131, drawing from the shared engine
    bool Generate(int const N) override
    {
        indices.assign((size_t)N * Ncouple, 0);
        offset_in_indices.assign((size_t)N + 1, 0);
        return nn_net_uniform_random(N, Ncouple, &Engine(), indices.data(), offset_in_indices.data()) == NN_OK;
    }
    // the reference's Utility::UnseededRandomEngine (src/defines.cu:4-10)
    static uint32_t& Engine()
    {
        static uint32_t state = 1;
        return state;
    }

protected:
    int Ncouple;
};

// -------------------------------------------------------------- paracrine --
// ParacrineModule (src/paracrine.cuh:212-267).
class ParacrineModule {
public:
    // d_x/d_y/d_z: device coordinates (the reference passes device_vectors)
    ParacrineModule(Float*& d_g_paracrine, int const neuron_count, int const x_grid_count, int const y_grid_count,
                    int const z_grid_count, Float const par_dt_, int const timescale_, Float const coup_strength_,
                    Float const spatial_gridsize, Float const diffusion_coef, Float const decay_coef,
                    const Float* d_x_coords, const Float* d_y_coords, const Float* d_z_coords)
        : x_gridcount(x_grid_count), y_gridcount(y_grid_count), z_gridcount(z_grid_count), timescale(timescale_)
    {
        nn_paracrine_ref_params p;
        nn_paracrine_ref_params_default(&p);
        p.nx = x_grid_count; p.ny = y_grid_count; p.nz = z_grid_count;
        p.h = spatial_gridsize; p.D = diffusion_coef; p.decay = decay_coef;
        p.par_dt = par_dt_; p.coup_strength = coup_strength_;
        ctx().check(nn_paracrine_ref_create(ctx().get(), &p, neuron_count, d_x_coords, d_y_coords, d_z_coords,
                                            d_g_paracrine, &pm_),
                    "ParacrineModule");
        ctx().finish("ParacrineModule");
    }
    ~ParacrineModule()
    {
        if (pm_) nn_paracrine_destroy(pm_);
    }
    ParacrineModule(const ParacrineModule&) = delete;
    ParacrineModule& operator=(const ParacrineModule&) = delete;

    void update_on_fine_timescale(AtomicCoupling const& coupling)
    {
        ctx().check(nn_paracrine_ref_fine(pm_, coupling.handle()), "update_on_fine_timescale");
        ctx().finish("update_on_fine_timescale");
    }
    void update_on_own_timescale()
    {
        ctx().check(nn_paracrine_ref_own(pm_, nullptr, nullptr), "update_on_own_timescale");
        ctx().finish("update_on_own_timescale");
    }
    // get_grid().density(): device pointer, x fastest
    const Float* density() const { return nn_paracrine_density(pm_); }

    int x_gridcount, y_gridcount, z_gridcount, timescale;

private:
    nn_paracrine* pm_ = nullptr;
};

}  // namespace neuronephys
