/* Driver-API harness for the reference's own CUDA kernels.  TEST
 * INFRASTRUCTURE ONLY: loaded by the GPU parity tests and by bench.py's
 * reference arm, never by the product library.
 *
 * oracle/build.py compiles the reference's src/ephys.cu and src/coupling.cu,
 * and their whole-brain variants src_wholebrain/ephys.cu and
 * src_wholebrain/coupling.cu (where the reference checkout is present), into
 * device-only cubins under oracle/_ref/.  A cubin holds no host code, so the same file runs on any
 * host architecture.  This file stands in for the reference's host launch
 * code, which is a few lines per kernel:
 *
 *   HHEphys::SimulateEphys        src/ephys.cu:98-103    Leapfrog_HH<<<NBLOCKS, NTHREADS>>>
 *   Ephys::Ephys                  src/ephys.cu:20-26     init_random<<<NBLOCKS, NTHREADS>>>(0, N, states)
 *   AtomicCoupling::operator()    src/coupling.cu:133-136 signal_spikes_kernel<<<NBLOCKS, NTHREADS>>>
 *                                 src/coupling.cu:166-172 signal_spikes_kernel_chunked<<<NBLOCKS, NTHREADS>>>
 *                                                         merge_kernel<<<NBLOCKS, NTHREADS>>>
 *
 *   HHEphys::SimulateEphys        src_wholebrain/ephys.cu:219-224  Leapfrog_HH<<<NBLOCKS, NTHREADS>>>
 *   AtomicCoupling::PerformCoupling src_wholebrain/coupling.cu:62-65 signal_spikes_kernel<<<NBLOCKS, NTHREADS>>>
 *
 * with NBLOCKS = 32, NTHREADS = 64 (src/defines.cuh:81-82; the whole-brain
 * variant uses 512 threads, src_wholebrain/defines.cuh:46-47) unless the
 * caller asks for another grid.  Every launch is followed by a context
 * synchronisation, as the reference does (gpuErrchk(cudaDeviceSynchronize())).
 * The kernels run in the device's primary context, the one the CUDA runtime
 * (and so the product library and PyTorch) uses, so device pointers from
 * either side are valid here.
 *
 * Kernel names are the Itanium-mangled names of the reference's signatures:
 *   Leapfrog_HH(Float**, int, Float, curandState_t*)            src/ephys.cu:28, src_wholebrain/ephys.cu:149
 *   init_random(unsigned int, int, curandState_t*)                src/ephys.cu:4
 *   signal_spikes_kernel(int, int const*, int const*, int const*, Float*, Float const*)
 *                                                src/coupling.cu:34-39, src_wholebrain/coupling.cu:12-17
 *   signal_spikes_kernel_chunked(int, int* const*, int* const*, int const*, Float*, Float*, Float const*)
 *                                                                 src/coupling.cu:50-57
 *   merge_kernel(Float*, Float*)                                  src/coupling.cu:90-92
 */
#include <cuda.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#define RK_API __attribute__((visibility("default")))

/* Variant 0: src/; variant 1: src_wholebrain/ (no chunked coupling). */
static char g_err[512];
static CUcontext g_ctx;
static CUmodule g_ephys[2], g_coupling[2];
static CUfunction f_leapfrog[2], f_init_random[2], f_signal[2], f_signal_chunked, f_merge;
static int g_loaded;

RK_API const char* rk_last_error(void) { return g_err; }

static int fail(CUresult r, const char* what)
{
    const char* s = NULL;
    cuGetErrorString(r, &s);
    snprintf(g_err, sizeof g_err, "%s: %s (%d)", what, s ? s : "unknown error", (int)r);
    return (int)r;
}

#define RK_TRY(call, what)                      \
    do {                                        \
        CUresult r_ = (call);                   \
        if (r_ != CUDA_SUCCESS) return fail(r_, what); \
    } while (0)

/* Load the four cubins on `device` (primary context): the src/ ephys and
 * coupling modules, then the whole-brain ones.  Returns 0 or a CUresult. */
RK_API int rk_load(int device, const char* ephys_cubin, const char* coupling_cubin, const char* wb_ephys_cubin,
                   const char* wb_coupling_cubin)
{
    if (g_loaded) return 0;
    CUdevice dev;
    RK_TRY(cuInit(0), "cuInit");
    RK_TRY(cuDeviceGet(&dev, device), "cuDeviceGet");
    RK_TRY(cuDevicePrimaryCtxRetain(&g_ctx, dev), "cuDevicePrimaryCtxRetain");
    RK_TRY(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent");
    const char* ephys[2] = {ephys_cubin, wb_ephys_cubin};
    const char* coupling[2] = {coupling_cubin, wb_coupling_cubin};
    for (int v = 0; v < 2; ++v) {
        RK_TRY(cuModuleLoad(&g_ephys[v], ephys[v]), "cuModuleLoad(ephys)");
        RK_TRY(cuModuleLoad(&g_coupling[v], coupling[v]), "cuModuleLoad(coupling)");
        RK_TRY(cuModuleGetFunction(&f_leapfrog[v], g_ephys[v], "_Z11Leapfrog_HHPPfifP17curandStateXORWOW"),
               "Leapfrog_HH");
        RK_TRY(cuModuleGetFunction(&f_init_random[v], g_ephys[v], "_Z11init_randomjiP17curandStateXORWOW"),
               "init_random");
        RK_TRY(cuModuleGetFunction(&f_signal[v], g_coupling[v], "_Z20signal_spikes_kerneliPKiS0_S0_PfPKf"),
               "signal_spikes_kernel");
    }
    RK_TRY(cuModuleGetFunction(&f_signal_chunked, g_coupling[0], "_Z28signal_spikes_kernel_chunkediPKPiS1_PKiPfS4_PKf"),
           "signal_spikes_kernel_chunked");
    RK_TRY(cuModuleGetFunction(&f_merge, g_coupling[0], "_Z12merge_kernelPfS_"), "merge_kernel");
    g_loaded = 1;
    return 0;
}

static int variant_ok(int v, const char* what)
{
    if (v == 0 || v == 1) return 1;
    snprintf(g_err, sizeof g_err, "%s: variant must be 0 (src) or 1 (src_wholebrain)", what);
    return 0;
}

static int launch(CUfunction f, int grid, int block, void** args, const char* what)
{
    if (!g_loaded) {
        snprintf(g_err, sizeof g_err, "%s: rk_load has not succeeded", what);
        return -1;
    }
    RK_TRY(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent");
    RK_TRY(cuLaunchKernel(f, (unsigned)grid, 1, 1, (unsigned)block, 1, 1, 0, NULL, args, NULL), what);
    RK_TRY(cuCtxSynchronize(), what);
    return 0;
}

/* Leapfrog_HH(sim_vars, N, timestep, random_states): d_sim_vars is a device
 * array of 17 device pointers (the SoA table), d_states N curandState_t. */
RK_API int rk_leapfrog(int variant, uint64_t d_sim_vars, int n, float dt, uint64_t d_states, int grid, int block)
{
    if (!variant_ok(variant, "rk_leapfrog")) return -1;
    CUdeviceptr vars = (CUdeviceptr)d_sim_vars, st = (CUdeviceptr)d_states;
    void* args[] = {&vars, &n, &dt, &st};
    return launch(f_leapfrog[variant], grid, block, args, "Leapfrog_HH");
}

/* init_random(seed, N, states): curand_init(seed, idx, 0, &states[idx]). */
RK_API int rk_init_random(unsigned seed, int n, uint64_t d_states, int grid, int block)
{
    CUdeviceptr st = (CUdeviceptr)d_states;
    void* args[] = {&seed, &n, &st};
    return launch(f_init_random[0], grid, block, args, "init_random");
}

/* signal_spikes_kernel(num_firing, connectivity, offsets, firing_inds, spikes, outputs). */
RK_API int rk_signal_spikes(int variant, int num_firing, uint64_t d_conn, uint64_t d_off, uint64_t d_firing,
                            uint64_t d_spikes, uint64_t d_outputs, int grid, int block)
{
    if (!variant_ok(variant, "rk_signal_spikes")) return -1;
    CUdeviceptr c = (CUdeviceptr)d_conn, o = (CUdeviceptr)d_off, f = (CUdeviceptr)d_firing;
    CUdeviceptr s = (CUdeviceptr)d_spikes, out = (CUdeviceptr)d_outputs;
    void* args[] = {&num_firing, &c, &o, &f, &s, &out};
    return launch(f_signal[variant], grid, block, args, "signal_spikes_kernel");
}

/* signal_spikes_kernel_chunked + merge_kernel, both <<<32, 64>>> as the
 * reference launches them (their indexing uses gridDim.x).  d_conn_chunks /
 * d_off_chunks: device arrays of 2 device pointers; d_copies: 32 * 2 * 7319
 * floats; d_spikes: at least 2 * 7319 floats (merge_kernel writes the whole
 * chunk range).  The caller zeroes d_spikes and d_copies first, as the
 * reference does after the first call. */
RK_API int rk_signal_spikes_chunked(int num_firing, uint64_t d_conn_chunks, uint64_t d_off_chunks, uint64_t d_firing,
                                    uint64_t d_copies, uint64_t d_spikes, uint64_t d_outputs)
{
    CUdeviceptr c = (CUdeviceptr)d_conn_chunks, o = (CUdeviceptr)d_off_chunks, f = (CUdeviceptr)d_firing;
    CUdeviceptr cp = (CUdeviceptr)d_copies, s = (CUdeviceptr)d_spikes, out = (CUdeviceptr)d_outputs;
    void* args[] = {&num_firing, &c, &o, &f, &cp, &s, &out};
    int rc = launch(f_signal_chunked, 32, 64, args, "signal_spikes_kernel_chunked");
    if (rc) return rc;
    void* margs[] = {&cp, &s};
    return launch(f_merge, 32, 64, margs, "merge_kernel");
}

/* Mean milliseconds per Leapfrog_HH launch over `reps` back-to-back launches
 * (CUDA events on the legacy stream, no synchronisation between launches). */
RK_API int rk_time_leapfrog(int variant, uint64_t d_sim_vars, int n, float dt, uint64_t d_states, int grid, int block, int reps,
                            float* ms)
{
    if (!g_loaded || reps < 1 || !ms || !variant_ok(variant, "rk_time_leapfrog")) {
        if (!g_err[0]) snprintf(g_err, sizeof g_err, "rk_time_leapfrog: bad arguments or not loaded");
        return -1;
    }
    CUdeviceptr vars = (CUdeviceptr)d_sim_vars, st = (CUdeviceptr)d_states;
    void* args[] = {&vars, &n, &dt, &st};
    CUevent e0, e1;
    RK_TRY(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent");
    RK_TRY(cuEventCreate(&e0, CU_EVENT_DEFAULT), "cuEventCreate");
    RK_TRY(cuEventCreate(&e1, CU_EVENT_DEFAULT), "cuEventCreate");
    RK_TRY(cuEventRecord(e0, NULL), "cuEventRecord");
    for (int r = 0; r < reps; ++r)
        RK_TRY(cuLaunchKernel(f_leapfrog[variant], (unsigned)grid, 1, 1, (unsigned)block, 1, 1, 0, NULL, args, NULL),
               "Leapfrog_HH");
    RK_TRY(cuEventRecord(e1, NULL), "cuEventRecord");
    RK_TRY(cuEventSynchronize(e1), "cuEventSynchronize");
    float t = 0.0f;
    RK_TRY(cuEventElapsedTime(&t, e0, e1), "cuEventElapsedTime");
    cuEventDestroy(e0);
    cuEventDestroy(e1);
    *ms = t / (float)reps;
    return 0;
}

/* Mean milliseconds per signal_spikes_kernel launch (same timing rule). */
RK_API int rk_time_signal_spikes(int variant, int num_firing, uint64_t d_conn, uint64_t d_off, uint64_t d_firing,
                                 uint64_t d_spikes, uint64_t d_outputs, int grid, int block, int reps, float* ms)
{
    if (!g_loaded || reps < 1 || !ms || !variant_ok(variant, "rk_time_signal_spikes")) {
        if (!g_err[0]) snprintf(g_err, sizeof g_err, "rk_time_signal_spikes: bad arguments or not loaded");
        return -1;
    }
    CUdeviceptr c = (CUdeviceptr)d_conn, o = (CUdeviceptr)d_off, f = (CUdeviceptr)d_firing;
    CUdeviceptr s = (CUdeviceptr)d_spikes, out = (CUdeviceptr)d_outputs;
    void* args[] = {&num_firing, &c, &o, &f, &s, &out};
    CUevent e0, e1;
    RK_TRY(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent");
    RK_TRY(cuEventCreate(&e0, CU_EVENT_DEFAULT), "cuEventCreate");
    RK_TRY(cuEventCreate(&e1, CU_EVENT_DEFAULT), "cuEventCreate");
    RK_TRY(cuEventRecord(e0, NULL), "cuEventRecord");
    for (int r = 0; r < reps; ++r)
        RK_TRY(cuLaunchKernel(f_signal[variant], (unsigned)grid, 1, 1, (unsigned)block, 1, 1, 0, NULL, args, NULL),
               "signal_spikes_kernel");
    RK_TRY(cuEventRecord(e1, NULL), "cuEventRecord");
    RK_TRY(cuEventSynchronize(e1), "cuEventSynchronize");
    float t = 0.0f;
    RK_TRY(cuEventElapsedTime(&t, e0, e1), "cuEventElapsedTime");
    cuEventDestroy(e0);
    cuEventDestroy(e1);
    *ms = t / (float)reps;
    return 0;
}

/* Device memory for callers that use the harness without the product
 * library (the benchmark's reference arm). */
RK_API int rk_malloc(uint64_t bytes, uint64_t* dptr)
{
    if (!g_loaded || !dptr) {
        snprintf(g_err, sizeof g_err, "rk_malloc: not loaded or bad argument");
        return -1;
    }
    CUdeviceptr p = 0;
    RK_TRY(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent");
    RK_TRY(cuMemAlloc(&p, (size_t)(bytes ? bytes : 1)), "cuMemAlloc");
    *dptr = (uint64_t)p;
    return 0;
}

RK_API int rk_free(uint64_t dptr)
{
    if (!g_loaded) return -1;
    RK_TRY(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent");
    RK_TRY(cuMemFree((CUdeviceptr)dptr), "cuMemFree");
    return 0;
}

RK_API int rk_h2d(uint64_t dst, const void* src, uint64_t bytes)
{
    if (!g_loaded) return -1;
    RK_TRY(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent");
    RK_TRY(cuMemcpyHtoD((CUdeviceptr)dst, src, (size_t)bytes), "cuMemcpyHtoD");
    return 0;
}

RK_API int rk_d2h(void* dst, uint64_t src, uint64_t bytes)
{
    if (!g_loaded) return -1;
    RK_TRY(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent");
    RK_TRY(cuMemcpyDtoH(dst, (CUdeviceptr)src, (size_t)bytes), "cuMemcpyDtoH");
    return 0;
}

RK_API int rk_memset(uint64_t dst, uint64_t bytes)
{
    if (!g_loaded) return -1;
    RK_TRY(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent");
    RK_TRY(cuMemsetD8((CUdeviceptr)dst, 0, (size_t)bytes), "cuMemsetD8");
    return 0;
}

RK_API int rk_num_sms(int* out)
{
    if (!g_loaded || !out) return -1;
    CUdevice dev;
    RK_TRY(cuCtxGetDevice(&dev), "cuCtxGetDevice");
    RK_TRY(cuDeviceGetAttribute(out, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, dev), "cuDeviceGetAttribute");
    return 0;
}
