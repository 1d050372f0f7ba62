/* The device-resident simulation driven from a plain C host through the C ABI
 * (include/neuronephys.h), the way a caller replaces the reference's step loop
 * (src/main.cu:166-181): a seeded random network handed over as host CSR, the
 * default initial state, steps advanced on the device, electrode recording
 * inside the step (ElectrodeNet, src/electrode_net.cu:3-49), then the step
 * counter, the spike total, the membrane potentials and the electrode samples
 * read back.
 * Usage: sim_host <N> <steps> <delivery>; prints
 * "N step spikes mean_V samples first_step last_sample_region0_mean". */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "neuronephys.h"

#define CHECK(call)                                                                                    \
    do {                                                                                               \
        nn_status st_ = (call);                                                                        \
        if (st_ != NN_OK) {                                                                            \
            fprintf(stderr, "%s: %s (%s)\n", #call, nn_status_string(st_), ctx ? nn_ctx_last_error(ctx) : ""); \
            return 1;                                                                                  \
        }                                                                                              \
    } while (0)

enum { K = 10, DMAX = 20, REGION = 50, CAPACITY = 1024, EVERY = 40 };

/* 64-bit linear congruential generator (Knuth's MMIX constants), top 31 bits */
static uint32_t lcg(uint64_t* s)
{
    *s = *s * 6364136223846793005ULL + 1442695040888963407ULL;
    return (uint32_t)(*s >> 33);
}

int main(int argc, char** argv)
{
    const int n = argc > 1 ? atoi(argv[1]) : 2000;
    const int steps = argc > 2 ? atoi(argv[2]) : 1000;
    const int delivery = argc > 3 ? atoi(argv[3]) : NN_DELIVERY_PULL;
    const int64_t nnz = (int64_t)n * K;
    const int regions = n / REGION;
    nn_ctx* ctx = NULL;
    nn_sim* sim = NULL;
    nn_sim_config cfg;
    uint64_t seed = 12345;
    int64_t i, step = 0, spikes = 0, first = 0;
    int samples = 0;
    double mean = 0.0;

    int64_t* row_ptr = malloc(sizeof(int64_t) * (size_t)(n + 1));
    int32_t* col = malloc(sizeof(int32_t) * (size_t)nnz);
    float* weight = malloc(sizeof(float) * (size_t)nnz);
    uint8_t* delay = malloc((size_t)nnz);
    uint8_t* is_inh = malloc((size_t)n);
    int* members = malloc(sizeof(int) * (size_t)(regions * REGION));
    int* offsets = malloc(sizeof(int) * (size_t)(regions + 1));
    float* v = malloc(sizeof(float) * (size_t)n);
    float* avg = malloc(sizeof(float) * (size_t)CAPACITY * (size_t)regions);
    int* firing = malloc(sizeof(int) * (size_t)CAPACITY * (size_t)regions);
    if (!row_ptr || !col || !weight || !delay || !is_inh || !members || !offsets || !v || !avg || !firing) return 1;

    /* K random targets per neuron, weights U(0, 0.5] nS, delays 1..DMAX, the
     * last fifth inhibitory */
    for (i = 0; i < n; ++i) {
        int j;
        row_ptr[i] = i * K;
        for (j = 0; j < K; ++j) {
            const int64_t e = i * K + j;
            col[e] = (int32_t)(lcg(&seed) % (uint32_t)n);
            weight[e] = 0.5f * (float)(lcg(&seed) % 1000u + 1u) / 1000.0f;
            delay[e] = (uint8_t)(1u + lcg(&seed) % DMAX);
        }
        is_inh[i] = (uint8_t)(i >= n - n / 5);
    }
    row_ptr[n] = nnz;
    for (i = 0; i < (int64_t)regions * REGION; ++i) members[i] = (int)i;
    for (i = 0; i <= regions; ++i) offsets[i] = (int)(i * REGION);

    CHECK(nn_ctx_create(0, &ctx));
    nn_sim_config_default(&cfg, n);
    cfg.max_delay = DMAX;
    cfg.grid = 16;
    cfg.delivery = delivery;
    CHECK(nn_sim_create(ctx, &cfg, &sim));
    CHECK(nn_sim_set_network(sim, row_ptr, col, weight, delay, nnz, is_inh));
    CHECK(nn_sim_init_state(sim, -65.0f, 6.0f, 12.0f));
    CHECK(nn_sim_set_electrodes(sim, members, offsets, regions, EVERY, CAPACITY));
    CHECK(nn_sim_step(sim, steps));
    CHECK(nn_sim_counters(sim, &step, &spikes));
    CHECK(nn_sim_get_field(sim, NN_F_V, v));
    CHECK(nn_sim_read_electrodes(sim, avg, firing, &first, &samples));
    for (i = 0; i < n; ++i) mean += v[i];
    printf("%d %lld %lld %.9f %d %lld %.9f\n", n, (long long)step, (long long)spikes, mean / n, samples,
           (long long)first, samples > 0 ? (double)avg[(size_t)(samples - 1) * (size_t)regions] : 0.0);
    CHECK(nn_sim_destroy(sim));
    CHECK(nn_ctx_destroy(ctx));
    free(row_ptr); free(col); free(weight); free(delay); free(is_inh);
    free(members); free(offsets); free(v); free(avg); free(firing);
    return 0;
}
