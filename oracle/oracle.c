/*
 * oracle.c -- CPU restatement of the neuronephys simulation path.
 * TEST INFRASTRUCTURE ONLY (see oracle.h): the product library never links
 * or calls this file.  Build: gcc -O2 -ffp-contract=off -fopenmp -shared.
 *
 * -ffp-contract=off keeps every float operation individually rounded, so the
 * counter-based generators reproduce the CUDA generators (which use explicit
 * __fmul_rn/__fadd_rn) bit for bit.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ RNG -- */

static inline void mulhilo32(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo)
{
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
        mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Philox2x32-10, same paper: two counter words, one key word */
void orc_philox2x32_10(const uint32_t ctr[2], uint32_t key, uint32_t out[2])
{
    uint32_t c0 = ctr[0], c1 = ctr[1];
    for (int r = 0; r < 10; ++r) {
        uint32_t hi, lo;
        mulhilo32(0xD256D193u, c0, &hi, &lo);
        const uint32_t n0 = hi ^ key ^ c1;
        c1 = lo;
        c0 = n0;
        key += 0x9E3779B9u;
    }
    out[0] = c0;
    out[1] = c1;
}

/* the neuron-update noise key: both seed words and the high step word mixed
 * into Philox2x32's single key word */
static inline uint32_t noise_key(uint64_t seed, uint64_t step)
{
    return (uint32_t)seed + 0x9E3779B9u * (uint32_t)(seed >> 32) + 0x85EBCA6Bu * (uint32_t)(step >> 32);
}

static inline void philox(uint64_t seed, uint32_t a, uint32_t b, uint32_t c, uint32_t purpose, uint32_t out[4])
{
    uint32_t ctr[4] = {a, b, c, purpose};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    orc_philox4x32_10(ctr, key, out);
}

static inline double u01_closed_open(uint32_t x) { return (double)(x >> 8) * (1.0 / 16777216.0); }
static inline double u01_open_closed(uint32_t x) { return (double)((x >> 8) + 1u) * (1.0 / 16777216.0); }

double orc_normal_ctr(uint64_t seed, uint32_t i, uint64_t step, uint32_t purpose)
{
    /* one Philox2x32-10 draw per neuron pair (i>>1) and step, counter
     * (pair, low step word), key noise_key(seed, step): cos branch for even i,
     * sin for odd i.  (purpose: the noise stream is the only user) */
    (void)purpose;
    const uint32_t ctr[2] = {i >> 1, (uint32_t)step};
    uint32_t r[2];
    orc_philox2x32_10(ctr, noise_key(seed, step), r);
    double u1 = u01_open_closed(r[0]);
    double u2 = u01_closed_open(r[1]);
    double rad = sqrt(-2.0 * log(u1));
    return (i & 1u) ? rad * sin(2.0 * M_PI * u2) : rad * cos(2.0 * M_PI * u2);
}

uint32_t orc_minstd_next(uint32_t* state)
{
    uint64_t x = ((uint64_t)(*state) * 16807u) % 2147483647u;
    *state = (uint32_t)x;
    return (uint32_t)x;
}

/* libstdc++ uniform_int_distribution<int>::operator(): the generator's range
 * [1, 2147483646] is wider than the requested range, so it downscales by
 * rejection: scaling = urngrange / (b - a + 1), reject draws >= past. */
int orc_uniform_int(uint32_t* state, int a, int b)
{
    const uint64_t urngmin = 1, urngmax = 2147483646u;
    const uint64_t urngrange = urngmax - urngmin;
    const uint64_t urange = (uint64_t)((int64_t)b - (int64_t)a);
    uint64_t ret;
    if (urngrange > urange) {
        const uint64_t uerange = urange + 1;
        const uint64_t scaling = urngrange / uerange;
        const uint64_t past = uerange * scaling;
        do {
            ret = (uint64_t)orc_minstd_next(state) - urngmin;
        } while (ret >= past);
        ret /= scaling;
    } else {
        ret = (uint64_t)orc_minstd_next(state) - urngmin;
    }
    return (int)(ret + (uint64_t)(int64_t)a);
}

/* ------------------------------------------- reference network factory -- */

/* src/network_factory.cu:96-131: for every neuron draw ncouple distinct
 * targets from U{0..n-1} (self-loops allowed), redrawing duplicates. */
void orc_uniform_random_network(int n, int ncouple, uint32_t* engine, int* indices, int* offsets)
{
    for (int i = 0; i < n; ++i) {
        int* row = indices + (int64_t)i * ncouple;
        for (int j = 0; j < ncouple; ++j) {
            int d;
            int dup;
            do {
                d = orc_uniform_int(engine, 0, n - 1);
                dup = 0;
                for (int q = 0; q < j; ++q)
                    if (row[q] == d) { dup = 1; break; }
            } while (dup);
            row[j] = d;
        }
        offsets[i] = i * ncouple;
    }
    offsets[n] = n * ncouple;
}

/* src/network_factory.cu:19-22 (and :40-43): ++Tcount[target] per entry. */
void orc_tcount(const int* indices, int64_t nnz, int n, float* tcount)
{
    for (int i = 0; i < n; ++i) tcount[i] = 0.0f;
    for (int64_t e = 0; e < nnz; ++e) tcount[indices[e]] += 1.0f;
}

/* src/network_factory.cu:45-63. */
void orc_chunked(const int* indices, const int* offsets, int n, int nchunks, int n_per_chunk,
                 int** chunk_indices, int** chunk_offsets, int64_t* chunk_nnz)
{
    for (int c = 0; c < nchunks; ++c) {
        chunk_nnz[c] = 0;
        chunk_offsets[c][0] = 0;
    }
    for (int i = 1; i < n + 1; ++i) {
        for (int c = 0; c < nchunks; ++c) chunk_offsets[c][i] = chunk_offsets[c][i - 1];
        for (int j = offsets[i - 1]; j < offsets[i]; ++j) {
            int ds = indices[j];
            int c = ds / n_per_chunk;
            chunk_indices[c][chunk_nnz[c]++] = ds % n_per_chunk;
            chunk_offsets[c][i] += 1;
        }
    }
}

/* --------------------------------------------------- reference ephys ---- */

void orc_leapfrog_params_src(orc_leapfrog_params* p)
{
    /* src/defines.cuh:87-102 */
    p->gna = 120.0f; p->ena = 55.0f; p->gk = 36.0f; p->ek = -72.0f; p->gl = 0.3f; p->el = -50.0f;
    p->Tmax = 1.0f; p->Vt = -20.0f; p->Kp = 3.0f; p->Ar = 5.0f; p->Ad = 0.18f;
    p->g_local = 0.1f; p->e_local = 0.0f; p->g_gaba = 0.1f; p->e_gaba = -70.0f;
    p->g_exc = 0.1f; p->e_exc = 0.0f;
    p->noise_mean = 3.0f; p->noise_intensity = 1.5f;
}

void orc_leapfrog_params_wholebrain(orc_leapfrog_params* p)
{
    /* src_wholebrain/ephys.cuh:47-61: grey AMPA on the local channel, no
     * GABA, no white-matter AMPA, zero-mean noise of intensity 2. */
    orc_leapfrog_params_src(p);
    p->g_local = 0.1f; p->g_gaba = 0.0f; p->g_exc = 0.0f;
    p->noise_mean = 0.0f; p->noise_intensity = 2.0f;
}

static inline double kinetic_cn(double A, double B, double x, double dt)
{
    /* Crank-Nicolson update of dx/dt = A (1-x) - B x  (src/ephys.cu:65-67). */
    return (A * dt + (1.0 - dt / 2.0 * (A + B)) * x) / (dt / 2.0 * (A + B) + 1.0);
}

void orc_hh_leapfrog(float* const* vars, int n, float dtf, const orc_leapfrog_params* p, const double* z)
{
    const double dt = dtf;
    for (int i = 0; i < n; ++i) {
        const double V = vars[ORC_V][i], M = vars[ORC_M][i], N = vars[ORC_N][i], H = vars[ORC_H][i];
        const double LY = vars[ORC_LOCAL_Y][i], IY = vars[ORC_IY][i], EY = vars[ORC_EY][i];
        /* src/ephys.cu:57-63 */
        const double Am = (3.5 + 0.1 * V) / (1.0 - exp(-3.5 - 0.1 * V));
        const double An = (-0.5 - 0.01 * V) / (exp(-5.0 - 0.1 * V) - 1.0);
        const double Ah = 0.07 * exp(-V / 20.0 - 3.0);
        const double Bm = 4.0 * exp(-(V + 60.0) / 18.0);
        const double Bn = 0.125 * exp(-(V + 60.0) / 80.0);
        const double Bh = 1.0 / (exp(-3.0 - 0.1 * V) + 1.0);
        /* :65-67 */
        const double nM = kinetic_cn(Am, Bm, M, dt);
        const double nN = kinetic_cn(An, Bn, N, dt);
        const double nH = kinetic_cn(Ah, Bh, H, dt);
        /* :69-76: transmitter input normalised by in-degree */
        const double lin = vars[ORC_LOCAL_IN][i], lcnt = vars[ORC_LOCAL_COUNT][i];
        const double iin = vars[ORC_IIN][i], icnt = vars[ORC_ICOUNT][i];
        const double ein = vars[ORC_EIN][i], ecnt = vars[ORC_ECOUNT][i];
        const double lT = lcnt > 0 ? lin / lcnt : 0.0;
        const double iT = icnt > 0 ? iin / icnt : 0.0;
        const double eT = ecnt > 0 ? ein / ecnt : 0.0;
        const double nLY = kinetic_cn(p->Ar * lT, p->Ad, LY, dt);
        const double nIY = kinetic_cn(p->Ar * iT, p->Ad, IY, dt);
        const double nEY = kinetic_cn(p->Ar * eT, p->Ad, EY, dt);
        /* :78-79 */
        const double gna = p->gna * nM * nM * nM * nH;
        const double gk = p->gk * nN * nN * nN * nN;
        const double G = gna + gk + p->gl + p->g_local * nLY + p->g_gaba * nIY + p->g_exc * nEY;
        const double E = gna * p->ena + gk * p->ek + p->gl * p->el + p->g_local * nLY * p->e_local
                       + p->g_gaba * nIY * p->e_gaba + p->g_exc * nEY * p->e_exc;
        /* :82-85 */
        const double noise = (double)p->noise_intensity * z[i] + (double)p->noise_mean;
        const double appcur = vars[ORC_APPCUR][i];
        const double nV = ((noise + appcur) * dt + E * dt + (1.0 - dt / 2.0 * G) * V) / (1.0 + dt / 2.0 * G);
        vars[ORC_V][i] = (float)nV;
        vars[ORC_M][i] = (float)nM;
        vars[ORC_N][i] = (float)nN;
        vars[ORC_H][i] = (float)nH;
        vars[ORC_LOCAL_Y][i] = (float)nLY;
        vars[ORC_IY][i] = (float)nIY;
        vars[ORC_EY][i] = (float)nEY;
        /* :94: transmitter output from the stored (float) voltage */
        const double out = (double)p->Tmax / (1.0 + exp(-((double)vars[ORC_V][i] - (double)p->Vt) / (double)p->Kp));
        vars[ORC_LOCAL_OUTPUT][i] = vars[ORC_IOUTPUT][i] = vars[ORC_EOUTPUT][i] = (float)out;
    }
}

/* ------------------------------------------------ reference coupling ---- */

int orc_coupling_push(int n, const int* indices, const int* offsets, const float* outputs,
                      float* inputs, int signal_mode, int* firing_list)
{
    int nf = 0;
    for (int i = 0; i < n; ++i) inputs[i] = 0.0f;
    for (int i = 0; i < n; ++i)
        if (outputs[i] > 0.1f) firing_list[nf++] = i;
    for (int f = 0; f < nf; ++f) {
        const int pre = firing_list[f];
        const float sig = signal_mode ? outputs[pre] : 1.0f;
        for (int e = offsets[pre]; e < offsets[pre + 1]; ++e) inputs[indices[e]] += sig;
    }
    return nf;
}

/* ----------------------------------------------- reference paracrine ---- */

void orc_trilinear_setup(int n, const float* x, const float* y, const float* z,
                         int nx, int ny, int nz, float h, int* idx8, float* w8)
{
    const float Lx = (float)(nx - 1) * h, Ly = (float)(ny - 1) * h, Lz = (float)(nz - 1) * h;
    for (int i = 0; i < n; ++i) {
        /* src/paracrine.cu:143-147 (and y, z) */
        const float xr = x[i] / Lx + 0.5f, yr = y[i] / Ly + 0.5f, zr = z[i] / Lz + 0.5f;
        const float sx = (float)(nx - 1) * xr, sy = (float)(ny - 1) * yr, sz = (float)(nz - 1) * zr;
        const int m = (int)sx, q = (int)sy, p = (int)sz;
        /* :201-205 */
        const float fx = sx - (float)m, fy = sy - (float)q, fz = sz - (float)p;
        /* :172-178 and the corner offsets :189-195 */
        const int base = m + q * nx + p * nx * ny;
        const int off[8] = {0, 1, nx, nx + 1, nx * ny, nx * ny + 1, nx * ny + nx, nx * ny + nx + 1};
        /* :223-257: w0..3 = xy products times (1 - fz); w4..7 times fz */
        const float kx0 = 1.0f - fx, ky0 = 1.0f - fy, kz0 = 1.0f - fz;
        const float kx1 = 1.0f - (1.0f - fx), ky1 = 1.0f - (1.0f - fy), kz1 = 1.0f - (1.0f - fz);
        const float xy[4] = {kx0 * ky0, kx1 * ky0, kx0 * ky1, kx1 * ky1};
        for (int c = 0; c < 4; ++c) {
            w8[8 * i + c + 4] = xy[c] * kz1;
            w8[8 * i + c] = xy[c] * kz0;
        }
        for (int c = 0; c < 8; ++c) idx8[8 * i + c] = base + off[c];
    }
}

void orc_scatter(int n, const int* idx8, const float* w8, const double* s, double* grid)
{
    for (int i = 0; i < n; ++i)
        for (int c = 0; c < 8; ++c) grid[idx8[8 * i + c]] += (double)w8[8 * i + c] * s[i];
}

void orc_interp(int n, const int* idx8, const float* w8, const double* grid, double* out)
{
    for (int i = 0; i < n; ++i) {
        double acc = 0.0;
        for (int c = 0; c < 8; ++c) acc += (double)w8[8 * i + c] * grid[idx8[8 * i + c]];
        out[i] = acc;
    }
}

void orc_conv27(const double* in, double* out, int nx, int ny, int nz, const double K[27])
{
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double acc = 0.0;
                for (int c = -1; c <= 1; ++c) {
                    const int kk = k + c;
                    if (kk < 0 || kk >= nz) continue;
                    for (int b = -1; b <= 1; ++b) {
                        const int jj = j + b;
                        if (jj < 0 || jj >= ny) continue;
                        for (int a = -1; a <= 1; ++a) {
                            const int ii = i + a;
                            if (ii < 0 || ii >= nx) continue;
                            acc += K[(a + 1) + 3 * (b + 1) + 9 * (c + 1)] * in[ii + nx * ((int64_t)jj + (int64_t)ny * kk)];
                        }
                    }
                }
                out[i + nx * ((int64_t)j + (int64_t)ny * k)] = acc;
            }
}

static double dot(const double* a, const double* b, int64_t n)
{
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

int orc_paracrine_cn_solve(double* u, int nx, int ny, int nz, double h, double D, double k,
                           double dt, double abs_tol, int max_iter, int quirk_b, double* final_rr)
{
    /* src/paracrine.cu:40-43: {1,3,14,-128} compact stencil scaled by 1/(30 h^2). */
    static const double st[27] = {1, 3, 1, 3, 14, 3, 1, 3, 1, 3, 14, 3, 14, -128, 14, 3, 14, 3,
                                  1, 3, 1, 3, 14, 3, 1, 3, 1};
    double L[27], A[27];
    for (int q = 0; q < 27; ++q) {
        L[q] = st[q] * (1.0 / (h * h * 30.0));
        A[q] = -0.5 * D * dt * L[q]; /* :80 */
    }
    A[13] += 1.0 + 0.5 * dt * k; /* :81 */
    const int64_t G = (int64_t)nx * ny * nz;
    double* lap = (double*)malloc(sizeof(double) * G);
    double* x = (double*)malloc(sizeof(double) * G);
    double* b = (double*)malloc(sizeof(double) * G);
    double* r = (double*)malloc(sizeof(double) * G);
    double* p = (double*)malloc(sizeof(double) * G);
    double* Ap = (double*)malloc(sizeof(double) * G);
    orc_conv27(u, lap, nx, ny, nz, L); /* :70 */
    const double c = quirk_b ? h : dt; /* :105 uses spatial_gridsize */
    for (int64_t q = 0; q < G; ++q) {
        x[q] = (1.0 - dt * k) * u[q] + dt * D * lap[q];          /* :73 */
        b[q] = (1.0 - c * k / 2.0) * u[q] + c * D / 2.0 * lap[q]; /* :105 */
    }
    orc_conv27(x, Ap, nx, ny, nz, A);
    for (int64_t q = 0; q < G; ++q) { r[q] = b[q] - Ap[q]; p[q] = r[q]; } /* :110-112 */
    double rr = dot(r, r, G);
    int it = 0;
    if (rr < abs_tol) {
        /* :114-116: the density is left unchanged */
        if (final_rr) *final_rr = rr;
        free(lap); free(x); free(b); free(r); free(p); free(Ap);
        return 0;
    }
    for (int i = 0; i < max_iter; ++i) { /* :118-129 */
        it = i + 1;
        orc_conv27(p, Ap, nx, ny, nz, A);
        const double pAp = dot(p, Ap, G);
        const double alpha = rr / pAp;
        for (int64_t q = 0; q < G; ++q) { x[q] += alpha * p[q]; r[q] -= alpha * Ap[q]; }
        const double rr_new = dot(r, r, G);
        if (rr_new < abs_tol) { rr = rr_new; break; }
        const double beta = rr_new / rr;
        for (int64_t q = 0; q < G; ++q) p[q] = r[q] + beta * p[q];
        rr = rr_new;
    }
    memcpy(u, x, sizeof(double) * G); /* :130 */
    if (final_rr) *final_rr = rr;
    free(lap); free(x); free(b); free(r); free(p); free(Ap);
    return it;
}

/* ------------------------------------------- GB300 model semantics ------ */

void orc_hh_params_standard(orc_hh_params* p)
{
    p->C = 1.0; p->gNa = 120.0; p->gK = 36.0; p->gL = 0.3;
    p->ENa = 50.0; p->EK = -77.0; p->EL = -54.4;
    p->E_exc = 0.0; p->E_inh = -80.0; p->tau_exc = 5.0; p->tau_inh = 5.0;
    p->v_thresh = -20.0; p->noise_sigma = 1.0; p->dt = 0.01;
    p->g_par = 0.0; p->E_par = 0.0;
}

/* u / (1 - exp(-u)), with its series near u = 0. */
static inline double xexprel(double u)
{
    if (fabs(u) < 1e-4) return 1.0 + 0.5 * u + u * u / 12.0;
    return u / (-expm1(-u));
}

static inline void hh_rates(double V, double r[6])
{
    r[0] = xexprel((V + 40.0) / 10.0);            /* alpha_m = 0.1 (V+40) / (1 - e^{-(V+40)/10}) */
    r[1] = 4.0 * exp(-(V + 65.0) / 18.0);         /* beta_m  */
    r[2] = 0.07 * exp(-(V + 65.0) / 20.0);        /* alpha_h */
    r[3] = 1.0 / (1.0 + exp(-(V + 35.0) / 10.0)); /* beta_h  */
    r[4] = 0.1 * xexprel((V + 55.0) / 10.0);      /* alpha_n = 0.01 (V+55) / (1 - e^{-(V+55)/10}) */
    r[5] = 0.125 * exp(-(V + 65.0) / 80.0);       /* beta_n  */
}

void orc_hh_steady_state(double v, double* m, double* h, double* n)
{
    double r[6];
    hh_rates(v, r);
    *m = r[0] / (r[0] + r[1]);
    *h = r[2] / (r[2] + r[3]);
    *n = r[4] / (r[4] + r[5]);
}

static inline void hh_rhs(const orc_hh_params* p, double gna_scale, double i_ext, double u_par,
                          const double y[6], double f[6])
{
    const double V = y[0], m = y[1], h = y[2], n = y[3], ge = y[4], gi = y[5];
    double r[6];
    hh_rates(V, r);
    const double n2 = n * n;
    const double i_ion = p->gNa * gna_scale * m * m * m * h * (V - p->ENa) + p->gK * n2 * n2 * (V - p->EK)
                       + p->gL * (V - p->EL);
    const double i_syn = ge * (V - p->E_exc) + gi * (V - p->E_inh) + p->g_par * u_par * (V - p->E_par);
    f[0] = (i_ext - i_ion - i_syn) / p->C;
    f[1] = r[0] * (1.0 - m) - r[1] * m;
    f[2] = r[2] * (1.0 - h) - r[3] * h;
    f[3] = r[4] * (1.0 - n) - r[5] * n;
    f[4] = -ge / p->tau_exc;
    f[5] = -gi / p->tau_inh;
}

void orc_hh_rk4(const orc_hh_params* p, double gna_scale, double i_ext, double u_par, double y[6])
{
    const double dt = p->dt;
    double k1[6], k2[6], k3[6], k4[6], t[6];
    hh_rhs(p, gna_scale, i_ext, u_par, y, k1);
    for (int q = 0; q < 6; ++q) t[q] = y[q] + 0.5 * dt * k1[q];
    hh_rhs(p, gna_scale, i_ext, u_par, t, k2);
    for (int q = 0; q < 6; ++q) t[q] = y[q] + 0.5 * dt * k2[q];
    hh_rhs(p, gna_scale, i_ext, u_par, t, k3);
    for (int q = 0; q < 6; ++q) t[q] = y[q] + dt * k3[q];
    hh_rhs(p, gna_scale, i_ext, u_par, t, k4);
    for (int q = 0; q < 6; ++q) y[q] += dt / 6.0 * (k1[q] + 2.0 * k2[q] + 2.0 * k3[q] + k4[q]);
}

void orc_csr_to_csc(const orc_csr* a, int64_t* col_ptr, int32_t* src, float* w, uint8_t* d, int64_t* edge_of)
{
    const int n = a->n;
    int64_t* fill = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    for (int i = 0; i <= n; ++i) col_ptr[i] = 0;
    for (int64_t e = 0; e < a->nnz; ++e) col_ptr[a->col[e] + 1]++;
    for (int i = 0; i < n; ++i) col_ptr[i + 1] += col_ptr[i];
    for (int i = 0; i < n; ++i) {
        for (int64_t e = a->row_ptr[i]; e < a->row_ptr[i + 1]; ++e) {
            const int t = a->col[e];
            const int64_t pos = col_ptr[t] + fill[t]++;
            src[pos] = i;
            if (w) w[pos] = a->weight[e];
            if (d) d[pos] = a->delay[e];
            if (edge_of) edge_of[pos] = e;
        }
    }
    free(fill);
}

/* Purposes of the counter-based streams (shared with the CUDA generators). */
enum { P_NOISE = 1, P_DRIVE = 2, P_POS = 3, P_ER = 4, P_GAUSS = 5, P_WEIGHT = 6, P_TYPE = 7, P_BLOCK = 8, P_REGION = 9 };

void orc_gen_er(int n, double p, float wmax, uint64_t seed, orc_csr* out)
{
    double tf = floor(p * 4294967296.0);
    const uint32_t thr = tf >= 4294967295.0 ? 4294967295u : (uint32_t)tf;
    const int fill = out->col != NULL;
    int64_t pos = 0;
    if (!fill) out->row_ptr[0] = 0;
    for (int i = 0; i < n; ++i) {
        int64_t e = 0;
        uint32_t r[4];
        for (int j = 0; j < n; ++j) {
            if ((j & 3) == 0) philox(seed, (uint32_t)i, (uint32_t)(j >> 2), 0u, P_ER, r);
            if (j == i) continue;
            if (r[j & 3] < thr) {
                if (fill) {
                    uint32_t rw[4];
                    philox(seed, (uint32_t)i, (uint32_t)e, 0u, P_WEIGHT, rw);
                    out->col[pos] = j;
                    out->weight[pos] = wmax * (float)((double)(rw[0] >> 8) * (1.0 / 16777216.0));
                    out->delay[pos] = 1;
                }
                ++pos;
                ++e;
            }
        }
        if (!fill) out->row_ptr[i + 1] = pos;
    }
    out->nnz = pos;
}

/* Inverse normal CDF by bisection on erfc (deterministic, host-side table). */
static double inv_phi(double pr)
{
    double lo = -40.0, hi = 40.0;
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        const double c = 0.5 * erfc(-mid / sqrt(2.0));
        if (c < pr) lo = mid; else hi = mid;
    }
    return 0.5 * (lo + hi);
}

void orc_gauss_table(double sigma_sites, int16_t* table)
{
    for (int m = 0; m < 4096; ++m) {
        const double z = inv_phi(((double)m + 0.5) / 4096.0);
        table[m] = (int16_t)lround(sigma_sites * z);
    }
}

static int lattice_side(int n)
{
    int L = (int)cbrt((double)n);
    while ((int64_t)L * L * L < n) ++L;
    while (L > 1 && (int64_t)(L - 1) * (L - 1) * (L - 1) >= n) --L;
    return L;
}

void orc_lattice_positions(int n, uint64_t seed, float* x, float* y, float* z)
{
    const int L = lattice_side(n);
    for (int i = 0; i < n; ++i) {
        uint32_t r[4];
        philox(seed, (uint32_t)i, 0u, 0u, P_POS, r);
        const int cx = i % L, cy = (i / L) % L, cz = i / (L * L);
        const float ux = (float)(r[0] >> 8) * (1.0f / 16777216.0f);
        const float uy = (float)(r[1] >> 8) * (1.0f / 16777216.0f);
        const float uz = (float)(r[2] >> 8) * (1.0f / 16777216.0f);
        x[i] = ((float)cx + ux) / (float)L;
        y[i] = ((float)cy + uy) / (float)L;
        z[i] = ((float)cz + uz) / (float)L;
    }
}

/* Per-neuron drive current lo + (hi - lo) u, u the 24-bit uniform of the
 * neuron's P_DRIVE draw, in FP32 as the device's k_init_state forms it. */
void orc_init_drive(int n, uint64_t seed, float lo, float hi, float* out)
{
    for (int i = 0; i < n; ++i) {
        uint32_t r[4];
        philox(seed, (uint32_t)i, 0u, 0u, P_DRIVE, r);
        const float u = (float)(r[0] >> 8) * (1.0f / 16777216.0f);
        const float span = hi - lo;
        const float t = span * u;
        out[i] = lo + t;
    }
}

/* Inhibitory flags: the last round(frac * n) indices, or (random) each
 * neuron's P_TYPE draw below floor(frac * 2^32), as the device's k_inh. */
void orc_inh_flags(int n, double frac, int random, uint64_t seed, uint8_t* out)
{
    const int n_inh = (int)llround(frac * n);
    const double tf = floor(frac * 4294967296.0);
    const uint32_t thr = tf >= 4294967295.0 ? 0xffffffffu : (uint32_t)tf;
    for (int i = 0; i < n; ++i) {
        if (random) {
            uint32_t r[4];
            philox(seed, (uint32_t)i, 0u, 0u, P_TYPE, r);
            out[i] = r[0] < thr ? 1 : 0;
        } else {
            out[i] = i >= n - n_inh ? 1 : 0;
        }
    }
}

void orc_gen_gauss(int n, int k, double sigma, double w_mu, double w_sigma, int dmax,
                   uint64_t seed, orc_csr* out)
{
    const int L = lattice_side(n);
    int16_t table[4096];
    orc_gauss_table(sigma * (double)L, table);
    out->nnz = (int64_t)n * k;
    for (int i = 0; i <= n; ++i) out->row_ptr[i] = (int64_t)i * k;
    if (!out->col) return;
    for (int i = 0; i < n; ++i) {
        const int cx = i % L, cy = (i / L) % L, cz = i / (L * L);
        for (int e = 0; e < k; ++e) {
            int tgt = (i + 1) % n;
            for (int a = 0; a < 64; ++a) {
                uint32_t r[4];
                philox(seed, (uint32_t)i, (uint32_t)e, (uint32_t)a, P_GAUSS, r);
                const int tx = cx + table[r[0] >> 20], ty = cy + table[r[1] >> 20], tz = cz + table[r[2] >> 20];
                if (tx < 0 || ty < 0 || tz < 0 || tx >= L || ty >= L || tz >= L) continue;
                const int64_t s = (int64_t)tx + (int64_t)L * ((int64_t)ty + (int64_t)L * tz);
                if (s >= n || s == i) continue;
                tgt = (int)s;
                break;
            }
            uint32_t rw[4];
            philox(seed, (uint32_t)i, (uint32_t)e, 0u, P_WEIGHT, rw);
            const double u1 = u01_open_closed(rw[0]), u2 = u01_closed_open(rw[1]);
            const double zz = sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
            const int64_t pos = (int64_t)i * k + e;
            out->col[pos] = tgt;
            out->weight[pos] = (float)exp(w_mu + w_sigma * zz);
            out->delay[pos] = (uint8_t)(1u + (uint32_t)(((uint64_t)rw[2] * (uint64_t)dmax) >> 32));
        }
    }
}

/* Region-block generator of the 10M-neuron workload (the library's own
 * generator; no reference counterpart).  Regions: lognormal(0, size_sigma)
 * size weights and uniform centroids from Philox(seed; r, 0|1, 0, REGION);
 * sizes 1 + largest-remainder shares of n - R.  Block densities: row r over
 * target regions t, lognormal(0, density_sigma) x size[t], as cumulative
 * 32-bit thresholds; delay 1 + (dmax - 1) * centroid distance / max distance,
 * rounded.  Synapse e of neuron i: target region by the first threshold above
 * u.x of Philox(seed; i, e, attempt, BLOCK), target neuron uniform in it
 * (u.y), redrawn if it is i (64 attempts, then i + 1); weight as in
 * orc_gen_gauss; delay from the region pair. */
void orc_block_tables(int n, int R, double size_sigma, double density_sigma, int dmax, uint64_t seed,
                      int* start, int* size, uint32_t* cum, uint8_t* pdelay)
{
    double* w = (double*)malloc(sizeof(double) * R * 5);
    double *cx = w + R, *cy = w + 2 * R, *cz = w + 3 * R, *fr = w + 4 * R;
    int* order = (int*)malloc(sizeof(int) * R);
    double sw = 0.0;
    for (int r = 0; r < R; ++r) {
        uint32_t u[4], v[4];
        philox(seed, (uint32_t)r, 0u, 0u, P_REGION, u);
        const double u1 = u01_open_closed(u[0]), u2 = u01_closed_open(u[1]);
        const double z = sqrt(-2.0 * log(u1)) * cos(6.283185307179586476925 * u2);
        w[r] = exp(size_sigma * z);
        sw += w[r];
        cx[r] = u01_closed_open(u[2]);
        philox(seed, (uint32_t)r, 1u, 0u, P_REGION, v);
        cy[r] = u01_closed_open(v[0]);
        cz[r] = u01_closed_open(v[1]);
    }
    const int left = n - R;
    int assigned = 0;
    for (int r = 0; r < R; ++r) {
        const double want = left * w[r] / sw;
        const int fl = (int)floor(want);
        size[r] = 1 + fl;
        assigned += fl;
        fr[r] = want - fl;
        order[r] = r;
    }
    /* stable sort by descending remainder (insertion sort; R is small) */
    for (int a = 1; a < R; ++a) {
        const int v = order[a];
        int b = a - 1;
        while (b >= 0 && fr[order[b]] < fr[v]) {
            order[b + 1] = order[b];
            --b;
        }
        order[b + 1] = v;
    }
    for (int q = 0; q < left - assigned; ++q) size[order[q]] += 1;
    start[0] = 0;
    for (int r = 1; r < R; ++r) start[r] = start[r - 1] + size[r - 1];
    double dmax_dist = 0.0;
    for (int r = 0; r < R; ++r)
        for (int t = 0; t < R; ++t) {
            const double d = sqrt((cx[r] - cx[t]) * (cx[r] - cx[t]) + (cy[r] - cy[t]) * (cy[r] - cy[t]) +
                                  (cz[r] - cz[t]) * (cz[r] - cz[t]));
            if (d > dmax_dist) dmax_dist = d;
        }
    double* row = (double*)malloc(sizeof(double) * R);
    for (int r = 0; r < R; ++r) {
        double s = 0.0;
        for (int t = 0; t < R; ++t) {
            uint32_t u[4];
            philox(seed, (uint32_t)r, (uint32_t)t, 0u, P_BLOCK + 16u, u);
            const double u1 = u01_open_closed(u[0]), u2 = u01_closed_open(u[1]);
            const double z = sqrt(-2.0 * log(u1)) * cos(6.283185307179586476925 * u2);
            row[t] = exp(density_sigma * z) * (double)size[t];
            s += row[t];
            const double dist = sqrt((cx[r] - cx[t]) * (cx[r] - cx[t]) + (cy[r] - cy[t]) * (cy[r] - cy[t]) +
                                     (cz[r] - cz[t]) * (cz[r] - cz[t]));
            const double dd = dmax_dist > 0 ? 1.0 + (dmax - 1) * dist / dmax_dist : 1.0;
            long q = lround(dd);
            if (q < 1) q = 1;
            if (q > dmax) q = dmax;
            pdelay[(size_t)r * R + t] = (uint8_t)q;
        }
        double acc = 0.0;
        for (int t = 0; t < R; ++t) {
            acc += row[t];
            double th = floor(acc / s * 4294967296.0);
            if (th > 4294967295.0) th = 4294967295.0;
            cum[(size_t)r * R + t] = t == R - 1 ? 0xffffffffu : (uint32_t)th;
        }
    }
    free(row);
    free(order);
    free(w);
}

void orc_gen_block(int n, int k, int R, double size_sigma, double density_sigma, int dmax, double w_mu,
                   double w_sigma, uint64_t seed, orc_csr* out)
{
    int* start = (int*)malloc(sizeof(int) * R);
    int* size = (int*)malloc(sizeof(int) * R);
    uint32_t* cum = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)R * R);
    uint8_t* pdelay = (uint8_t*)malloc((size_t)R * R);
    orc_block_tables(n, R, size_sigma, density_sigma, dmax, seed, start, size, cum, pdelay);
    out->nnz = (int64_t)n * k;
    for (int i = 0; i <= n; ++i) out->row_ptr[i] = (int64_t)i * k;
    int r_of = 0;
    for (int i = 0; i < n; ++i) {
        while (r_of + 1 < R && i >= start[r_of + 1]) ++r_of;
        for (int e = 0; e < k; ++e) {
            int tgt = (i + 1) % n, sreg = r_of;
            for (int a = 0; a < 64; ++a) {
                uint32_t u[4];
                philox(seed, (uint32_t)i, (uint32_t)e, (uint32_t)a, P_BLOCK, u);
                const uint32_t* row = cum + (size_t)r_of * R;
                int lo = 0, hi = R - 1;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (row[mid] > u[0]) hi = mid; else lo = mid + 1;
                }
                sreg = lo;
                const int off = (int)(((uint64_t)u[1] * (uint64_t)size[sreg]) >> 32);
                const int cand = start[sreg] + off;
                if (cand == i) continue;
                tgt = cand;
                break;
            }
            uint32_t rw[4];
            philox(seed, (uint32_t)i, (uint32_t)e, 0u, P_WEIGHT, rw);
            const double u1 = u01_open_closed(rw[0]), u2 = u01_closed_open(rw[1]);
            const double zz = sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
            const int64_t pos = (int64_t)i * k + e;
            out->col[pos] = tgt;
            out->weight[pos] = (float)exp(w_mu + w_sigma * zz);
            out->delay[pos] = pdelay[(size_t)r_of * R + sreg];
        }
    }
    free(start); free(size); free(cum); free(pdelay);
}

/* Local Gaussian-ball network (the library's GPU restatement of NormalNetwork,
 * src_wholebrain/network_factory.cu:95-138, with counter-based draws): cells
 * of side n_stddevs * stddev over the bounding box, members ascending, rows
 * visiting the 27 neighbouring cells (dz, dy, dx = -1..1) in order; pair
 * (i, j) accepted when d2 <= r2 (FP32, no contraction) and
 * u53(Philox(seed; i, j, 0, 10)) < exp(-d2 / (2 stddev^2)) (FP64).
 * offsets: n + 1 ints; indices: capacity ints (NULL: count only).  Returns nnz. */
int64_t orc_local_gaussian(int n, const float* x, const float* y, const float* z, float stddev, int n_stddevs,
                           uint64_t seed, int* offsets, int* indices, int64_t capacity)
{
    float lo[3] = {x[0], y[0], z[0]}, hi[3] = {x[0], y[0], z[0]};
    for (int i = 0; i < n; ++i) {
        const float v[3] = {x[i], y[i], z[i]};
        for (int a = 0; a < 3; ++a) {
            if (v[a] < lo[a]) lo[a] = v[a];
            if (v[a] > hi[a]) hi[a] = v[a];
        }
    }
    const float h = stddev * (float)n_stddevs;
    const float inv_h = 1.0f / h;
    int g[3];
    for (int a = 0; a < 3; ++a) {
        g[a] = (int)ceil((hi[a] - lo[a]) / h);
        if (g[a] < 1) g[a] = 1;
    }
    const int64_t ncells = (int64_t)g[0] * g[1] * g[2];
    int* cell = (int*)malloc(sizeof(int) * n);
    int* cc = (int*)malloc(sizeof(int) * 3 * n);
    int64_t* start = (int64_t*)calloc((size_t)ncells + 1, sizeof(int64_t));
    int* members = (int*)malloc(sizeof(int) * n);
    for (int i = 0; i < n; ++i) {
        const float p[3] = {x[i], y[i], z[i]};
        int c[3];
        for (int a = 0; a < 3; ++a) {
            int q = (int)((p[a] - lo[a]) * inv_h);
            if (q < 0) q = 0;
            if (q > g[a] - 1) q = g[a] - 1;
            c[a] = q;
            cc[3 * i + a] = q;
        }
        cell[i] = c[0] + g[0] * (c[1] + g[1] * c[2]);
        start[cell[i] + 1] += 1;
    }
    for (int64_t c = 0; c < ncells; ++c) start[c + 1] += start[c];
    int64_t* fillp = (int64_t*)malloc(sizeof(int64_t) * (size_t)ncells);
    for (int64_t c = 0; c < ncells; ++c) fillp[c] = start[c];
    for (int i = 0; i < n; ++i) members[fillp[cell[i]]++] = i;  /* ascending within a cell */
    const float r2 = h * h;
    const double inv_2var = 1.0 / (2.0 * (double)stddev * (double)stddev);
    int64_t total = 0;
    offsets[0] = 0;
    for (int i = 0; i < n; ++i) {
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int ax = cc[3 * i] + dx, ay = cc[3 * i + 1] + dy, az = cc[3 * i + 2] + dz;
                    if (ax < 0 || ay < 0 || az < 0 || ax >= g[0] || ay >= g[1] || az >= g[2]) continue;
                    const int64_t c = ax + (int64_t)g[0] * (ay + (int64_t)g[1] * az);
                    for (int64_t q = start[c]; q < start[c + 1]; ++q) {
                        const int j = members[q];
                        if (j == i) continue;
                        const float ddx = x[i] - x[j], ddy = y[i] - y[j], ddz = z[i] - z[j];
                        const float d2 = (ddx * ddx + ddy * ddy) + ddz * ddz;
                        if (!(d2 <= r2)) continue;
                        uint32_t r[4];
                        philox(seed, (uint32_t)i, (uint32_t)j, 0u, 10u, r);
                        const double u = ((double)(r[0] >> 5) * 67108864.0 + (double)(r[1] >> 6)) *
                                         (1.0 / 9007199254740992.0);
                        if (u < exp(-(double)d2 * inv_2var)) {
                            if (indices && total < capacity) indices[total] = j;
                            ++total;
                        }
                    }
                }
        offsets[i + 1] = (int)total;
    }
    free(cell); free(cc); free(start); free(members); free(fillp);
    return total;
}

int orc_sim_step(orc_sim* s, uint64_t step, int32_t* spikes)
{
    const int n = s->n, D = s->D;
    const orc_hh_params* hp = &s->hp;
    const int slot = (int)(step % (uint64_t)D);
    int ns = 0;
    /* neuron updates are independent: spikes[i] first holds a fired flag */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double* y = s->y + 6 * (int64_t)i;
        double* in = s->ring + 2 * ((int64_t)slot * n + i);
        y[4] += in[0];
        y[5] += in[1];
        in[0] = in[1] = 0.0;
        const double z = orc_normal_ctr(s->seed, (uint32_t)i, step, P_NOISE);
        const double iext = (double)s->i_drive[i] + hp->noise_sigma * z;
        const double gs = s->gna_scale ? (double)s->gna_scale[i] : 1.0;
        const double up = s->u_par ? s->u_par[i] : 0.0;
        const double v_old = y[0];
        orc_hh_rk4(hp, gs, iext, up, y);
        spikes[i] = (v_old < hp->v_thresh && y[0] >= hp->v_thresh) ? 1 : 0;
        if (spikes[i] && s->margin) {
            const double a = hp->v_thresh - v_old, b = y[0] - hp->v_thresh;
            s->margin[i] = a < b ? a : b;
        }
    }
    for (int i = 0; i < n; ++i)
        if (spikes[i]) spikes[ns++] = i;
    const orc_csr* a = s->net;
    for (int f = 0; f < ns; ++f) {
        const int j = spikes[f];
        const int ch = s->is_inh[j] ? 1 : 0;
        for (int64_t e = a->row_ptr[j]; e < a->row_ptr[j + 1]; ++e) {
            const int sl = (int)((step + a->delay[e]) % (uint64_t)D);
            s->ring[2 * ((int64_t)sl * n + a->col[e]) + ch] += (double)a->weight[e];
        }
        if (s->src) s->src[s->vox[j]] += 1.0;
    }
    return ns;
}

static inline double face_coef(const float* Dc, int64_t c, int64_t nb, int inside)
{
    if (!Dc) return 1.0;
    if (!inside) return (double)Dc[c];
    const double a = Dc[c], b = Dc[nb];
    return 2.0 * a * b / (a + b);
}

static void diag7(double* dg, int nx, int ny, int nz, double alpha, double beta, const float* Dc)
{
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int64_t c = i + (int64_t)nx * (j + (int64_t)ny * k);
                double s = 0.0;
                s += face_coef(Dc, c, c - 1, i > 0);
                s += face_coef(Dc, c, c + 1, i < nx - 1);
                s += face_coef(Dc, c, c - nx, j > 0);
                s += face_coef(Dc, c, c + nx, j < ny - 1);
                s += face_coef(Dc, c, c - (int64_t)nx * ny, k > 0);
                s += face_coef(Dc, c, c + (int64_t)nx * ny, k < nz - 1);
                dg[c] = 1.0 + beta + alpha * s;
            }
}

void orc_apply7(const double* x, double* y, int nx, int ny, int nz, double alpha, double beta, const float* Dc)
{
    const int64_t sx = 1, sy = nx, sz = (int64_t)nx * ny;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int64_t c = i + sy * j + sz * k;
                const double xc = x[c];
                double acc = (1.0 + beta) * xc;
                const int inside[6] = {i > 0, i < nx - 1, j > 0, j < ny - 1, k > 0, k < nz - 1};
                const int64_t off[6] = {-sx, sx, -sy, sy, -sz, sz};
                for (int f = 0; f < 6; ++f) {
                    const double cf = face_coef(Dc, c, c + off[f], inside[f]);
                    const double xn = inside[f] ? x[c + off[f]] : 0.0;
                    acc += alpha * cf * (xc - xn);
                }
                y[c] = acc;
            }
}

int orc_pcg7(double* x, const double* b, int nx, int ny, int nz, double alpha, double beta,
             const float* Dc, double rtol, int max_iter, double* relres)
{
    const int64_t G = (int64_t)nx * ny * nz;
    double* r = (double*)malloc(sizeof(double) * G);
    double* z = (double*)malloc(sizeof(double) * G);
    double* p = (double*)malloc(sizeof(double) * G);
    double* Ap = (double*)malloc(sizeof(double) * G);
    double* dg = (double*)malloc(sizeof(double) * G);
    diag7(dg, nx, ny, nz, alpha, beta, Dc);
    orc_apply7(x, Ap, nx, ny, nz, alpha, beta, Dc);
    for (int64_t q = 0; q < G; ++q) { r[q] = b[q] - Ap[q]; z[q] = r[q] / dg[q]; p[q] = z[q]; }
    const double bnorm = sqrt(dot(b, b, G));
    double rz = dot(r, z, G);
    double rn = sqrt(dot(r, r, G));
    int it = 0, ret = -1;
    if (bnorm == 0.0 || rn <= rtol * bnorm) {
        ret = 0;
    } else {
        for (it = 1; it <= max_iter; ++it) {
            orc_apply7(p, Ap, nx, ny, nz, alpha, beta, Dc);
            const double a = rz / dot(p, Ap, G);
#pragma omp parallel for schedule(static)
            for (int64_t q = 0; q < G; ++q) { x[q] += a * p[q]; r[q] -= a * Ap[q]; z[q] = r[q] / dg[q]; }
            rn = sqrt(dot(r, r, G));
            if (rn <= rtol * bnorm) { ret = it; break; }
            const double rz_new = dot(r, z, G);
            const double bt = rz_new / rz;
            rz = rz_new;
#pragma omp parallel for schedule(static)
            for (int64_t q = 0; q < G; ++q) p[q] = z[q] + bt * p[q];
        }
    }
    if (relres) *relres = bnorm > 0.0 ? rn / bnorm : 0.0;
    free(r); free(z); free(p); free(Ap); free(dg);
    return ret;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
