// Hodgkin-Huxley right-hand side and RK4 step in FP32 (register resident).
//
// Standard HH (-65 mV rest) with conductance synapses decaying exponentially:
//   C dV/dt = I_ext - gNa s m^3 h (V-ENa) - gK n^4 (V-EK) - gL (V-EL)
//             - ge (V-Ee) - gi (V-Ei) - g_par u (V-E_par)
//   dx/dt   = a_x(V) (1-x) - b_x(V) x,  x in {m,h,n}
//   dge/dt  = -ge/tau_e, dgi/dt = -gi/tau_i
// The external current I_ext (drive + noise) is held across the four stages.
//
// Rate functions use the fast exponential.  a_m and a_n have the removable
// singularity u/(1-e^{-u}); near u = 0 it is evaluated from its series
// 1 + u/2 + u^2/12 - u^4/720 + u^6/30240 (error < 4e-9 for |u| < 0.5),
// elsewhere as u/(1-e^{-u}) (relative error < 1e-6 for |u| >= 0.5).
#pragma once

#include "nn_internal.cuh"

struct nn_hh_dev {
    float C_inv, gNa, gK, gL, ENa, EK, EL, Ee, Ei, inv_tau_e, inv_tau_i;
    float v_thresh, noise_sigma, dt, g_par, E_par;
};

inline nn_hh_dev nn_hh_to_dev(const nn_hh_params& p)
{
    nn_hh_dev d;
    d.C_inv = 1.0f / p.C;
    d.gNa = p.gNa; d.gK = p.gK; d.gL = p.gL;
    d.ENa = p.ENa; d.EK = p.EK; d.EL = p.EL;
    d.Ee = p.E_exc; d.Ei = p.E_inh;
    d.inv_tau_e = 1.0f / p.tau_exc; d.inv_tau_i = 1.0f / p.tau_inh;
    d.v_thresh = p.v_thresh; d.noise_sigma = p.noise_sigma; d.dt = p.dt;
    d.g_par = p.g_par; d.E_par = p.E_par;
    return d;
}

__device__ __forceinline__ float nn_xexprel(float u, float emu)
{
    const float u2 = u * u;
    const float series = 1.0f + u * 0.5f + u2 * (1.0f / 12.0f + u2 * (-1.0f / 720.0f + u2 * (1.0f / 30240.0f)));
    const float direct = __fdividef(u, 1.0f - emu);
    return fabsf(u) < 0.5f ? series : direct;
}

struct nn_rates { float am, bm, ah, bh, an, bn; };

__device__ __forceinline__ nn_rates nn_hh_rates(float V)
{
    nn_rates r;
    const float um = (V + 40.0f) * 0.1f;
    const float un = (V + 55.0f) * 0.1f;  // = um + 1.5
    const float em = __expf(-um);
    r.am = nn_xexprel(um, em);
    r.an = 0.1f * nn_xexprel(un, em * 0.22313016014842982f);  // e^{-un} = e^{-um} e^{-1.5}
    const float q = __expf((V + 65.0f) * (-1.0f / 80.0f));  // e^{-(V+65)/80}
    r.bn = 0.125f * q;
    const float q2 = q * q;
    const float q4 = q2 * q2;                                 // e^{-(V+65)/20}
    r.ah = 0.07f * q4;
    const float q8 = q4 * q4;                                 // e^{-(V+65)/10}
    r.bh = __fdividef(1.0f, 1.0f + 20.085536923187668f * q8); // 1/(1+e^{-(V+35)/10})
    r.bm = 4.0f * __expf((V + 65.0f) * (-1.0f / 18.0f));
    return r;
}

struct nn_hh_state { float V, m, h, n, ge, gi; };

__device__ __forceinline__ nn_hh_state nn_hh_rhs(const nn_hh_dev& p, float gna, float iext, float gpu,
                                                 const nn_hh_state& y)
{
    const nn_rates r = nn_hh_rates(y.V);
    const float m3h = y.m * y.m * y.m * y.h;
    const float n2 = y.n * y.n;
    const float n4 = n2 * n2;
    float cur = iext;
    cur -= gna * m3h * (y.V - p.ENa);
    cur -= p.gK * n4 * (y.V - p.EK);
    cur -= p.gL * (y.V - p.EL);
    cur -= y.ge * (y.V - p.Ee);
    cur -= y.gi * (y.V - p.Ei);
    cur -= gpu * (y.V - p.E_par);
    nn_hh_state f;
    f.V = cur * p.C_inv;
    f.m = r.am - (r.am + r.bm) * y.m;
    f.h = r.ah - (r.ah + r.bh) * y.h;
    f.n = r.an - (r.an + r.bn) * y.n;
    f.ge = -y.ge * p.inv_tau_e;
    f.gi = -y.gi * p.inv_tau_i;
    return f;
}

__device__ __forceinline__ nn_hh_state nn_axpy(const nn_hh_state& y, float a, const nn_hh_state& k)
{
    return nn_hh_state{y.V + a * k.V, y.m + a * k.m, y.h + a * k.h, y.n + a * k.n, y.ge + a * k.ge, y.gi + a * k.gi};
}

// gna = gNa * (per-neuron scale); gpu = g_par * interpolated density.
__device__ __forceinline__ void nn_hh_rk4(const nn_hh_dev& p, float gna, float iext, float gpu, nn_hh_state& y)
{
    const float dt = p.dt, h2 = 0.5f * p.dt, s6 = p.dt * (1.0f / 6.0f);
    const nn_hh_state k1 = nn_hh_rhs(p, gna, iext, gpu, y);
    const nn_hh_state k2 = nn_hh_rhs(p, gna, iext, gpu, nn_axpy(y, h2, k1));
    const nn_hh_state k3 = nn_hh_rhs(p, gna, iext, gpu, nn_axpy(y, h2, k2));
    const nn_hh_state k4 = nn_hh_rhs(p, gna, iext, gpu, nn_axpy(y, dt, k3));
    y.V += s6 * (k1.V + 2.0f * (k2.V + k3.V) + k4.V);
    y.m += s6 * (k1.m + 2.0f * (k2.m + k3.m) + k4.m);
    y.h += s6 * (k1.h + 2.0f * (k2.h + k3.h) + k4.h);
    y.n += s6 * (k1.n + 2.0f * (k2.n + k3.n) + k4.n);
    y.ge += s6 * (k1.ge + 2.0f * (k2.ge + k3.ge) + k4.ge);
    y.gi += s6 * (k1.gi + 2.0f * (k2.gi + k3.gi) + k4.gi);
}

// Standard normals for the neuron pair (2k, 2k+1) at one step from the
// counter-based stream: one Philox call and one Box-Muller transform per pair
// (cos branch for the even neuron, sin branch for the odd one).
__device__ __forceinline__ void nn_normal_pair(uint64_t seed, uint32_t k, uint64_t step, float& z0, float& z1)
{
    const nn_u4 r = nn_philox(seed, k, (uint32_t)step, (uint32_t)(step >> 32), NN_P_NOISE);
    const float u1 = nn_u01f_open(r.x), u2 = nn_u01f(r.y);
    // hardware approximations (absolute error ~1e-6 in the normal deviate, far
    // below the 1e-4 parity bound): log2 and sin/cos on [-pi, pi), with
    // (cos, sin)(2 pi u2) = -(cos, sin)(2 pi u2 - pi)
    const float rad = sqrtf(fmaxf(-2.0f * __logf(u1), 0.0f));
    float s, c;
    __sincosf(6.283185307179586f * u2 - 3.141592653589793f, &s, &c);
    z0 = -rad * c;
    z1 = -rad * s;
}

__device__ __forceinline__ float nn_normal(uint64_t seed, uint32_t i, uint64_t step)
{
    float z0, z1;
    nn_normal_pair(seed, i >> 1, step, z0, z1);
    return (i & 1u) ? z1 : z0;
}
