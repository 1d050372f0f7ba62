// Hodgkin-Huxley right-hand side and RK4 step in FP32 (register resident).
//
// Standard HH (-65 mV rest) with conductance synapses decaying exponentially:
//   C dV/dt = I_ext - gNa s m^3 h (V-ENa) - gK n^4 (V-EK) - gL (V-EL)
//             - ge (V-Ee) - gi (V-Ei) - g_par u (V-E_par)
//   dx/dt   = a_x(V) (1-x) - b_x(V) x,  x in {m,h,n}
//   dge/dt  = -ge/tau_e, dgi/dt = -gi/tau_i
// The external current I_ext (drive + noise) is held across the four stages.
//
// Rate functions use the hardware 2^x and 1/x.  a_m and a_n have the
// removable singularity u/(1-e^{-u}); near u = 0 it is evaluated from its
// series 1 + u/2 + u^2/12 - u^4/720 + u^6/30240 (error < 4e-9 for
// |u| < 0.5), elsewhere as u/(1-e^{-u}) (relative error < 1e-6 for
// |u| >= 0.5).
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

// ---- lane vectors ----
// W neurons computed together.  With W = 2 every add, subtract, multiply and
// fused multiply-add is one packed two-lane FP32 instruction (PTX .f32x2,
// sm_100 family); with W = 1 the same operations run one lane at a time.
// Each operation is explicitly rounded and the packed instructions round each
// lane as the scalar ones do.  The assembler may still fuse a packed multiply
// whose result feeds a packed add into one fused multiply-add, depending on
// the surrounding code; so no product below feeds a sum directly (sums of
// products are written as explicit fused multiply-adds, and constant factors
// are folded into the coefficients that use them).  The two forms then give
// bit-identical results.  Exponentials and reciprocals stay per lane.
template <int W>
struct nn_vf {
    float v[W];
};

template <int W>
__device__ __forceinline__ nn_vf<W> vb(float x)  // broadcast
{
    nn_vf<W> r;
#pragma unroll
    for (int l = 0; l < W; ++l) r.v[l] = x;
    return r;
}

#define NN_F32X2(op, ins)                                                                                  \
    __device__ __forceinline__ nn_vf<2> op(const nn_vf<2>& a, const nn_vf<2>& b)                          \
    {                                                                                                      \
        nn_vf<2> d;                                                                                        \
        asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t" ins         \
            " rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"                                                   \
            : "=f"(d.v[0]), "=f"(d.v[1])                                                                   \
            : "f"(a.v[0]), "f"(a.v[1]), "f"(b.v[0]), "f"(b.v[1]));                                          \
        return d;                                                                                          \
    }
NN_F32X2(vadd, "add.rn.f32x2")
NN_F32X2(vsub, "sub.rn.f32x2")
NN_F32X2(vmul, "mul.rn.f32x2")
#undef NN_F32X2

__device__ __forceinline__ nn_vf<2> vfma(const nn_vf<2>& a, const nn_vf<2>& b, const nn_vf<2>& c)  // a*b + c
{
    nn_vf<2> d;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
        "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.v[0]), "=f"(d.v[1])
        : "f"(a.v[0]), "f"(a.v[1]), "f"(b.v[0]), "f"(b.v[1]), "f"(c.v[0]), "f"(c.v[1]));
    return d;
}

__device__ __forceinline__ nn_vf<1> vadd(const nn_vf<1>& a, const nn_vf<1>& b) { return {{__fadd_rn(a.v[0], b.v[0])}}; }
__device__ __forceinline__ nn_vf<1> vsub(const nn_vf<1>& a, const nn_vf<1>& b) { return {{__fsub_rn(a.v[0], b.v[0])}}; }
__device__ __forceinline__ nn_vf<1> vmul(const nn_vf<1>& a, const nn_vf<1>& b) { return {{__fmul_rn(a.v[0], b.v[0])}}; }
__device__ __forceinline__ nn_vf<1> vfma(const nn_vf<1>& a, const nn_vf<1>& b, const nn_vf<1>& c)
{
    return {{__fmaf_rn(a.v[0], b.v[0], c.v[0])}};
}

// Per-lane hardware approximations: 2^x and 1/x (ex2.approx.ftz,
// rcp.approx.ftz: relative error ~2^-22).
__device__ __forceinline__ float nn_ex2(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float nn_rcp(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

template <int W>
__device__ __forceinline__ nn_vf<W> vex2(const nn_vf<W>& x)
{
    nn_vf<W> r;
#pragma unroll
    for (int l = 0; l < W; ++l) r.v[l] = nn_ex2(x.v[l]);
    return r;
}

template <int W>
__device__ __forceinline__ nn_vf<W> vrcp(const nn_vf<W>& x)
{
    nn_vf<W> r;
#pragma unroll
    for (int l = 0; l < W; ++l) r.v[l] = nn_rcp(x.v[l]);
    return r;
}

// u / (1 - e^{-u}) given den = 1 - e^{-u}: u / den, except for |u| < 0.5,
// where 1 - e^{-u} cancels and the series
// 1 + u/2 + u^2/12 - u^4/720 + u^6/30240 (error < 4e-9) is used.  Both forms
// are computed and selected per lane (a warp-uniform branch around the series
// was measured slower: 19.6 vs 18.1 us per 1M-neuron step).
template <int W>
__device__ __forceinline__ nn_vf<W> nn_xexprel(const nn_vf<W>& u, const nn_vf<W>& den)
{
    nn_vf<W> r = vmul(u, vrcp(den));
    const nn_vf<W> u2 = vmul(u, u);
    // series = 1 + u (1/2 + u (1/12 + u^2 (-1/720 + u^2 / 30240)))
    nn_vf<W> t = vfma(u2, vfma(u2, vb<W>(1.0f / 30240.0f), vb<W>(-1.0f / 720.0f)), vb<W>(1.0f / 12.0f));
    t = vfma(u, t, vb<W>(0.5f));
    const nn_vf<W> series = vfma(u, t, vb<W>(1.0f));
#pragma unroll
    for (int l = 0; l < W; ++l)
        if (fabsf(u.v[l]) < 0.5f) r.v[l] = series.v[l];
    return r;
}

// Opening rates a_x and the totals s_x = a_x + b_x.
template <int W>
struct nn_rates {
    nn_vf<W> am, sm, ah, sh, an, sn;
};

constexpr float NN_LOG2E = 1.4426950408889634f;

// The three exponentials come from ex2 of arguments formed directly in log2
// units (one fused multiply-add of V each); e^{-u_n} = e^{-u_m} e^{-1.5}, and
// the h rates use powers of e^{-(V+65)/80}.
template <int W>
__device__ __forceinline__ nn_rates<W> nn_hh_rates(const nn_vf<W>& V)
{
    nn_rates<W> r;
    const nn_vf<W> um = vfma(V, vb<W>(0.1f), vb<W>(4.0f));  // (V + 40) / 10
    const nn_vf<W> un = vadd(um, vb<W>(1.5f));              // (V + 55) / 10
    const nn_vf<W> em = vex2(vmul(um, vb<W>(-NN_LOG2E)));                                           // e^{-um}
    const nn_vf<W> q = vex2(vfma(V, vb<W>(-NN_LOG2E / 80.0f), vb<W>(-65.0f * NN_LOG2E / 80.0f)));   // e^{-(V+65)/80}
    const nn_vf<W> eb = vex2(vfma(V, vb<W>(-NN_LOG2E / 18.0f), vb<W>(-65.0f * NN_LOG2E / 18.0f)));  // e^{-(V+65)/18}
    r.am = nn_xexprel(um, vsub(vb<W>(1.0f), em));
    const nn_vf<W> xn = nn_xexprel(un, vfma(vb<W>(-0.22313016014842982f), em, vb<W>(1.0f)));  // e^{-un} = e^{-um} e^{-1.5}
    r.an = vmul(vb<W>(0.1f), xn);
    r.sn = vfma(vb<W>(0.125f), q, r.an);                // + b_n = 0.125 e^{-(V+65)/80}
    const nn_vf<W> q2 = vmul(q, q);
    const nn_vf<W> q4 = vmul(q2, q2);                   // e^{-(V+65)/20}
    r.ah = vmul(vb<W>(0.07f), q4);
    const nn_vf<W> q8 = vmul(q4, q4);                   // e^{-(V+65)/10}
    const nn_vf<W> bh = vrcp(vfma(vb<W>(20.085536923187668f), q8, vb<W>(1.0f)));  // 1 / (1 + e^{-(V+35)/10})
    r.sh = vfma(vb<W>(0.07f), q4, bh);
    r.sm = vfma(vb<W>(4.0f), eb, r.am);                 // + b_m = 4 e^{-(V+65)/18}
    return r;
}

template <int W>
struct nn_hh_state {
    nn_vf<W> V, m, h, n, ge, gi;
};

// Terms of the right-hand side that do not change within a step: the
// current is written as
//   I = base + gv V + m^3 h (na_v V + na_0) + n^4 (-gK V + gK EK)
//       + ge (Ee - V) + gi (Ei - V)
// with base = I_ext + gL EL + g_par u E_par, gv = -gL - g_par u,
// na_v = -gNa s, na_0 = gNa s ENa (s the per-neuron gNa scale, u the
// paracrine density at the neuron).  nn_hh_drive holds them per neuron;
// nn_hh_drive_uniform is the common case s = 1 and g_par u = 0, where only
// base varies between neurons and the rest are launch constants.
template <int W>
struct nn_hh_drive {
    nn_vf<W> base, gv_, na_v_, na_0_;
    __device__ __forceinline__ nn_vf<W> gv() const { return gv_; }
    __device__ __forceinline__ nn_vf<W> na_v() const { return na_v_; }
    __device__ __forceinline__ nn_vf<W> na_0() const { return na_0_; }
};

template <int W>
struct nn_hh_drive_uniform {
    nn_vf<W> base;
    float gv_, na_v_, na_0_;
    __device__ __forceinline__ nn_vf<W> gv() const { return vb<W>(gv_); }
    __device__ __forceinline__ nn_vf<W> na_v() const { return vb<W>(na_v_); }
    __device__ __forceinline__ nn_vf<W> na_0() const { return vb<W>(na_0_); }
};

// ngna = -gNa * (per-neuron scale), ngpu = -g_par * density
template <int W>
__device__ __forceinline__ nn_hh_drive<W> nn_hh_make_drive(const nn_hh_dev& p, const nn_vf<W>& ngna,
                                                           const nn_vf<W>& iext, const nn_vf<W>& ngpu)
{
    nn_hh_drive<W> d;
    // base = iext + gL EL - ngpu E_par, gv = ngpu - gL
    d.base = vfma(ngpu, vb<W>(-p.E_par), vadd(iext, vb<W>(p.gL * p.EL)));
    d.gv_ = vsub(ngpu, vb<W>(p.gL));
    d.na_v_ = ngna;
    d.na_0_ = vmul(ngna, vb<W>(-p.ENa));
    return d;
}

template <int W>
__device__ __forceinline__ nn_hh_drive_uniform<W> nn_hh_make_drive_uniform(const nn_hh_dev& p, const nn_vf<W>& iext)
{
    nn_hh_drive_uniform<W> d;
    d.base = vadd(iext, vb<W>(p.gL * p.EL));
    d.gv_ = -p.gL;
    d.na_v_ = -p.gNa;
    d.na_0_ = p.gNa * p.ENa;
    return d;
}

// Right-hand side with two factors left out: the V component is the total
// current (dV/dt = current / C) and the g_e, g_i components are the
// conductances themselves (dg/dt = -g / tau); the RK4 coefficients below
// carry 1/C and -1/tau.
template <int W, class Drive>
__device__ __forceinline__ nn_hh_state<W> nn_hh_rhs(const nn_hh_dev& p, const Drive& d, const nn_hh_state<W>& y)
{
    const nn_rates<W> r = nn_hh_rates(y.V);
    const nn_vf<W> m3h = vmul(vmul(vmul(y.m, y.m), y.m), y.h);
    const nn_vf<W> n2 = vmul(y.n, y.n);
    const nn_vf<W> n4 = vmul(n2, n2);
    nn_vf<W> cur = vfma(d.gv(), y.V, d.base);
    cur = vfma(m3h, vfma(d.na_v(), y.V, d.na_0()), cur);
    cur = vfma(n4, vfma(vb<W>(-p.gK), y.V, vb<W>(p.gK * p.EK)), cur);
    cur = vfma(y.ge, vsub(vb<W>(p.Ee), y.V), cur);
    cur = vfma(y.gi, vsub(vb<W>(p.Ei), y.V), cur);
    nn_hh_state<W> f;
    f.V = cur;
    f.m = vfma(vmul(vb<W>(-1.0f), r.sm), y.m, r.am);
    f.h = vfma(vmul(vb<W>(-1.0f), r.sh), y.h, r.ah);
    f.n = vfma(vmul(vb<W>(-1.0f), r.sn), y.n, r.an);
    f.ge = y.ge;
    f.gi = y.gi;
    return f;
}

// Per-component factors of the right-hand side (1/C for V, 1 for the gates,
// -1/tau for the conductances) times a step length.
struct nn_hh_coef {
    float V, x, ge, gi;
};

__device__ __forceinline__ nn_hh_coef nn_hh_scaled(const nn_hh_dev& p, float h)
{
    return nn_hh_coef{h * p.C_inv, h, -h * p.inv_tau_e, -h * p.inv_tau_i};
}

template <int W>
__device__ __forceinline__ nn_hh_state<W> nn_axpy(const nn_hh_state<W>& y, const nn_hh_coef& c, const nn_hh_state<W>& k)
{
    return nn_hh_state<W>{vfma(k.V, vb<W>(c.V), y.V), vfma(k.m, vb<W>(c.x), y.m), vfma(k.h, vb<W>(c.x), y.h),
                          vfma(k.n, vb<W>(c.x), y.n), vfma(k.ge, vb<W>(c.ge), y.ge), vfma(k.gi, vb<W>(c.gi), y.gi)};
}

// y + c (k1 + 2 (k2 + k3) + k4)
template <int W>
__device__ __forceinline__ nn_vf<W> nn_rk4_comb(const nn_vf<W>& y, float c, const nn_vf<W>& k1, const nn_vf<W>& k2,
                                                const nn_vf<W>& k3, const nn_vf<W>& k4)
{
    const nn_vf<W> t = vadd(vfma(vadd(k2, k3), vb<W>(2.0f), k1), k4);
    return vfma(t, vb<W>(c), y);
}

// One RK4 step of W neurons (external current held over the stages), given
// the step's constant terms (nn_hh_make_drive / nn_hh_make_drive_uniform).
template <int W, class Drive>
__device__ __forceinline__ void nn_hh_rk4(const nn_hh_dev& p, const Drive& d, nn_hh_state<W>& y)
{
    const nn_hh_coef c2 = nn_hh_scaled(p, 0.5f * p.dt), c4 = nn_hh_scaled(p, p.dt);
    const nn_hh_coef c6 = nn_hh_scaled(p, p.dt * (1.0f / 6.0f));
    const nn_hh_state<W> k1 = nn_hh_rhs<W>(p, d, y);
    const nn_hh_state<W> k2 = nn_hh_rhs<W>(p, d, nn_axpy(y, c2, k1));
    const nn_hh_state<W> k3 = nn_hh_rhs<W>(p, d, nn_axpy(y, c2, k2));
    const nn_hh_state<W> k4 = nn_hh_rhs<W>(p, d, nn_axpy(y, c4, k3));
    y.V = nn_rk4_comb(y.V, c6.V, k1.V, k2.V, k3.V, k4.V);
    y.m = nn_rk4_comb(y.m, c6.x, k1.m, k2.m, k3.m, k4.m);
    y.h = nn_rk4_comb(y.h, c6.x, k1.h, k2.h, k3.h, k4.h);
    y.n = nn_rk4_comb(y.n, c6.x, k1.n, k2.n, k3.n, k4.n);
    y.ge = nn_rk4_comb(y.ge, c6.ge, k1.ge, k2.ge, k3.ge, k4.ge);
    y.gi = nn_rk4_comb(y.gi, c6.gi, k1.gi, k2.gi, k3.gi, k4.gi);
}

// Standard normals for the neuron pair (2k, 2k+1) at one step from the
// counter-based stream: one Philox2x32-10 draw (counter (k, low step word),
// key nn_noise_key) and one Box-Muller transform per pair (cos branch for the
// even neuron, sin branch for the odd one).
__device__ __forceinline__ void nn_normal_pair(uint64_t seed, uint32_t k, uint64_t step, float& z0, float& z1)
{
    uint32_t r0, r1;
    nn_philox2(nn_noise_key(seed, step), k, (uint32_t)step, r0, r1);
    const float u1 = nn_u01f_open(r0), u2 = nn_u01f(r1);
    // hardware approximations (absolute error ~1e-6 in the normal deviate, far
    // below the 1e-4 parity bound): log2 and sin/cos on [-pi, pi), with
    // (cos, sin)(2 pi u2) = -(cos, sin)(2 pi u2 - pi)
    const float r2 = fmaxf(-2.0f * __logf(u1), 1e-30f);
    const float rad = r2 * rsqrtf(r2);
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
