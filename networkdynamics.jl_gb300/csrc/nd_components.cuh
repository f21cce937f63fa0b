// Device-side component library: the vertex and edge functions of the benchmark models,
// written with explicitly rounded operations (no FMA contraction) so that the FP64 results
// equal the reference's plain Julia arithmetic operation by operation.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "nd_gb300.h"

namespace nd {

template <typename T>
struct Arith;

template <>
struct Arith<double> {
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
    // FP64 keeps the raw phase difference, like the reference's sin(θs - θd).
    static __device__ __forceinline__ double sin_phase(double x) { return sin(x); }
    static __device__ __forceinline__ double cos_phase(double x) { return cos(x); }
};

// 2π split for a two-step Cody–Waite reduction of a phase difference to [-π, π].
constexpr float kTwoPiHi = 6.28318548202514648f;      // nearest float to 2π
constexpr float kTwoPiLo = -1.74845560984535e-07f;    // 2π - kTwoPiHi
constexpr float kInvTwoPi = 0.159154943091895336f;
constexpr float kPiF = 3.14159274101257324f;

template <>
struct Arith<float> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    // FP32 wraps the phase difference to [-π, π] before sin/cos so that phases that have
    // drifted far from zero do not lose the difference's digits in the argument reduction.
    static __device__ __forceinline__ float wrap(float x) {
        if (fabsf(x) > kPiF) {
            float k = rintf(x * kInvTwoPi);
            x = fmaf(-k, kTwoPiHi, x);
            x = fmaf(-k, kTwoPiLo, x);
        }
        return x;
    }
    static __device__ __forceinline__ float sin_phase(float x) { return sinf(wrap(x)); }
    static __device__ __forceinline__ float cos_phase(float x) { return cosf(wrap(x)); }
};

// Read-only load of a component parameter (a plain read for value types that are not
// float / double, such as the dual numbers of nd_dual.cuh).
template <typename T>
__device__ __forceinline__ T ldv(const T* p) {
    return __ldg(p);
}

// y_dst of the single-sided edge function g(vs, vd, p) for edge e.
template <typename T, int EK>
__device__ __forceinline__ T edge_g(T vs, T vd, const T* __restrict__ pe, int32_t e) {
    using A = Arith<T>;
    if constexpr (EK == ND_E_DIFFUSION) {
        return A::mul(__ldg(pe + e), A::sub(vs, vd));  // e .= p * (v_s[1] .- v_d[1])
    } else if constexpr (EK == ND_E_DIFFUSION_UNIT) {
        return A::sub(vs, vd);                         // e .= v_s .- v_d
    } else {
        return A::mul(__ldg(pe + e), A::sin_phase(A::sub(vs, vd)));  // e .= K .* sin(θs - θd)
    }
}

// y_dst of g(vs, vd) with the edge parameter already loaded (w is ignored by the
// parameter-free unit diffusion edge).
template <typename T, int EK>
__device__ __forceinline__ T edge_g_w(T vs, T vd, T w) {
    using A = Arith<T>;
    if constexpr (EK == ND_E_DIFFUSION) {
        return A::mul(w, A::sub(vs, vd));
    } else if constexpr (EK == ND_E_DIFFUSION_UNIT) {
        return A::sub(vs, vd);
    } else {
        return A::mul(w, A::sin_phase(A::sub(vs, vd)));
    }
}

// The incidence contribution from preloaded operands (see incidence_term).
template <typename T, int EK>
__device__ __forceinline__ T incidence_term_w(T uv, T un, T w, bool src_side) {
    const T vs = src_side ? uv : un;
    const T vd = src_side ? un : uv;
    const T y = edge_g_w<T, EK>(vs, vd, w);
    if constexpr (sizeof(T) == 8) {
        return __longlong_as_double(__double_as_longlong(y) ^ ((long long)src_side << 63));
    } else {
        return __int_as_float(__float_as_int(y) ^ ((int)src_side << 31));
    }
}

// Contribution of one incidence to the aggregation at the row vertex (value uv).  The
// AntiSymmetric wrapper evaluates g once per edge with the edge's own orientation and
// hands -y_dst to the source (src/component_functions.jl:117-127), so the source side
// negates g(uv, un) instead of evaluating g(un, uv).
template <typename T, int EK>
__device__ __forceinline__ T incidence_term(T uv, T un, const T* __restrict__ pe, int32_t eid_bits) {
    const bool src_side = eid_bits < 0;
    const int32_t e = eid_bits & 0x7fffffff;
    const T vs = src_side ? uv : un;
    const T vd = src_side ? un : uv;
    const T y = edge_g<T, EK>(vs, vd, pe, e);
    // negate by flipping the sign bit (an integer op, not an FP64 subtraction)
    if constexpr (sizeof(T) == 8) {
        return __longlong_as_double(__double_as_longlong(y) ^ ((long long)src_side << 63));
    } else {
        return __int_as_float(__float_as_int(y) ^ ((int)src_side << 31));
    }
}

template <int VK>
struct VertexDims {
    static constexpr int dim = VK == ND_V_SWING || VK == ND_V_SWING_UNIT ? 2 : 1;
    static constexpr int pdim = VK == ND_V_DIFFUSION ? 0 : (VK == ND_V_KURAMOTO || VK == ND_V_SWING_UNIT ? 1 : 3);
};

// Vertex f of the vertex whose states start at u[s] and parameters at p[q], with the
// aggregated input `acc` (the reference's aggbuf entry).
template <typename T, int VK>
__device__ __forceinline__ void vertex_f_at(T* __restrict__ du, const T* __restrict__ u, const T* __restrict__ p,
                                            int64_t s, int64_t q, T acc) {
    using A = Arith<T>;
    if constexpr (VK == ND_V_DIFFUSION) {
        du[s] = acc;  // dv[1] = acc[1]
    } else if constexpr (VK == ND_V_KURAMOTO) {
        du[s] = A::add(__ldg(p + q), acc);  // dθ[1] = ω + esum[1]
    } else if constexpr (VK == ND_V_SWING) {
        const T w = u[s + 1];
        const T M = __ldg(p + q), D = __ldg(p + q + 1), Pm = __ldg(p + q + 2);
        du[s] = w;  // dv[1] = v[2]
        // dv[2] = 1 / M * (Pm - D * v[2] + acc[1])
        du[s + 1] = A::mul(A::div(T(1), M), A::add(A::sub(Pm, A::mul(D, w)), acc));
    } else {
        const T w = u[s + 1];
        du[s] = w;  // dv[1] = v[2]
        // dv[2] = P - 1.0 * v[2]; dv[2] += esum[1]   (1.0 * v[2] is v[2] exactly)
        du[s + 1] = A::add(A::sub(__ldg(p + q), w), acc);
    }
}

// Vertex f of vertex v of a homogeneous batch.
template <typename T, int VK>
__device__ __forceinline__ void vertex_f(T* __restrict__ du, const T* __restrict__ u,
                                         const T* __restrict__ pv, int64_t v, T acc) {
    vertex_f_at<T, VK>(du, u, pv, v * VertexDims<VK>::dim, v * VertexDims<VK>::pdim, acc);
}

// ODE edge f of diffusion_dedge!: de1 = rate (sin(vs - vd) - e1), de2 = rate (sin(vd - vs) - e2)
// with rate = 1 / τ (ND_E_DIFFUSION_ODE; Julia evaluates 1 / τ * x as (1 / τ) * x) or the
// constant 100.0 (ND_E_DIFFUSION_ODE_FIXED).  vd - vs is exactly -(vs - vd) and the device
// sine is exactly odd (checked by the tests), so sin(vd - vs) is the negated sin(vs - vd):
// one sine per edge, the same bits as two.
template <typename T>
__device__ __forceinline__ void ode_edge_f(T rate, T vs, T vd, T e1, T e2, T& de1, T& de2) {
    using A = Arith<T>;
    const T s = A::sin_phase(A::sub(vs, vd));
    de1 = A::mul(rate, A::sub(s, e1));
    de2 = A::mul(rate, A::sub(-s, e2));
}

// ---- power-grid components: complex values (outputs of dimension 2) ------------------------
// Complex arithmetic as Julia defines it: the product (ac - bd, ad + bc) and division by
// the robust method of Baudin & Smith ("A Robust Complex Division in Scilab", 2012, with
// their improved r = 0 / br = 0 branches), which Julia's Base uses.  The method's range
// scaling only acts near the overflow / underflow thresholds and is left out.
template <typename T>
struct Cx {
    T r, i;
};

template <typename T>
__device__ __forceinline__ Cx<T> cmul(Cx<T> a, Cx<T> b) {
    using A = Arith<T>;
    return {A::sub(A::mul(a.r, b.r), A::mul(a.i, b.i)), A::add(A::mul(a.r, b.i), A::mul(a.i, b.r))};
}

template <typename T>
__device__ __forceinline__ T cdiv_part(T a, T b, T c, T d, T r, T t) {
    using A = Arith<T>;
    if (r != T(0)) {
        const T br = A::mul(b, r);
        return br != T(0) ? A::mul(A::add(a, br), t) : A::add(A::mul(a, t), A::mul(A::mul(b, t), r));
    }
    return A::mul(A::add(a, A::mul(d, A::div(b, c))), t);
}

template <typename T>
__device__ __forceinline__ Cx<T> cdiv(Cx<T> x, Cx<T> y) {
    using A = Arith<T>;
    T a = x.r, b = x.i, c = y.r, d = y.i;
    const bool swap = !(fabs(d) <= fabs(c));
    if (swap) {
        T t0 = a;
        a = b;
        b = t0;
        t0 = c;
        c = d;
        d = t0;
    }
    const T r = A::div(d, c);
    const T t = A::div(T(1), A::add(c, A::mul(d, r)));
    const T p = cdiv_part<T>(a, b, c, d, r, t);
    const T q = cdiv_part<T>(b, -a, c, d, r, t);
    return {p, swap ? -q : q};
}

// 2π·50 as Julia evaluates 2π*50 in Float64
constexpr double kPiLineOmega = 314.1592653589793;

// piline! (benchmark/benchmark_models.jl:46-63): currents out of a π-line with series
// impedance R + iωL and shunt capacitances C1, C2, from the complex source / destination
// voltages.  Outputs y_src = -isrc, y_dst = -idst.
template <typename T>
__device__ __forceinline__ void piline_g(Cx<T> vs, Cx<T> vd, T L, T R, T C1, T C2, Cx<T>& ysrc, Cx<T>& ydst) {
    using A = Arith<T>;
    const T w = T(kPiLineOmega);
    const Cx<T> imain = cdiv<T>({A::sub(vs.r, vd.r), A::sub(vs.i, vd.i)}, {R, A::mul(w, L)});  // R + im*ω*L
    const Cx<T> ic1 = {A::mul(A::mul(-vs.i, w), C1), A::mul(A::mul(vs.r, w), C1)};        // Vsrc*im*ω*C1
    const Cx<T> ic2 = {A::mul(A::mul(-vd.i, w), C2), A::mul(A::mul(vd.r, w), C2)};
    // isrc = -(imain + iC1), idst = imain - iC2; the outputs are their negatives
    ysrc = {A::add(imain.r, ic1.r), A::add(imain.i, ic1.i)};
    ydst = {-A::sub(imain.r, ic2.r), -A::sub(imain.i, ic2.i)};
}

// Vertex f of the power-grid vertices with the aggregated complex current `in`.
//   pq!   (benchmark_models.jl:65-73)  algebraic bus: du = S / conj(i), S = P + iQ
//   gen!  (benchmark_models.jl:76-109) 4-state generator (u_r, u_i, θ, ω)
template <typename T, int VK>
__device__ __forceinline__ void vertex_f2_at(T* __restrict__ du, const T* __restrict__ u, const T* __restrict__ p,
                                             int64_t s, int64_t q, Cx<T> in) {
    using A = Arith<T>;
    if constexpr (VK == ND_V_PQ) {
        const Cx<T> uc = cdiv<T>({ldv(p + q), ldv(p + q + 1)}, {in.r, -in.i});
        du[s] = uc.r;
        du[s + 1] = uc.i;
    } else {
        const T H = ldv(p + q), P = ldv(p + q + 1), D = ldv(p + q + 2), Om = ldv(p + q + 3);
        const T E_f = ldv(p + q + 4), T_d_dash = ldv(p + q + 5), T_q_dash = ldv(p + q + 6);
        const T X_q_dash = ldv(p + q + 7), X_d_dash = ldv(p + q + 8), X_d = ldv(p + q + 9);
        const T X_q = ldv(p + q + 10);
        const T Om_H = A::div(Om, A::mul(T(2), H));
        const Cx<T> uc = {u[s], u[s + 1]};
        const T th = u[s + 2], w = u[s + 3];
        const T ct = A::cos_phase(th), st = A::sin_phase(th);
        const Cx<T> em = {ct, -st};                        // exp(-im*θ) = (cos θ, -sin θ)
        const Cx<T> i_c = cmul<T>({-in.i, in.r}, em);     // (im*i)*exp(-im*θ)
        const Cx<T> e_c = cmul<T>({-uc.i, uc.r}, em);     // (im*u)*exp(-im*θ)
        const T pw = cmul<T>(uc, {in.r, -in.i}).r;        // real(u*conj(i))
        const T de_d = A::mul(A::div(T(1), T_q_dash), A::add(-e_c.r, A::mul(A::sub(X_q, X_q_dash), i_c.i)));
        const T de_q = A::mul(A::div(T(1), T_d_dash),
                              A::add(A::sub(-e_c.i, A::mul(A::sub(X_d, X_d_dash), i_c.r)), E_f));
        const Cx<T> t1 = cmul<T>({de_q, -de_d}, {ct, st}); // (-im*de_c)*exp(im*θ)
        du[s] = A::add(t1.r, A::mul(-uc.i, w));            // + (u*im)*ω
        du[s + 1] = A::add(t1.i, A::mul(uc.r, w));
        du[s + 2] = w;
        du[s + 3] = A::mul(A::sub(A::sub(A::sub(P, A::mul(D, w)), pw),
                                  A::mul(A::mul(A::sub(X_q_dash, X_d_dash), i_c.r), i_c.i)),
                           Om_H);
    }
}

}  // namespace nd
