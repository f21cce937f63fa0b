// Batched ensembles of networks: many instances of one component pair on different
// graphs, packed one after another, each in the reference's flat layout.
//
//   nd_ensemble_rhs           du of every instance (the same sums as nd_rhs)
//   nd_ensemble_solve_tsit5   every instance integrated with its own adaptive Tsit5 steps
//                             by one persistent kernel, replayed from a CUDA graph
//   nd_ensemble_fixpoint      steady states of swing ensembles by Newton's method, each
//                             linear system solved by conjugate gradients on the analytic
//                             Jacobian (weighted graph Laplacian)
//
// A block owns one instance at a time and takes the next from a work queue (instances
// sorted by size, largest first).  Instance state lives in global scratch sized for the
// whole ensemble; every loop is bounded (step, Newton and CG budgets) and a failing
// instance reports its status instead of stalling the kernel.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <type_traits>
#include <vector>

#include "nd_components.cuh"
#include "nd_df.cuh"
#include "nd_internal.h"

struct nd_ensemble {
    int dtype = ND_F64;
    int vertex_kind = 0, edge_kind = 0;
    int device = 0;
    int64_t n_inst = 0, nv = 0, ne = 0, dim = 0, pdim = 0;
    int max_rows = 0;  // largest instance, vertices
    // device arrays
    int64_t* v0 = nullptr;    // [n+1] first packed vertex of each instance
    int64_t* e0 = nullptr;    // [n+1] first packed edge
    int32_t* order = nullptr; // [n] instances by size, descending
    uint32_t* row_ptr = nullptr;  // [nv+1] incidences of each packed vertex
    int32_t* incid_nbr = nullptr; // [2ne] local neighbour index
    int32_t* incid_eid = nullptr; // [2ne] local edge index | src-side bit
    int* counter = nullptr;       // work queue
    // scratch for the integrator / Newton
    double* work = nullptr;  // Tsit5: 8 vectors of dim; Newton: 5 vectors of nv + incidence weights
    size_t work_bytes = 0;
    int tuned_threads = 0;
};

namespace nd {

namespace {

constexpr unsigned kFullMask = 0xffffffffu;

__constant__ double e_a[7][6];
__constant__ double e_bt[7];
const double eh_a[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {0.161, 0, 0, 0, 0, 0},
    {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0},
    {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0},
    {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0},
    {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0},
    {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774}};
const double eh_bt[7] = {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
                         -0.1447110071732629,     0.5823571654525552,     -0.45808210592918697,
                         0.015151515151515152};
bool g_etab[64] = {};

cudaError_t upload_tableau() {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!g_etab[dev]) {
        cudaError_t err = cudaMemcpyToSymbol(e_a, eh_a, sizeof eh_a);
        if (err == cudaSuccess) err = cudaMemcpyToSymbol(e_bt, eh_bt, sizeof eh_bt);
        if (err != cudaSuccess) return err;
        g_etab[dev] = true;
    }
    return cudaSuccess;
}

struct EnsArgs {
    int64_t n_inst;
    const int64_t* v0;
    const int64_t* e0;
    const int32_t* order;
    const uint32_t* row_ptr;
    const int32_t* nbr;
    const int32_t* eid;
    int* counter;
};

// Tag of the double-float RHS (ND_F32X2): FP64 state and parameters, arithmetic in pairs
// of floats on the FP32 pipe (nd_df.cuh).
struct F32x2 {};
template <typename T>
struct Elem {
    using type = T;  // element type of p and of the RHS's caller buffers
};
template <>
struct Elem<F32x2> {
    using type = double;
};

// Instance views.
struct Inst {
    int64_t vbase, nvi, ebase, nei;  // packed vertex / edge ranges
    int64_t ubase, pbase;            // offsets of its u and p in the packed vectors
};

template <int VK, int EK>
__device__ __forceinline__ Inst instance(const EnsArgs& a, int64_t i) {
    Inst s;
    s.vbase = a.v0[i];
    s.nvi = a.v0[i + 1] - s.vbase;
    s.ebase = a.e0[i];
    s.nei = a.e0[i + 1] - s.ebase;
    s.ubase = s.vbase * VertexDims<VK>::dim;
    s.pbase = s.vbase * VertexDims<VK>::pdim + s.ebase * (EK == ND_E_DIFFUSION_UNIT ? 0 : 1);
    return s;
}

// du = f(y) for one instance, one vertex per thread, sequential order (bitwise equal to
// nd_rhs).  The state is read in FP64 and computed in T (the RHS precision).
template <typename T, int VK, int EK, typename TU>
__device__ void instance_rhs(const EnsArgs& a, const Inst& s, const TU* __restrict__ y, const T* __restrict__ p,
                             double* __restrict__ du_d, T* __restrict__ du_t) {
    using A = Arith<T>;
    constexpr int DV = VertexDims<VK>::dim;
    const T* pv = p + s.pbase;
    const T* pe = pv + s.nvi * VertexDims<VK>::pdim;
    const TU* yi = y + s.ubase;
    for (int64_t v = threadIdx.x; v < s.nvi; v += blockDim.x) {
        const uint32_t beg = a.row_ptr[s.vbase + v], end = a.row_ptr[s.vbase + v + 1];
        const T uv = (T)yi[v * DV];
        T acc = T(0);
        if constexpr (sizeof(T) < sizeof(TU)) {
            // FP32 RHS on the FP64 state: the difference u_n - u_v is taken in the state's
            // precision and rounded once, so phases that have wound far from zero keep
            // their full resolution before the FP32 wrap and sine.  Both sides of an
            // AntiSymmetric edge then contribute g applied to that difference.
            const TU uvd = yi[v * DV];
            for (uint32_t k = beg; k < end; ++k) {
                const int32_t nb = a.nbr[k], ebits = a.eid[k];
                const T d = (T)(yi[(int64_t)nb * DV] - uvd);
                const int32_t e = ebits & 0x7fffffff;
                T term;
                if constexpr (EK == ND_E_DIFFUSION) term = A::mul(pe[e], d);
                else if constexpr (EK == ND_E_DIFFUSION_UNIT) term = d;
                else term = A::mul(pe[e], A::sin_phase(d));
                acc = A::add(acc, term);
            }
        } else {
            for (uint32_t k = beg; k < end; ++k) {
                const int32_t nb = a.nbr[k], ebits = a.eid[k];
                acc = A::add(acc, incidence_term<T, EK>(uv, (T)yi[(int64_t)nb * DV], pe, ebits));
            }
        }
        // vertex f into a local buffer of the instance's dim
        T out[DV];
        T uloc[DV];
#pragma unroll
        for (int d = 0; d < DV; ++d) uloc[d] = (T)yi[v * DV + d];
        if constexpr (VK == ND_V_DIFFUSION) {
            out[0] = acc;
        } else if constexpr (VK == ND_V_KURAMOTO) {
            out[0] = A::add(pv[v], acc);
        } else {
            const T M = pv[3 * v], D = pv[3 * v + 1], Pm = pv[3 * v + 2];
            out[0] = uloc[1];
            out[1] = A::mul(A::div(T(1), M), A::add(A::sub(Pm, A::mul(D, uloc[1])), acc));
        }
#pragma unroll
        for (int d = 0; d < DV; ++d) {
            if (du_d) du_d[s.ubase + v * DV + d] = (double)out[d];
            if (du_t) du_t[s.ubase + v * DV + d] = out[d];
        }
    }
}

// The same RHS in double-float: each incidence's phase difference is taken in FP64 (one
// subtraction, exact up to the state's rounding) and split into floats; the sine, the
// products, the row sum and the vertex function run in double-float; du is rounded to FP64.
// Errors stay near 1e-14 relative where the FP32 RHS has ~1e-7.
template <int VK, int EK>
__device__ void instance_rhs_df(const EnsArgs& a, const Inst& s, const double* __restrict__ y,
                                const double* __restrict__ p, double* __restrict__ du_d) {
    using namespace df;
    constexpr int DV = VertexDims<VK>::dim;
    const double* pv = p + s.pbase;
    const double* pe = pv + s.nvi * VertexDims<VK>::pdim;
    const double* yi = y + s.ubase;
    for (int64_t v = threadIdx.x; v < s.nvi; v += blockDim.x) {
        const uint32_t beg = a.row_ptr[s.vbase + v], end = a.row_ptr[s.vbase + v + 1];
        const double uvd = yi[v * DV];
        Df acc{0.f, 0.f};
        for (uint32_t k = beg; k < end; ++k) {
            const int32_t nb = a.nbr[k], e = a.eid[k] & 0x7fffffff;
            const double dd = __dsub_rn(yi[(int64_t)nb * DV], uvd);
            Df term;
            if constexpr (EK == ND_E_DIFFUSION) term = mul(from_double(pe[e]), from_double(dd));
            else if constexpr (EK == ND_E_DIFFUSION_UNIT) term = from_double(dd);
            else term = mul(from_double(pe[e]), df::sin(from_double3(dd)));
            acc = add(acc, term);
        }
        double* out = du_d + s.ubase + v * DV;
        if constexpr (VK == ND_V_DIFFUSION) {
            out[0] = to_double(acc);
        } else if constexpr (VK == ND_V_KURAMOTO) {
            out[0] = to_double(add(from_double(pv[v]), acc));
        } else {
            // dv[2] = 1 / M * (Pm - D * v[2] + acc)
            const double w = yi[v * DV + 1];
            const Df inv = df::div(Df{1.f, 0.f}, from_double(pv[3 * v]));
            const Df t = add(sub(from_double(pv[3 * v + 2]), mul(from_double(pv[3 * v + 1]), from_double(w))), acc);
            out[0] = w;
            out[1] = to_double(mul(inv, t));
        }
    }
}

template <typename T, int VK, int EK>
__device__ __forceinline__ void any_instance_rhs(const EnsArgs& a, const Inst& s, const double* __restrict__ y,
                                                 const typename Elem<T>::type* __restrict__ p, double* __restrict__ du) {
    if constexpr (std::is_same<T, F32x2>::value) instance_rhs_df<VK, EK>(a, s, y, p, du);
    else instance_rhs<T, VK, EK, double>(a, s, y, p, du, nullptr);
}

template <typename T, int VK, int EK>
__global__ void ens_rhs_kernel(EnsArgs a, const typename Elem<T>::type* __restrict__ u,
                               const typename Elem<T>::type* __restrict__ p, typename Elem<T>::type* __restrict__ du) {
    for (int64_t i = blockIdx.x; i < a.n_inst; i += gridDim.x) {
        const Inst s = instance<VK, EK>(a, i);
        if constexpr (std::is_same<T, F32x2>::value) instance_rhs_df<VK, EK>(a, s, u, p, du);
        else instance_rhs<T, VK, EK, T>(a, s, u, p, nullptr, du);
    }
}

__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(kFullMask, v, off);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    double t = 0.0;
    for (int k = 0; k < nw; ++k) t += red[k];  // fixed order: deterministic
    return t;
}

__device__ __forceinline__ int take_instance(const EnsArgs& a, int* sh) {
    __syncthreads();
    if (threadIdx.x == 0) *sh = atomicAdd(a.counter, 1);
    __syncthreads();
    return *sh;
}

// ---- batched Tsit5 ----------------------------------------------------------------------
struct SolveParams {
    double t0, t1, reltol, abstol;
    int64_t max_steps;
    int64_t dim;  // packed dim (stride of the stage vectors)
    // per instance (t, dt, qold) written at the end of the solve (NULL: none); with resume,
    // read at the start instead of the initial-step heuristic
    double* control;
    int resume;
};

template <typename T, int VK, int EK>
__global__ void ens_tsit5_kernel(EnsArgs a, SolveParams sp, double* __restrict__ U,
                                 const typename Elem<T>::type* __restrict__ p,
                                 double* __restrict__ work, int32_t* __restrict__ status, int64_t* __restrict__ nsteps) {
    __shared__ double red[32];
    __shared__ int sh_inst;
    __shared__ double sh_dt, sh_t, sh_qold;
    __shared__ int sh_accept, sh_done, sh_status;
    __shared__ long long sh_steps;
    double* K[7];
#pragma unroll
    for (int j = 0; j < 7; ++j) K[j] = work + (size_t)j * sp.dim;
    double* Y = work + (size_t)7 * sp.dim;
    for (;;) {
        const int q = take_instance(a, &sh_inst);
        if (q >= a.n_inst) break;
        const int64_t i = a.order[q];
        const Inst s = instance<VK, EK>(a, i);
        const int64_t n = s.nvi * VertexDims<VK>::dim;
        double* u = U + s.ubase;
        // k0 = f(u); initial step (Hairer & Wanner)
        any_instance_rhs<T, VK, EK>(a, s, U, p, K[0]);
        __syncthreads();
        double d0 = 0, d1 = 0;
        for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
            const double sc = sp.abstol + fabs(u[j]) * sp.reltol;
            d0 += (u[j] / sc) * (u[j] / sc);
            d1 += (K[0][s.ubase + j] / sc) * (K[0][s.ubase + j] / sc);
        }
        d0 = sqrt(block_sum(d0, red) / (double)(n ? n : 1));
        __syncthreads();
        d1 = sqrt(block_sum(d1, red) / (double)(n ? n : 1));
        double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
        h0 = fmin(h0, sp.t1 - sp.t0);
        for (int64_t j = threadIdx.x; j < n; j += blockDim.x) Y[s.ubase + j] = u[j] + h0 * K[0][s.ubase + j];
        __syncthreads();
        any_instance_rhs<T, VK, EK>(a, s, Y, p, K[1]);
        __syncthreads();
        double d2 = 0;
        for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
            const double sc = sp.abstol + fabs(u[j]) * sp.reltol;
            const double r = (K[1][s.ubase + j] - K[0][s.ubase + j]) / sc;
            d2 += r * r;
        }
        __syncthreads();
        d2 = sqrt(block_sum(d2, red) / (double)(n ? n : 1)) / h0;
        if (threadIdx.x == 0) {
            const double h1 = (fmax(d1, d2) <= 1e-15) ? fmax(1e-6, h0 * 1e-3) : pow(0.01 / fmax(d1, d2), 1.0 / 5.0);
            sh_dt = fmin(fmin(100 * h0, h1), sp.t1 - sp.t0);
            sh_t = sp.t0;
            sh_qold = 1e-4;
            if (sp.control && sp.resume) {  // continue with the step size and error history of a snapshot
                const double dt = sp.control[3 * i + 1], qold = sp.control[3 * i + 2];
                if (dt > 0.0 && dt < INFINITY) sh_dt = fmin(dt, sp.t1 - sp.t0);
                if (qold > 0.0 && qold < INFINITY) sh_qold = qold;
            }
            sh_done = 0;
            sh_status = ND_OK;
            sh_steps = 0;
        }
        __syncthreads();
        while (!sh_done) {
            const double h = sh_dt;
            for (int st = 1; st < 7; ++st) {
                for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
                    double acc = 0.0;
                    for (int m = 0; m < st; ++m) acc = __dadd_rn(acc, __dmul_rn(e_a[st][m], K[m][s.ubase + j]));
                    Y[s.ubase + j] = __dadd_rn(u[j], __dmul_rn(h, acc));
                }
                __syncthreads();
                any_instance_rhs<T, VK, EK>(a, s, Y, p, K[st]);
                __syncthreads();
            }
            double se = 0.0;
            for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
                double acc = 0.0;
                for (int m = 0; m < 7; ++m) acc = __dadd_rn(acc, __dmul_rn(e_bt[m], K[m][s.ubase + j]));
                const double e = __dmul_rn(h, acc);
                const double sc = sp.abstol + sp.reltol * fmax(fabs(u[j]), fabs(Y[s.ubase + j]));
                const double r = e / sc;
                se += r * r;
            }
            const double tot = block_sum(se, red);
            if (threadIdx.x == 0) {
                double EEst = sqrt(tot / (double)(n ? n : 1));
                if (!(EEst == EEst)) EEst = 1e10;
                const double beta1 = 7.0 / 50.0, beta2 = 2.0 / 25.0, gamma = 0.9, qmin = 0.2, qmax = 10.0;
                const double q11 = pow(EEst, beta1);
                sh_steps++;
                if (EEst <= 1.0) {
                    double qq = q11 / pow(sh_qold, beta2);
                    qq = fmax(1.0 / qmax, fmin(1.0 / qmin, qq / gamma));
                    const double tn = sh_t + h;
                    sh_t = (fabs(sp.t1 - tn) <= 1e-14 * fmax(1.0, fabs(sp.t1))) ? sp.t1 : tn;
                    sh_qold = fmax(EEst, 1e-4);
                    sh_accept = 1;
                    sh_dt = h / qq;
                } else {
                    sh_accept = 0;
                    sh_dt = h / fmin(1.0 / qmin, q11 / gamma);
                }
                if (sh_accept && sh_t >= sp.t1) {
                    sh_done = 1;
                } else if (sh_steps >= sp.max_steps) {
                    sh_done = 1;
                    sh_status = ND_ERR_MAXITERS;
                } else if (sh_dt < 1e-14 * fmax(1.0, fabs(sh_t))) {
                    sh_done = 1;
                    sh_status = ND_ERR_NOT_CONVERGED;
                } else if (sp.t1 - sh_t < sh_dt * (1 + 1e-12)) {
                    sh_dt = sp.t1 - sh_t;
                }
            }
            __syncthreads();
            if (sh_accept) {
                for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
                    u[j] = Y[s.ubase + j];
                    K[0][s.ubase + j] = K[6][s.ubase + j];
                }
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            status[i] = sh_status;
            nsteps[i] = sh_steps;
            if (sp.control) {
                sp.control[3 * i] = sh_t;
                sp.control[3 * i + 1] = sh_dt;
                sp.control[3 * i + 2] = sh_qold;
            }
        }
    }
}

// ---- batched Newton-CG for swing steady states ------------------------------------------------
// Reduced system at ω = 0: G_v(θ) = Pm_v + Σ_e (K sin terms of the edges at v), exactly
// the aggregation of the RHS.  -∂G/∂θ is the weighted Laplacian with w = K cos(θ_n - θ_v);
// each Newton step solves -J δ = G by CG in the subspace orthogonal to the uniform phase
// shift (G and every Laplacian image are orthogonal to it).
struct NewtonParams {
    double tol;
    int max_newton, max_cg;
    int64_t nv, ninc;  // packed vertices, incidences (scratch strides)
    double cg_rtol;
};

template <int EK>
__global__ void ens_newton_kernel(EnsArgs a, NewtonParams np, double* __restrict__ U, const double* __restrict__ p,
                                  double* __restrict__ work, int32_t* __restrict__ iters, double* __restrict__ resid,
                                  int32_t* __restrict__ status, int32_t* __restrict__ cg_total) {
    using A = Arith<double>;
    __shared__ double red[32];
    __shared__ int sh_inst;
    double* X = work;               // Newton step / CG solution
    double* R = work + np.nv;       // CG residual
    double* Pd = work + 2 * np.nv;  // CG direction
    double* Q = work + 3 * np.nv;   // -J · direction
    double* G = work + 4 * np.nv;   // power mismatch
    double* W = work + 5 * np.nv;   // [ninc] incidence weights K cos(θ_n - θ_v)
    for (;;) {
        const int q = take_instance(a, &sh_inst);
        if (q >= a.n_inst) break;
        const int64_t i = a.order[q];
        const Inst s = instance<ND_V_SWING, EK>(a, i);
        const int64_t nvi = s.nvi;
        double* th = U + s.ubase;  // θ at even, ω at odd positions
        const double* pv = p + s.pbase;
        const double* pe = pv + nvi * 3;
        int it = 0, cgsum = 0, st = ND_OK;
        double res = 0.0;
        for (;;) {
            // residual of the full RHS at ω = 0: max |(Pm + Σ)/M|, and G
            double mx = 0.0;
            for (int64_t v = threadIdx.x; v < nvi; v += blockDim.x) {
                const uint32_t beg = a.row_ptr[s.vbase + v], end = a.row_ptr[s.vbase + v + 1];
                const double uv = th[2 * v];
                double acc = 0.0;
                for (uint32_t k = beg; k < end; ++k)
                    acc = A::add(acc, incidence_term<double, EK>(uv, th[2 * (int64_t)a.nbr[k]], pe, a.eid[k]));
                const double M = pv[3 * v], D = pv[3 * v + 1], Pm = pv[3 * v + 2];
                const double r = A::mul(A::div(1.0, M), A::add(A::sub(Pm, A::mul(D, 0.0)), acc));
                G[s.vbase + v] = A::add(Pm, acc);
                mx = fmax(mx, fabs(r));
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(kFullMask, mx, off));
            __syncthreads();
            if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
            __syncthreads();
            res = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) res = fmax(res, red[w]);
            __syncthreads();
            if (res <= np.tol) break;
            if (!(res == res)) {
                st = ND_ERR_NOT_CONVERGED;
                break;
            }
            if (it >= np.max_newton) {
                st = ND_ERR_MAXITERS;
                break;
            }
            // weights and CG init: X = 0, R = G, P = R
            for (int64_t v = threadIdx.x; v < nvi; v += blockDim.x) {
                const uint32_t beg = a.row_ptr[s.vbase + v], end = a.row_ptr[s.vbase + v + 1];
                const double uv = th[2 * v];
                for (uint32_t k = beg; k < end; ++k) {
                    const int32_t eb = a.eid[k];
                    const double Kk = EK == ND_E_DIFFUSION_UNIT ? 1.0 : pe[eb & 0x7fffffff];
                    const double dth = th[2 * (int64_t)a.nbr[k]] - uv;
                    W[k] = EK == ND_E_KURAMOTO ? Kk * cos(dth) : Kk;
                }
                X[s.vbase + v] = 0.0;
                R[s.vbase + v] = G[s.vbase + v];
                Pd[s.vbase + v] = G[s.vbase + v];
            }
            __syncthreads();
            // keep the right-hand side orthogonal to the uniform shift (it is, up to rounding):
            // a component along the null space would make CG grow x without bound along it
            double gm = 0.0;
            for (int64_t v = threadIdx.x; v < nvi; v += blockDim.x) gm += R[s.vbase + v];
            gm = block_sum(gm, red) / (double)nvi;
            for (int64_t v = threadIdx.x; v < nvi; v += blockDim.x) {
                R[s.vbase + v] -= gm;
                Pd[s.vbase + v] -= gm;
            }
            __syncthreads();
            double rr = 0.0;
            for (int64_t v = threadIdx.x; v < nvi; v += blockDim.x) rr += R[s.vbase + v] * R[s.vbase + v];
            rr = block_sum(rr, red);
            const double rr0 = rr;
            // stop at a relative residual of cg_rtol, or once the linear residual is far
            // below the Newton tolerance
            const double floor2 = (1e-3 * np.tol) * (1e-3 * np.tol);
            int cg = 0;
            while (cg < np.max_cg && rr > np.cg_rtol * np.cg_rtol * rr0 && rr > floor2) {
                __syncthreads();
                double pq = 0.0;
                for (int64_t v = threadIdx.x; v < nvi; v += blockDim.x) {
                    const uint32_t beg = a.row_ptr[s.vbase + v], end = a.row_ptr[s.vbase + v + 1];
                    const double pvv = Pd[s.vbase + v];
                    double acc = 0.0;
                    for (uint32_t k = beg; k < end; ++k) acc += W[k] * (pvv - Pd[s.vbase + a.nbr[k]]);
                    Q[s.vbase + v] = acc;
                    pq += pvv * acc;
                }
                pq = block_sum(pq, red);
                const double alpha = rr / pq;
                double rr_new = 0.0;
                for (int64_t v = threadIdx.x; v < nvi; v += blockDim.x) {
                    X[s.vbase + v] += alpha * Pd[s.vbase + v];
                    R[s.vbase + v] -= alpha * Q[s.vbase + v];
                    rr_new += R[s.vbase + v] * R[s.vbase + v];
                }
                rr_new = block_sum(rr_new, red);
                const double beta = rr_new / rr;
                rr = rr_new;
                for (int64_t v = threadIdx.x; v < nvi; v += blockDim.x)
                    Pd[s.vbase + v] = R[s.vbase + v] + beta * Pd[s.vbase + v];
                ++cg;
            }
            cgsum += cg;
            __syncthreads();
            // Newton update θ += δ with -J δ = G (δ = X, taken with zero mean: the uniform
            // phase shift is free)
            double xm = 0.0;
            for (int64_t v = threadIdx.x; v < nvi; v += blockDim.x) xm += X[s.vbase + v];
            xm = block_sum(xm, red) / (double)nvi;
            for (int64_t v = threadIdx.x; v < nvi; v += blockDim.x) th[2 * v] += X[s.vbase + v] - xm;
            ++it;
            __syncthreads();
        }
        for (int64_t v = threadIdx.x; v < nvi; v += blockDim.x) th[2 * v + 1] = 0.0;
        if (threadIdx.x == 0) {
            iters[i] = it;
            resid[i] = res;
            status[i] = st;
            if (cg_total) cg_total[i] = cgsum;
        }
        __syncthreads();
    }
}

template <typename T>
cudaError_t launch_ens_rhs(const nd_ensemble* e, const EnsArgs& a, const void* u, const void* p, void* du,
                           cudaStream_t s) {
    const unsigned grid = (unsigned)std::min<int64_t>(e->n_inst, 152 * 16);
#define ND_CASE(VK, EK)                                                                                       \
    if (e->vertex_kind == VK && e->edge_kind == EK) {                                                          \
        using E = typename Elem<T>::type;                                                                       \
        ens_rhs_kernel<T, VK, EK><<<grid, 128, 0, s>>>(a, static_cast<const E*>(u), static_cast<const E*>(p),   \
                                                       static_cast<E*>(du));                                    \
        return cudaGetLastError();                                                                             \
    }
    ND_CASE(ND_V_DIFFUSION, ND_E_DIFFUSION)
    ND_CASE(ND_V_DIFFUSION, ND_E_DIFFUSION_UNIT)
    ND_CASE(ND_V_DIFFUSION, ND_E_KURAMOTO)
    ND_CASE(ND_V_KURAMOTO, ND_E_DIFFUSION)
    ND_CASE(ND_V_KURAMOTO, ND_E_DIFFUSION_UNIT)
    ND_CASE(ND_V_KURAMOTO, ND_E_KURAMOTO)
    ND_CASE(ND_V_SWING, ND_E_DIFFUSION)
    ND_CASE(ND_V_SWING, ND_E_DIFFUSION_UNIT)
    ND_CASE(ND_V_SWING, ND_E_KURAMOTO)
#undef ND_CASE
    return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t launch_ens_tsit5(const nd_ensemble* e, const EnsArgs& a, const SolveParams& sp, double* u, const void* p,
                             int32_t* status, int64_t* nsteps, int threads, int blocks, cudaStream_t s) {
#define ND_CASE(VK, EK)                                                                                       \
    if (e->vertex_kind == VK && e->edge_kind == EK) {                                                          \
        ens_tsit5_kernel<T, VK, EK><<<blocks, threads, 0, s>>>(a, sp, u,                                       \
                                                               static_cast<const typename Elem<T>::type*>(p), e->work, \
                                                               status, nsteps);                                \
        return cudaGetLastError();                                                                             \
    }
    ND_CASE(ND_V_DIFFUSION, ND_E_DIFFUSION)
    ND_CASE(ND_V_DIFFUSION, ND_E_DIFFUSION_UNIT)
    ND_CASE(ND_V_DIFFUSION, ND_E_KURAMOTO)
    ND_CASE(ND_V_KURAMOTO, ND_E_DIFFUSION)
    ND_CASE(ND_V_KURAMOTO, ND_E_DIFFUSION_UNIT)
    ND_CASE(ND_V_KURAMOTO, ND_E_KURAMOTO)
    ND_CASE(ND_V_SWING, ND_E_DIFFUSION)
    ND_CASE(ND_V_SWING, ND_E_DIFFUSION_UNIT)
    ND_CASE(ND_V_SWING, ND_E_KURAMOTO)
#undef ND_CASE
    return cudaErrorInvalidValue;
}

EnsArgs args_of(nd_ensemble* e) {
    EnsArgs a;
    a.n_inst = e->n_inst;
    a.v0 = e->v0;
    a.e0 = e->e0;
    a.order = e->order;
    a.row_ptr = e->row_ptr;
    a.nbr = e->incid_nbr;
    a.eid = e->incid_eid;
    a.counter = e->counter;
    return a;
}

cudaError_t ensure_work(nd_ensemble* e, size_t bytes) {
    if (e->work_bytes >= bytes) return cudaSuccess;
    cudaFree(e->work);
    e->work = nullptr;
    e->work_bytes = 0;
    cudaError_t err = cudaMalloc(&e->work, bytes);
    if (err == cudaSuccess) e->work_bytes = bytes;
    return err;
}

void free_ensemble(nd_ensemble* e) {
    cudaFree(e->v0);
    cudaFree(e->e0);
    cudaFree(e->order);
    cudaFree(e->row_ptr);
    cudaFree(e->incid_nbr);
    cudaFree(e->incid_eid);
    cudaFree(e->counter);
    cudaFree(e->work);
}

}  // namespace

}  // namespace nd

using namespace nd;

extern "C" {

int nd_ensemble_create(const nd_ensemble_desc* d, int dtype, nd_ensemble** out) {
    clear_error();
    if (!d || !out) return fail(ND_ERR_ARG, "nd_ensemble_create: NULL argument");
    *out = nullptr;
    if (dtype != ND_F32 && dtype != ND_F64 && dtype != ND_F32X2)
        return fail(ND_ERR_DTYPE, "nd_ensemble_create: dtype must be ND_F32, ND_F64 or ND_F32X2");
    if (d->vertex_kind < ND_V_DIFFUSION || d->vertex_kind > ND_V_SWING || d->edge_kind < ND_E_DIFFUSION ||
        d->edge_kind > ND_E_KURAMOTO || d->coupling != ND_ANTISYMMETRIC)
        return fail(ND_ERR_UNSUPPORTED_COMPONENT, "nd_ensemble_create: component not in the GB300 library");
    if (d->n_instances <= 0 || !d->v_offset || !d->e_offset) return fail(ND_ERR_ARG, "nd_ensemble_create: no instances");
    const int64_t n = d->n_instances;
    const int64_t nv = d->v_offset[n], ne = d->e_offset[n];
    if (d->v_offset[0] != 0 || d->e_offset[0] != 0) return fail(ND_ERR_ARG, "offsets must start at 0");
    if (ne > 0 && (!d->src || !d->dst)) return fail(ND_ERR_ARG, "nd_ensemble_create: NULL edge arrays");
    if (2 * ne > (int64_t)UINT32_MAX || nv > INT32_MAX) return fail(ND_ERR_UNSUPPORTED, "ensemble too large");
    std::vector<uint32_t> deg(nv + 1, 0);
    int max_rows = 0;
    for (int64_t i = 0; i < n; ++i) {
        const int64_t vb = d->v_offset[i], vn = d->v_offset[i + 1] - vb;
        if (vn <= 0 || d->e_offset[i + 1] < d->e_offset[i]) return fail(ND_ERR_ARG, "empty instance or bad offsets");
        max_rows = std::max<int>(max_rows, (int)vn);
        for (int64_t e = d->e_offset[i]; e < d->e_offset[i + 1]; ++e) {
            const int64_t s = d->src[e], t = d->dst[e];
            if (s < 0 || s >= vn || t < 0 || t >= vn) return fail(ND_ERR_ARG, "edge endpoint out of its instance");
            deg[vb + s]++;
            deg[vb + t]++;
        }
    }
    std::vector<uint32_t> row_ptr(nv + 1, 0);
    for (int64_t v = 0; v < nv; ++v) row_ptr[v + 1] = row_ptr[v] + deg[v];
    std::vector<int32_t> nbr((size_t)2 * ne), eid((size_t)2 * ne);
    std::vector<uint32_t> fill(row_ptr.begin(), row_ptr.end() - 1);
    for (int64_t i = 0; i < n; ++i) {
        const int64_t vb = d->v_offset[i], eb = d->e_offset[i];
        for (int64_t e = eb; e < d->e_offset[i + 1]; ++e) {
            const int32_t s = (int32_t)d->src[e], t = (int32_t)d->dst[e];
            const int32_t le = (int32_t)(e - eb);
            nbr[fill[vb + s]] = t;
            eid[fill[vb + s]++] = le | kSrcSideBit;
            nbr[fill[vb + t]] = s;
            eid[fill[vb + t]++] = le;
        }
    }
    std::vector<int32_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
        return d->v_offset[x + 1] - d->v_offset[x] > d->v_offset[y + 1] - d->v_offset[y];
    });
    nd_ensemble* e = new nd_ensemble();
    e->dtype = dtype;
    e->vertex_kind = d->vertex_kind;
    e->edge_kind = d->edge_kind;
    cudaGetDevice(&e->device);
    e->n_inst = n;
    e->nv = nv;
    e->ne = ne;
    e->dim = nv * vertex_dim(d->vertex_kind);
    e->pdim = nv * vertex_pdim(d->vertex_kind) + ne * edge_pdim(d->edge_kind);
    e->max_rows = max_rows;
    auto up = [&](void** dp, const void* hp, size_t bytes) -> cudaError_t {
        cudaError_t err = cudaMalloc(dp, std::max<size_t>(bytes, 16));
        if (err == cudaSuccess && bytes) err = cudaMemcpy(*dp, hp, bytes, cudaMemcpyHostToDevice);
        return err;
    };
    cudaError_t err;
    if ((err = up((void**)&e->v0, d->v_offset, sizeof(int64_t) * (n + 1))) != cudaSuccess ||
        (err = up((void**)&e->e0, d->e_offset, sizeof(int64_t) * (n + 1))) != cudaSuccess ||
        (err = up((void**)&e->order, order.data(), sizeof(int32_t) * n)) != cudaSuccess ||
        (err = up((void**)&e->row_ptr, row_ptr.data(), sizeof(uint32_t) * (nv + 1))) != cudaSuccess ||
        (err = up((void**)&e->incid_nbr, nbr.data(), sizeof(int32_t) * nbr.size())) != cudaSuccess ||
        (err = up((void**)&e->incid_eid, eid.data(), sizeof(int32_t) * eid.size())) != cudaSuccess ||
        (err = cudaMalloc(&e->counter, sizeof(int))) != cudaSuccess) {
        free_ensemble(e);
        delete e;
        return cuda_fail(err, "nd_ensemble_create upload");
    }
    *out = e;
    return ND_OK;
}

int nd_ensemble_destroy(nd_ensemble* e) {
    clear_error();
    if (!e) return ND_OK;
    free_ensemble(e);
    delete e;
    return ND_OK;
}

int nd_ensemble_get_info(const nd_ensemble* e, int64_t* dim, int64_t* pdim) {
    clear_error();
    if (!e) return fail(ND_ERR_ARG, "nd_ensemble_get_info: NULL handle");
    if (dim) *dim = e->dim;
    if (pdim) *pdim = e->pdim;
    return ND_OK;
}

int nd_ensemble_rhs(nd_ensemble* e, int dtype, void* du, const void* u, const void* p, void* stream) {
    clear_error();
    ND_NVTX("nd_ensemble_rhs");
    if (!e || !du || !u) return fail(ND_ERR_ARG, "nd_ensemble_rhs: NULL argument");
    if (dtype != e->dtype) return fail(ND_ERR_DTYPE, "nd_ensemble_rhs: element type differs from the ensemble's");
    if (e->pdim > 0 && !p) return fail(ND_ERR_ARG, "nd_ensemble_rhs: p is NULL");
    const EnsArgs a = args_of(e);
    cudaError_t err = e->dtype == ND_F64   ? launch_ens_rhs<double>(e, a, u, p, du, (cudaStream_t)stream)
                      : e->dtype == ND_F32 ? launch_ens_rhs<float>(e, a, u, p, du, (cudaStream_t)stream)
                                           : launch_ens_rhs<F32x2>(e, a, u, p, du, (cudaStream_t)stream);
    return err == cudaSuccess ? ND_OK : cuda_fail(err, "nd_ensemble_rhs");
}

int nd_ensemble_solve_tsit5(nd_ensemble* e, double* u, const void* p, double t0, double t1, double reltol,
                            double abstol, int64_t max_steps, int threads, int32_t* status, int64_t* nsteps,
                            void* stream) {
    return nd_ensemble_solve_tsit5_ex(e, u, p, t0, t1, reltol, abstol, max_steps, threads, status, nsteps, nullptr, 0,
                                      stream);
}

int nd_ensemble_solve_tsit5_ex(nd_ensemble* e, double* u, const void* p, double t0, double t1, double reltol,
                               double abstol, int64_t max_steps, int threads, int32_t* status, int64_t* nsteps,
                               double* control, int resume, void* stream) {
    clear_error();
    ND_NVTX("nd_ensemble_solve_tsit5");
    if (resume && !control) return fail(ND_ERR_ARG, "nd_ensemble_solve_tsit5_ex: resume needs the control array");
    if (!e || !u || !status || !nsteps) return fail(ND_ERR_ARG, "nd_ensemble_solve_tsit5: NULL argument");
    if (!(t1 > t0) || !(reltol > 0) || !(abstol > 0)) return fail(ND_ERR_ARG, "nd_ensemble_solve_tsit5: bad time span or tolerances");
    if (e->pdim > 0 && !p) return fail(ND_ERR_ARG, "nd_ensemble_solve_tsit5: p is NULL");
    if (threads == 0) threads = e->tuned_threads ? e->tuned_threads : 128;
    if (threads != 64 && threads != 128 && threads != 256 && threads != 512)
        return fail(ND_ERR_ARG, "nd_ensemble_solve_tsit5: threads must be 64, 128, 256 or 512 (0 = tuned)");
    cudaError_t err = upload_tableau();
    if (err != cudaSuccess) return cuda_fail(err, "tableau upload");
    if ((err = ensure_work(e, sizeof(double) * 8 * (size_t)e->dim)) != cudaSuccess) return cuda_fail(err, "workspace");
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm,
        e->dtype == ND_F64   ? (const void*)ens_tsit5_kernel<double, ND_V_SWING, ND_E_KURAMOTO>
        : e->dtype == ND_F32 ? (const void*)ens_tsit5_kernel<float, ND_V_SWING, ND_E_KURAMOTO>
                             : (const void*)ens_tsit5_kernel<F32x2, ND_V_SWING, ND_E_KURAMOTO>,
        threads, 0);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->device);
    const int blocks = (int)std::min<int64_t>(e->n_inst, (int64_t)sms * std::max(1, per_sm));
    SolveParams sp{t0,     t1,     reltol,   abstol, max_steps > 0 ? max_steps : (int64_t)ND_ENSEMBLE_DEFAULT_MAX_STEPS,
                   e->dim, control, resume ? 1 : 0};
    const EnsArgs a = args_of(e);
    // The persistent kernel (and the reset of its work queue) run as one captured graph.
    cudaStream_t s = (cudaStream_t)stream;
    cudaStream_t cs;
    if ((err = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) return cuda_fail(err, "stream");
    cudaEvent_t ev;
    cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    cudaGraph_t g = nullptr;
    cudaGraphExec_t x = nullptr;
    err = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (err == cudaSuccess) {
        cudaMemsetAsync(e->counter, 0, sizeof(int), cs);
        err = e->dtype == ND_F64   ? launch_ens_tsit5<double>(e, a, sp, u, p, status, nsteps, threads, blocks, cs)
              : e->dtype == ND_F32 ? launch_ens_tsit5<float>(e, a, sp, u, p, status, nsteps, threads, blocks, cs)
                                   : launch_ens_tsit5<F32x2>(e, a, sp, u, p, status, nsteps, threads, blocks, cs);
        cudaError_t e2 = cudaStreamEndCapture(cs, &g);
        if (err == cudaSuccess) err = e2;
    }
    if (err == cudaSuccess) err = cudaGraphInstantiate(&x, g, 0);
    if (err == cudaSuccess) err = cudaEventRecord(ev, s);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(cs, ev, 0);
    if (err == cudaSuccess) err = cudaGraphLaunch(x, cs);
    if (err == cudaSuccess) err = cudaEventRecord(ev, cs);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(s, ev, 0);
    if (x) cudaGraphExecDestroy(x);
    if (g) cudaGraphDestroy(g);
    cudaEventDestroy(ev);
    cudaStreamDestroy(cs);
    return err == cudaSuccess ? ND_OK : cuda_fail(err, "nd_ensemble_solve_tsit5");
}

int nd_ensemble_set_threads(nd_ensemble* e, int threads) {
    clear_error();
    if (!e) return fail(ND_ERR_ARG, "nd_ensemble_set_threads: NULL handle");
    if (threads != 0 && threads != 64 && threads != 128 && threads != 256 && threads != 512)
        return fail(ND_ERR_ARG, "threads must be 0, 64, 128, 256 or 512");
    e->tuned_threads = threads;
    return ND_OK;
}

int nd_ensemble_fixpoint(nd_ensemble* e, double* u, const double* p, double tol, int max_newton, int max_cg,
                         int32_t* iters, double* resid, int32_t* status, int32_t* cg_iters, void* stream) {
    clear_error();
    ND_NVTX("nd_ensemble_fixpoint");
    if (!e || !u || !p || !iters || !resid || !status) return fail(ND_ERR_ARG, "nd_ensemble_fixpoint: NULL argument");
    if (e->vertex_kind != ND_V_SWING)
        return fail(ND_ERR_UNSUPPORTED, "nd_ensemble_fixpoint: steady states are implemented for swing vertices");
    if (e->dtype != ND_F64) return fail(ND_ERR_DTYPE, "nd_ensemble_fixpoint: the Newton solve runs in FP64");
    if (!(tol > 0) || max_newton <= 0) return fail(ND_ERR_ARG, "nd_ensemble_fixpoint: bad tolerance or budget");
    if (max_cg <= 0) max_cg = std::max(100, 4 * e->max_rows);
    cudaError_t err = ensure_work(e, sizeof(double) * ((size_t)5 * e->nv + (size_t)2 * e->ne + 1));
    if (err != cudaSuccess) return cuda_fail(err, "workspace");
    cudaStream_t s = (cudaStream_t)stream;
    if ((err = cudaMemsetAsync(e->counter, 0, sizeof(int), s)) != cudaSuccess) return cuda_fail(err, "memset");
    NewtonParams np{tol, max_newton, max_cg, e->nv, 2 * e->ne, 1e-10};
    const EnsArgs a = args_of(e);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->device);
    const int blocks = (int)std::min<int64_t>(e->n_inst, (int64_t)sms * 8);
    switch (e->edge_kind) {
        case ND_E_KURAMOTO:
            ens_newton_kernel<ND_E_KURAMOTO><<<blocks, 256, 0, s>>>(a, np, u, p, e->work, iters, resid, status, cg_iters);
            break;
        case ND_E_DIFFUSION:
            ens_newton_kernel<ND_E_DIFFUSION><<<blocks, 256, 0, s>>>(a, np, u, p, e->work, iters, resid, status, cg_iters);
            break;
        default:
            ens_newton_kernel<ND_E_DIFFUSION_UNIT><<<blocks, 256, 0, s>>>(a, np, u, p, e->work, iters, resid, status,
                                                                           cg_iters);
    }
    err = cudaGetLastError();
    return err == cudaSuccess ? ND_OK : cuda_fail(err, "nd_ensemble_fixpoint");
}

}  // extern "C"

// Autotuner: time a short solve of the ensemble with each block size and keep the
// fastest for later solves with threads = 0.  Works on a copy of u.
extern "C" int nd_ensemble_autotune(nd_ensemble* e, const double* u, const void* p, double t0, double t_probe,
                                    double reltol, double abstol, int* chosen, void* stream) {
    clear_error();
    ND_NVTX("nd_ensemble_autotune");
    if (!e || !u || !chosen) return fail(ND_ERR_ARG, "nd_ensemble_autotune: NULL argument");
    cudaStream_t s = (cudaStream_t)stream;
    double* uc = nullptr;
    int32_t* st = nullptr;
    int64_t* ns = nullptr;
    cudaError_t err = cudaMalloc(&uc, sizeof(double) * std::max<int64_t>(e->dim, 1));
    if (err == cudaSuccess) err = cudaMalloc(&st, sizeof(int32_t) * e->n_inst);
    if (err == cudaSuccess) err = cudaMalloc(&ns, sizeof(int64_t) * e->n_inst);
    cudaEvent_t a0, a1;
    cudaEventCreate(&a0);
    cudaEventCreate(&a1);
    const int cands[4] = {64, 128, 256, 512};
    float best = 1e30f;
    int best_t = 128;
    for (int c = 0; c < 4 && err == cudaSuccess; ++c) {
        for (int rep = 0; rep < 2 && err == cudaSuccess; ++rep) {  // first run warms up
            err = cudaMemcpyAsync(uc, u, sizeof(double) * e->dim, cudaMemcpyDeviceToDevice, s);
            if (err == cudaSuccess) err = cudaEventRecord(a0, s);
            if (err == cudaSuccess) {
                const int rc = nd_ensemble_solve_tsit5(e, uc, p, t0, t0 + t_probe, reltol, abstol, 0, cands[c], st, ns,
                                                       stream);
                if (rc != ND_OK) err = cudaErrorUnknown;
            }
            if (err == cudaSuccess) err = cudaEventRecord(a1, s);
            if (err == cudaSuccess) err = cudaEventSynchronize(a1);
        }
        float ms = 0;
        if (err == cudaSuccess) cudaEventElapsedTime(&ms, a0, a1);
        if (err == cudaSuccess && ms < best) {
            best = ms;
            best_t = cands[c];
        }
    }
    cudaEventDestroy(a0);
    cudaEventDestroy(a1);
    cudaFree(uc);
    cudaFree(st);
    cudaFree(ns);
    if (err != cudaSuccess) return cuda_fail(err, "nd_ensemble_autotune");
    e->tuned_threads = best_t;
    *chosen = best_t;
    return ND_OK;
}
