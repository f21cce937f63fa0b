// Analytic Jacobian-vector product of the network RHS, jv = (∂f/∂u)(u, p) · v.
//
// The reference differentiates the core loop with ForwardDiff (Dual numbers through
// src/coreloop.jl, cache promotion at :10-21; tested against finite differences in
// test/AD_test.jl:54-60).  For the library components the derivative is written out:
//   diffusion edge    d[w (u_s - u_d)]      = w (v_s - v_d)
//   unit diffusion    d[u_s - u_d]          = v_s - v_d
//   kuramoto / line   d[K sin(θ_s - θ_d)]   = K cos(θ_s - θ_d) (v_s - v_d)
// and AntiSymmetric hands -d(y_dst) to the source, so at row v with neighbour n every
// incidence contributes c (v_n - v_v) with c = w, 1 or K cos(θ_n - θ_v).  Vertices:
//   diffusion / kuramoto   jv = Σ                  swing   jv_θ = v_ω,  jv_ω = (Σ - D v_ω) / M
// One thread per row over the slot-ordered CSR, rows summed in edge order; rows of degree
// above 32 (the first slots) take a warp each.
#include <algorithm>

#include "nd_components.cuh"
#include "nd_internal.h"

namespace nd {

int jacobian_times(nd_handle* h, void* jv, const void* u, const void* p, const void* v, cudaStream_t s);

namespace {

// Contribution c (v_n - v_v) of one incidence (neighbour n) to row v.
template <typename T, int VK, int EK>
__device__ __forceinline__ T jvp_term(int2 inc, T uv, T dv, const T* __restrict__ u, const T* __restrict__ pe,
                                      const T* __restrict__ vv) {
    using A = Arith<T>;
    constexpr int DV = VertexDims<VK>::dim;
    const int64_t n = inc.x;
    const int32_t e = inc.y & 0x7fffffff;
    T c;
    if constexpr (EK == ND_E_DIFFUSION) c = pe[e];
    else if constexpr (EK == ND_E_DIFFUSION_UNIT) c = T(1);
    else c = A::mul(pe[e], A::cos_phase(A::sub(u[n * DV], uv)));
    return A::mul(c, A::sub(vv[n * DV], dv));
}

template <typename T, int VK>
__device__ __forceinline__ void jvp_vertex(int64_t v, T acc, const T* __restrict__ pv, const T* __restrict__ vv,
                                           T* __restrict__ jv) {
    using A = Arith<T>;
    if constexpr (VK == ND_V_SWING) {
        const T M = pv[3 * v], D = pv[3 * v + 1];
        jv[2 * v] = vv[2 * v + 1];
        jv[2 * v + 1] = A::div(A::sub(acc, A::mul(D, vv[2 * v + 1])), M);
    } else {
        jv[v] = acc;
    }
}

// Rows [first, nv) of the slot order, a thread each.
template <typename T, int VK, int EK>
__global__ void jvp_kernel(int64_t first, int64_t nv, const uint32_t* __restrict__ slot_ptr,
                           const int32_t* __restrict__ slot_vertex, const int2* __restrict__ incid,
                           const T* __restrict__ u, const T* __restrict__ p, const T* __restrict__ vv,
                           T* __restrict__ jv) {
    using A = Arith<T>;
    constexpr int DV = VertexDims<VK>::dim;
    const T* pe = p + nv * VertexDims<VK>::pdim;
    for (int64_t s = first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < nv;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = slot_vertex[s];
        const T uv = u[v * DV], dv = vv[v * DV];
        T acc = T(0);
        for (uint32_t k = slot_ptr[s]; k < slot_ptr[s + 1]; ++k)
            acc = A::add(acc, jvp_term<T, VK, EK>(incid[k], uv, dv, u, pe, vv));
        jvp_vertex<T, VK>(v, acc, p, vv, jv);
    }
}

// Rows [0, n_long) of the slot order (degree above 32: medium and heavy rows), a warp
// each: lane partial sums and a butterfly.
template <typename T, int VK, int EK>
__global__ void jvp_warp_kernel(int64_t n_long, int64_t nv, const uint32_t* __restrict__ slot_ptr,
                                const int32_t* __restrict__ slot_vertex, const int2* __restrict__ incid,
                                const T* __restrict__ u, const T* __restrict__ p, const T* __restrict__ vv,
                                T* __restrict__ jv) {
    using A = Arith<T>;
    constexpr int DV = VertexDims<VK>::dim;
    const T* pe = p + nv * VertexDims<VK>::pdim;
    const int lane = threadIdx.x & 31;
    const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (s >= n_long) return;  // warp-uniform
    const int64_t v = slot_vertex[s];
    const T uv = u[v * DV], dv = vv[v * DV];
    T acc = T(0);
    for (uint32_t k = slot_ptr[s] + lane; k < slot_ptr[s + 1]; k += 32)
        acc = A::add(acc, jvp_term<T, VK, EK>(incid[k], uv, dv, u, pe, vv));
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc = A::add(acc, __shfl_xor_sync(0xffffffffu, acc, off));
    if (lane == 0) jvp_vertex<T, VK>(v, acc, p, vv, jv);
}

template <typename T>
cudaError_t launch_jvp(const nd_handle* h, const void* u, const void* p, const void* v, void* jv, cudaStream_t s) {
    const Topology& t = h->topo;
    const int64_t n_long = (int64_t)t.n_heavy + t.n_medium;  // the first slots: degree > 32
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((t.nv - n_long + 255) / 256, 152 * 16));
    const unsigned wgrid = (unsigned)((n_long * 32 + 255) / 256);
    const int2* inc = reinterpret_cast<const int2*>(t.incid);
#define ND_CASE(VK, EK)                                                                                          \
    if (h->vertex_kind == VK && h->edge_kind == EK) {                                                             \
        if (n_long > 0)                                                                                           \
            jvp_warp_kernel<T, VK, EK><<<wgrid, 256, 0, s>>>(n_long, t.nv, t.slot_ptr, t.slot_vertex, inc,        \
                                                            static_cast<const T*>(u), static_cast<const T*>(p),   \
                                                            static_cast<const T*>(v), static_cast<T*>(jv));       \
        if (t.nv > n_long)                                                                                        \
            jvp_kernel<T, VK, EK><<<grid, 256, 0, s>>>(n_long, t.nv, t.slot_ptr, t.slot_vertex, inc,              \
                                                      static_cast<const T*>(u), static_cast<const T*>(p),         \
                                                      static_cast<const T*>(v), static_cast<T*>(jv));             \
        return cudaGetLastError();                                                                                \
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

}  // namespace

}  // namespace nd

using namespace nd;

extern "C" int nd_jvp(nd_handle* h, int dtype, void* jv, const void* u, const void* p, const void* v, double t,
                      void* stream) {
    ND_NVTX("nd_jvp");
    (void)t;
    clear_error();
    if (!h || !jv || !u || !v) return fail(ND_ERR_ARG, "nd_jvp: NULL argument");
    if (dtype != h->dtype) return fail(ND_ERR_DTYPE, "nd_jvp: element type differs from the handle's");
    if (h->pdim > 0 && !p) return fail(ND_ERR_ARG, "nd_jvp: p is NULL");
    if (h->batched.enabled) return jacobian_times(h, jv, u, p, v, (cudaStream_t)stream);
    cudaError_t err = h->dtype == ND_F64 ? launch_jvp<double>(h, u, p, v, jv, (cudaStream_t)stream)
                                         : launch_jvp<float>(h, u, p, v, jv, (cudaStream_t)stream);
    return err == cudaSuccess ? ND_OK : cuda_fail(err, "nd_jvp");
}
