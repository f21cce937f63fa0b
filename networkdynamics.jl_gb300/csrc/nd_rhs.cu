// Fused network right-hand side over the destination-sorted CSR.
//
// One RHS replaces the reference's phased core loop (src/coreloop.jl:22-101): vertex g,
// edge g/f, the gather of vertex outputs into edge inputs (src/gbufs.jl:7-25), the
// aggregation (src/aggregators.jl:133-151) and vertex f.  Vertex outputs are the first
// state (StateMask(1)), so edges read u directly; edge values live in registers; the
// per-vertex sum walks the row in ascending edge id, which is the SequentialAggregator
// order, and du is written once.  No output, gather or aggregation buffers exist.
//
// Degree buckets: rows with degree <= kThreadMaxDeg are summed by one thread each; longer
// rows (power-law hubs) by a warp that loads and evaluates 32 incidences at a time and
// then adds them in order (sequential mode) or as a fixed shuffle tree (tree mode).

#include "nd_components.cuh"
#include "nd_internal.h"

namespace nd {

namespace {

constexpr int kLightBlock = 256;
constexpr int kHubBlock = 256;
constexpr int kWarpsPerHubBlock = kHubBlock / 32;

template <typename T, int VK, int EK>
__global__ void __launch_bounds__(kLightBlock) rhs_light_kernel(RhsArgs a) {
    using A = Arith<T>;
    constexpr int DV = VertexDims<VK>::dim;
    const int i = blockIdx.x * kLightBlock + threadIdx.x;
    if (i >= a.n_light) return;
    const int64_t v = a.light[i];
    const T* __restrict__ u = static_cast<const T*>(a.u);
    const T* __restrict__ p = static_cast<const T*>(a.p);
    const T* __restrict__ pe = p + a.nv * VertexDims<VK>::pdim;
    const uint32_t beg = a.row_ptr[v], end = a.row_ptr[v + 1];
    const T uv = u[v * DV];
    T acc = T(0);
    for (uint32_t k = beg; k < end; ++k) {
        const Incidence inc = a.incid[k];
        const T un = u[(int64_t)inc.nbr * DV];
        acc = A::add(acc, incidence_term<T, EK>(uv, un, pe, inc.eid));
    }
    vertex_f<T, VK>(static_cast<T*>(a.du), u, p, v, acc);
}

// Sequential (in-order) warp-per-hub: lanes evaluate 32 consecutive incidences, lane 0
// adds them in row order.  With KAHAN (FP32 only) lane 0 keeps a compensation term.
template <typename T, int VK, int EK, bool KAHAN>
__global__ void __launch_bounds__(kHubBlock) rhs_hub_seq_kernel(RhsArgs a) {
    using A = Arith<T>;
    constexpr int DV = VertexDims<VK>::dim;
    __shared__ T stage[kWarpsPerHubBlock][32];
    const int warp_in_block = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * kWarpsPerHubBlock + warp_in_block;
    if (w >= a.n_hubs) return;
    const int64_t v = a.hubs[w];
    const T* __restrict__ u = static_cast<const T*>(a.u);
    const T* __restrict__ p = static_cast<const T*>(a.p);
    const T* __restrict__ pe = p + a.nv * VertexDims<VK>::pdim;
    const uint32_t beg = a.row_ptr[v], end = a.row_ptr[v + 1];
    const T uv = u[v * DV];
    T acc = T(0), comp = T(0);
    for (uint32_t c = beg; c < end; c += 32) {
        const uint32_t k = c + lane;
        T term = T(0);
        if (k < end) {
            const Incidence inc = a.incid[k];
            term = incidence_term<T, EK>(uv, u[(int64_t)inc.nbr * DV], pe, inc.eid);
        }
        stage[warp_in_block][lane] = term;
        __syncwarp();
        if (lane == 0) {
            const uint32_t n = min(32u, end - c);
            for (uint32_t j = 0; j < n; ++j) {
                if constexpr (KAHAN) {
                    const T y = A::sub(stage[warp_in_block][j], comp);
                    const T s = A::add(acc, y);
                    comp = A::sub(A::sub(s, acc), y);
                    acc = s;
                } else {
                    acc = A::add(acc, stage[warp_in_block][j]);
                }
            }
        }
        __syncwarp();
    }
    if (lane == 0) vertex_f<T, VK>(static_cast<T*>(a.du), u, p, v, acc);
}

// Tree warp-per-hub: each lane sums a strided slice, then a fixed xor-shuffle tree.  The
// result is deterministic but rounds differently from the sequential order.
template <typename T, int VK, int EK, bool KAHAN>
__global__ void __launch_bounds__(kHubBlock) rhs_hub_tree_kernel(RhsArgs a) {
    using A = Arith<T>;
    constexpr int DV = VertexDims<VK>::dim;
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * kWarpsPerHubBlock + (threadIdx.x >> 5);
    if (w >= a.n_hubs) return;
    const int64_t v = a.hubs[w];
    const T* __restrict__ u = static_cast<const T*>(a.u);
    const T* __restrict__ p = static_cast<const T*>(a.p);
    const T* __restrict__ pe = p + a.nv * VertexDims<VK>::pdim;
    const uint32_t beg = a.row_ptr[v], end = a.row_ptr[v + 1];
    const T uv = u[v * DV];
    T acc = T(0), comp = T(0);
    for (uint32_t k = beg + lane; k < end; k += 32) {
        const Incidence inc = a.incid[k];
        const T term = incidence_term<T, EK>(uv, u[(int64_t)inc.nbr * DV], pe, inc.eid);
        if constexpr (KAHAN) {
            const T y = A::sub(term, comp);
            const T s = A::add(acc, y);
            comp = A::sub(A::sub(s, acc), y);
            acc = s;
        } else {
            acc = A::add(acc, term);
        }
    }
    if constexpr (KAHAN) acc = A::sub(acc, comp);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc = A::add(acc, __shfl_xor_sync(0xffffffffu, acc, off));
    if (lane == 0) vertex_f<T, VK>(static_cast<T*>(a.du), u, p, v, acc);
}

template <typename T, int VK, int EK>
cudaError_t launch_typed(const RhsArgs& a, cudaStream_t s) {
    if (a.n_light > 0) {
        rhs_light_kernel<T, VK, EK><<<(a.n_light + kLightBlock - 1) / kLightBlock, kLightBlock, 0, s>>>(a);
    }
    if (a.n_hubs > 0) {
        const int grid = (a.n_hubs + kWarpsPerHubBlock - 1) / kWarpsPerHubBlock;
        constexpr bool kF32 = sizeof(T) == 4;
        if (a.sum_order == ND_ORDER_TREE) {
            rhs_hub_tree_kernel<T, VK, EK, kF32><<<grid, kHubBlock, 0, s>>>(a);
        } else {
            rhs_hub_seq_kernel<T, VK, EK, kF32><<<grid, kHubBlock, 0, s>>>(a);
        }
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_dtype(const RhsArgs& a, cudaStream_t s) {
#define ND_CASE(VK, EK) \
    if (a.vertex_kind == VK && a.edge_kind == EK) return launch_typed<T, VK, EK>(a, s);
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

cudaError_t launch_rhs(int dtype, const RhsArgs& a, cudaStream_t s) {
    return dtype == ND_F64 ? launch_dtype<double>(a, s) : launch_dtype<float>(a, s);
}

}  // namespace nd
