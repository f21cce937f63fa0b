// Two-phase (edge-centric) network right-hand side, for canonical edge lists.
//
// The reference evaluates every edge once (edge g, src/coreloop.jl:76-78), stores both
// outputs in the output buffer (AntiSymmetric: y_src = -y_dst,
// src/component_functions.jl:117-127) and then adds the buffer into each vertex in
// buffer order (SequentialAggregator, src/aggregators.jl:140-151).  The two phases here
// do the same on the GPU:
//   E  one thread per edge, in edge order: y_e = g(u_src, u_dst, p_e), written to y and,
//      grouped by destination, to ybkt (EdgeLayout in nd_internal.h);
//   R  one row per vertex: the row's destination-side values (edges (s, v), s < v, in
//      ascending edge id) followed by the negated values of its own source block, which
//      is exactly the order of the vertex's entries in the reference's output buffer, then
//      vertex f.  Rows reuse the window / heavy-row machinery of the fused kernel.
// The edge function and its FP64 operations run once per edge instead of once per
// incidence, edge parameters and incidence data are read in order, and the random
// traffic shrinks to the gather of u[dst] (kept in L2) and the bucket-local gathers of
// ybkt.
#include "nd_components.cuh"
#include "nd_exact.cuh"
#include "nd_internal.h"
#include "nd_scan.cuh"

namespace nd {

namespace {

using namespace dev;

template <typename T>
struct SmemR {
    static constexpr int kWin = kWindowIncidences * (int)sizeof(T) + 4 * kWindow * 4 + kWindowIncidences;
    static constexpr int kHeavy = kTile * (int)sizeof(double);
    static constexpr int kBytes = kWin > kHeavy ? kWin : kHeavy;
};

template <typename T>
__device__ __forceinline__ T negate(T x) {
    if constexpr (sizeof(T) == 8) return __longlong_as_double(__double_as_longlong(x) ^ (1ll << 63));
    else return __int_as_float(__float_as_int(x) ^ (int)0x80000000);
}

// ---- phase E -------------------------------------------------------------------------------
template <typename T, int VK, int EK>
__global__ void __launch_bounds__(kBlock) edge_phase_kernel(RhsArgs a) {
    constexpr int DV = VertexDims<VK>::dim;
    const T* __restrict__ u = static_cast<const T*>(a.u);
    const T* __restrict__ pe = static_cast<const T*>(a.p) + a.nv * VertexDims<VK>::pdim;
    T* __restrict__ y = static_cast<T*>(a.y);
    T* __restrict__ ybkt = static_cast<T*>(a.ybkt);
    const uint64_t keep = policy_evict_last(), stream = policy_evict_first();
    const int64_t e0 = (int64_t)blockIdx.x * kEdgeChunk;
    const int64_t e1 = min(e0 + (int64_t)kEdgeChunk, a.ne);
#pragma unroll 4
    for (int64_t e = e0 + threadIdx.x; e < e1; e += kBlock) {
        const int32_t s = ld_hint(a.esrc + e, stream);
        const int32_t d = ld_hint(a.edst + e, stream);
        const int32_t q = ld_hint(a.q + e, stream);
        const T us = ld_hint(u + (int64_t)s * DV, keep);
        const T ud = ld_hint(u + (int64_t)d * DV, keep);
        const T w = edge_param<T, EK>(pe, (int32_t)e, stream);
        const T yv = edge_g_w<T, EK>(us, ud, w);
        y[e] = yv;
        ybkt[q] = yv;
    }
}

// Term j (0-based, in row order) of a row whose destination-side entries start at dp
// (nd of them) and whose source block starts at sp.
template <typename T>
__device__ __forceinline__ T row_term(const RhsArgs& a, uint32_t dp, int nd, uint32_t sp, int j, uint64_t pol) {
    const T* __restrict__ y = static_cast<const T*>(a.y);
    const T* __restrict__ ybkt = static_cast<const T*>(a.ybkt);
    if (j < nd) return ld_hint(ybkt + ld_hint(a.loc + dp + j, pol), pol);
    return negate(ld_hint(y + sp + (j - nd), pol));
}

// ---- phase R: heavy rows, a block per row ---------------------------------------------------
template <typename T, int VK, int MODE>
__device__ __forceinline__ void heavy_row_r(const RhsArgs& a, int slot, unsigned char* smem) {
    using A = Arith<T>;
    const T* __restrict__ u = static_cast<const T*>(a.u);
    const T* __restrict__ p = static_cast<const T*>(a.p);
    const uint64_t stream = policy_evict_first();
    const int64_t v = __ldg(a.slot_vertex + slot);
    const uint32_t dp = __ldg(a.dptr + v), sp = __ldg(a.sptr + v);
    const int nd = (int)(__ldg(a.dptr + v + 1) - dp);
    const int deg = nd + (int)(__ldg(a.sptr + v + 1) - sp);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if constexpr (sizeof(T) == 8 && MODE != kModeTree) {
        double* tile = reinterpret_cast<double*>(smem);
        double S = 0.0;
        for (int base = 0; base < deg; base += kTile) {
            const int n = min(kTile, deg - base);
#pragma unroll 4
            for (int i = tid; i < n; i += kBlock) tile[i] = row_term<T>(a, dp, nd, sp, base + i, stream);
            __syncthreads();
            if (warp == 0) {
                if constexpr (MODE == kModeNative) {
                    if (lane == 0)
                        for (int i = 0; i < n; ++i) S = __dadd_rn(S, tile[i]);
                } else {
                    S = exact_scan_wide(S, tile, n, lane);
                }
            }
            __syncthreads();
        }
        if (tid == 0) vertex_f<T, VK>(static_cast<T*>(a.du), u, p, v, (T)S);
    } else {
        T* red = reinterpret_cast<T*>(smem);
        T acc = T(0), comp = T(0);
#pragma unroll 4
        for (int j = tid; j < deg; j += kBlock) {
            const T term = row_term<T>(a, dp, nd, sp, j, stream);
            if constexpr (sizeof(T) == 4) {
                const T yk = A::sub(term, comp);
                const T s = A::add(acc, yk);
                comp = A::sub(A::sub(s, acc), yk);
                acc = s;
            } else {
                acc = A::add(acc, term);
            }
        }
        if constexpr (sizeof(T) == 4) acc = A::sub(acc, comp);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc = A::add(acc, __shfl_xor_sync(kFull, acc, off));
        if (lane == 0) red[warp] = acc;
        __syncthreads();
        if (tid == 0) {
            T s = red[0];
#pragma unroll
            for (int w = 1; w < kWarpsPerBlock; ++w) s = A::add(s, red[w]);
            vertex_f<T, VK>(static_cast<T*>(a.du), u, p, v, s);
        }
    }
}

// ---- phase R: a block per window of rows ----------------------------------------------------
template <typename T, int VK, int MODE>
__device__ __forceinline__ void window_r(const RhsArgs& a, int win, unsigned char* smem) {
    using A = Arith<T>;
    const T* __restrict__ u = static_cast<const T*>(a.u);
    const T* __restrict__ p = static_cast<const T*>(a.p);
    T* s_term = reinterpret_cast<T*>(smem);                                    // [kWindowIncidences]
    uint32_t* s_dp = reinterpret_cast<uint32_t*>(s_term + kWindowIncidences);  // [kWindow]
    uint32_t* s_sp = s_dp + kWindow;
    int32_t* s_nd = reinterpret_cast<int32_t*>(s_sp + kWindow);
    int32_t* s_start = s_nd + kWindow;
    uint8_t* s_owner = reinterpret_cast<uint8_t*>(s_start + kWindow);  // [kWindowIncidences]
    const uint64_t stream = policy_evict_first();
    const int slot0 = a.n_heavy + __ldg(a.win_ptr + win), slot1 = a.n_heavy + __ldg(a.win_ptr + win + 1);
    const uint32_t i0 = __ldg(a.slot_ptr + slot0), i1 = __ldg(a.slot_ptr + slot1);
    const int n = (int)(i1 - i0);
    const int tid = threadIdx.x;
    const int s = slot0 + tid;
    const bool has_row = s < slot1;
    int64_t v = 0;
    int beg = 0, end = 0;
    if (has_row) {
        v = __ldg(a.slot_vertex + s);
        beg = (int)(__ldg(a.slot_ptr + s) - i0);
        end = (int)(__ldg(a.slot_ptr + s + 1) - i0);
        const uint32_t dp = __ldg(a.dptr + v);
        s_dp[tid] = dp;
        s_nd[tid] = (int)(__ldg(a.dptr + v + 1) - dp);
        s_sp[tid] = __ldg(a.sptr + v);
        s_start[tid] = beg;
        for (int j = beg; j < end; ++j) s_owner[j] = (uint8_t)tid;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = tid; k < n; k += kBlock) {
        const int t = s_owner[k];
        s_term[k] = row_term<T>(a, s_dp[t], s_nd[t], s_sp[t], k - s_start[t], stream);
    }
    __syncthreads();
    if (!has_row) return;
    T acc = T(0);
    if constexpr (sizeof(T) == 8) {
        for (int j = beg; j < end; ++j) acc = __dadd_rn(acc, s_term[j]);
    } else {
        if (end - beg > kLightMaxDeg) {
            T comp = T(0);
            for (int j = beg; j < end; ++j) {
                const T yk = A::sub(s_term[j], comp);
                const T t = A::add(acc, yk);
                comp = A::sub(A::sub(t, acc), yk);
                acc = t;
            }
            acc = A::sub(acc, comp);
        } else {
            for (int j = beg; j < end; ++j) acc = A::add(acc, s_term[j]);
        }
    }
    vertex_f<T, VK>(static_cast<T*>(a.du), u, p, v, acc);
}

template <typename T, int VK, int MODE>
__global__ void __launch_bounds__(kBlock, 8) row_phase_kernel(RhsArgs a) {
    __shared__ __align__(16) unsigned char smem[SmemR<T>::kBytes];
    const int nh = a.heavy_separate ? 0 : a.n_heavy;
    const int b = blockIdx.x;
    if (b < nh) heavy_row_r<T, VK, MODE>(a, b, smem);
    else window_r<T, VK, MODE>(a, b - nh, smem);
}

template <typename T, int VK, int EK>
cudaError_t launch_typed(const RhsArgs& a, cudaStream_t s, int phases) {
    if ((phases & kPhaseEdge) && a.n_chunks > 0)
        edge_phase_kernel<T, VK, EK><<<(unsigned)a.n_chunks, kBlock, 0, s>>>(a);
    const int grid = (a.heavy_separate ? 0 : a.n_heavy) + a.n_windows;
    if (!(phases & kPhaseRow) || grid == 0) return cudaGetLastError();
    if constexpr (sizeof(T) == 4) {
        row_phase_kernel<T, VK, kModeTree><<<grid, kBlock, 0, s>>>(a);
    } else {
        switch (a.mode) {
            case kModeNative: row_phase_kernel<T, VK, kModeNative><<<grid, kBlock, 0, s>>>(a); break;
            case kModeTree: row_phase_kernel<T, VK, kModeTree><<<grid, kBlock, 0, s>>>(a); break;
            default: row_phase_kernel<T, VK, kModeExact><<<grid, kBlock, 0, s>>>(a);
        }
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_dtype(const RhsArgs& a, cudaStream_t s, int phases) {
#define ND_CASE(VK, EK) \
    if (a.vertex_kind == VK && a.edge_kind == EK) return launch_typed<T, VK, EK>(a, s, phases);
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

cudaError_t launch_rhs_edge(int dtype, const RhsArgs& a, cudaStream_t s, int phases) {
    return dtype == ND_F64 ? launch_dtype<double>(a, s, phases) : launch_dtype<float>(a, s, phases);
}

}  // namespace nd
