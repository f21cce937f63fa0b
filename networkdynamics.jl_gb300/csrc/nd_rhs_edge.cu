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
    static constexpr int kBytes = kWindowIncidences * (int)sizeof(T) + 4 * kWindow * 4 + kWindowIncidences;
};

template <typename T>
__device__ __forceinline__ T negate(T x) {
    if constexpr (sizeof(T) == 8) return __longlong_as_double(__double_as_longlong(x) ^ (1ll << 63));
    else return __int_as_float(__float_as_int(x) ^ (int)0x80000000);
}

// ---- phase E -------------------------------------------------------------------------------
template <typename T>
struct Pair;
template <>
struct Pair<double> {
    using type = double2;
};
template <>
struct Pair<float> {
    using type = float2;
};

// A thread evaluates two consecutive edges per step, so the in-order streams (src, dst,
// bucket slot, parameter, y) move as 8- or 16-byte vectors.
template <typename T, int VK, int EK>
__global__ void __launch_bounds__(kBlock) edge_phase_kernel(RhsArgs a) {
    using P2 = typename Pair<T>::type;
    constexpr int DV = VertexDims<VK>::dim;
    const T* __restrict__ u = static_cast<const T*>(a.u);
    const T* __restrict__ pe = static_cast<const T*>(a.p) + a.nv * VertexDims<VK>::pdim;
    T* __restrict__ y = static_cast<T*>(a.y);
    T* __restrict__ ybkt = static_cast<T*>(a.ybkt);
    const uint64_t keep = policy_evict_last(), stream = policy_evict_first();
    const int64_t e0 = (int64_t)blockIdx.x * kEdgeChunk;  // even: kEdgeChunk is
    const int64_t e1 = min(e0 + (int64_t)kEdgeChunk, a.ne);
    // the parameter block starts after nv * pdim vertex parameters: pairs of it are
    // vector-aligned only when that offset is even
    const bool wvec = EK == ND_E_DIFFUSION_UNIT || (reinterpret_cast<uintptr_t>(pe) % sizeof(P2)) == 0;
    const int64_t npair = (e1 - e0) >> 1;
#pragma unroll 2
    for (int64_t k = threadIdx.x; k < npair; k += kBlock) {
        const int64_t e = e0 + 2 * k;
        const int2 s = ld_hint(reinterpret_cast<const int2*>(a.esrc + e), stream);
        const int2 d = ld_hint(reinterpret_cast<const int2*>(a.edst + e), stream);
        const int2 q = ld_hint(reinterpret_cast<const int2*>(a.q + e), stream);
        T w0, w1;
        if constexpr (EK == ND_E_DIFFUSION_UNIT) {
            w0 = w1 = T(0);
        } else if (wvec) {
            const P2 w = ld_hint(reinterpret_cast<const P2*>(pe + e), stream);
            w0 = w.x;
            w1 = w.y;
        } else {
            w0 = ld_hint(pe + e, stream);
            w1 = ld_hint(pe + e + 1, stream);
        }
        const T us0 = ld_hint(u + (int64_t)s.x * DV, keep);
        const T us1 = ld_hint(u + (int64_t)s.y * DV, keep);
        const T ud0 = ld_hint(u + (int64_t)d.x * DV, keep);
        const T ud1 = ld_hint(u + (int64_t)d.y * DV, keep);
        P2 yv;
        yv.x = edge_g_w<T, EK>(us0, ud0, w0);
        yv.y = edge_g_w<T, EK>(us1, ud1, w1);
        *reinterpret_cast<P2*>(y + e) = yv;
        ybkt[q.x] = yv.x;
        ybkt[q.y] = yv.y;
    }
    if (((e1 - e0) & 1) && threadIdx.x == 0) {  // odd tail of the last chunk
        const int64_t e = e1 - 1;
        const int32_t s = ld_hint(a.esrc + e, stream);
        const int32_t d = ld_hint(a.edst + e, stream);
        const T w = edge_param<T, EK>(pe, (int32_t)e, stream);
        const T yv = edge_g_w<T, EK>(ld_hint(u + (int64_t)s * DV, keep), ld_hint(u + (int64_t)d * DV, keep), w);
        y[e] = yv;
        ybkt[ld_hint(a.q + e, stream)] = yv;
    }
}

// Term j (0-based, in row order) of a row whose destination-side entries start at dp
// (nd of them) and whose source block starts at sp.  kNeg: the source-side terms come
// negated (their value in the reference's output buffer); without it they come as stored
// and the caller subtracts them.
template <typename T, bool kNeg = true>
__device__ __forceinline__ T row_term(const RhsArgs& a, uint32_t dp, int nd, uint32_t sp, int j, uint64_t pol) {
    const T* __restrict__ y = static_cast<const T*>(a.y);
    const T* __restrict__ ybkt = static_cast<const T*>(a.ybkt);
    if (j < nd) return ld_hint(ybkt + ld_hint(a.loc + dp + j, pol), pol);
    const T v = ld_hint(y + sp + (j - nd), pol);
    if constexpr (kNeg) return negate(v);
    else return v;
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
    // FP64 stages the source-side terms un-negated: the row adds its destination-side terms
    // and subtracts its source-side ones, x - y being x + (-y) exactly (IEEE 754), so no
    // separate negation runs on the scarce FP64 pipe.
    constexpr bool kNegTerms = sizeof(T) != 8;
#pragma unroll 4
    for (int k = tid; k < n; k += kBlock) {
        const int t = s_owner[k];
        s_term[k] = row_term<T, kNegTerms>(a, s_dp[t], s_nd[t], s_sp[t], k - s_start[t], stream);
    }
    __syncthreads();
    if (!has_row) return;
    T acc = T(0);
    if constexpr (sizeof(T) == 8) {
        const int mid = beg + s_nd[tid];
        int j = beg;
        if (mid > beg) {
            // the reference starts from 0: 0 + t is t, except that both zeros give +0
            const double t = s_term[beg];
            acc = (__double_as_longlong(t) << 1) == 0 ? 0.0 : t;
            j = beg + 1;
        }
        for (; j < mid; ++j) acc = __dadd_rn(acc, s_term[j]);
        for (; j < end; ++j) acc = __dsub_rn(acc, s_term[j]);
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

// ---- phase R: medium rows, a thread per row reading its terms from global memory -------------
// Medium rows (degree kLightMaxDeg+1 .. kMediumMaxDeg) are sorted by degree over all of
// them, so the 32 rows of a warp have nearly equal length and every lane of each add is
// busy; loads are issued kBatch terms ahead of the adds.
template <typename T, int VK>
__device__ __forceinline__ void medium_rows_r(const RhsArgs& a, int blk) {
    using A = Arith<T>;
    constexpr int kBatch = 8;
    const int slot = a.n_heavy + blk * kBlock + (int)threadIdx.x;
    if (slot >= a.n_heavy + a.n_medium) return;
    const T* __restrict__ y = static_cast<const T*>(a.y);
    const T* __restrict__ ybkt = static_cast<const T*>(a.ybkt);
    const uint64_t stream = policy_evict_first();
    const int64_t v = __ldg(a.slot_vertex + slot);
    const uint32_t dp = __ldg(a.dptr + v), sp = __ldg(a.sptr + v);
    const int nd = (int)(__ldg(a.dptr + v + 1) - dp);
    const int ns = (int)(__ldg(a.sptr + v + 1) - sp);
    T acc = T(0), comp = T(0);
    // F32: compensated sum of the buffer values (source side negated); FP64: the
    // sequential sum, source-side terms subtracted (x - y == x + (-y))
    auto add = [&](T t, bool src) {
        if constexpr (sizeof(T) == 8) {
            acc = src ? __dsub_rn(acc, t) : __dadd_rn(acc, t);
        } else {
            const T yk = A::sub(src ? -t : t, comp);
            const T s2 = A::add(acc, yk);
            comp = A::sub(A::sub(s2, acc), yk);
            acc = s2;
        }
    };
    for (int j0 = 0; j0 < nd; j0 += kBatch) {
        T t[kBatch];
#pragma unroll
        for (int k = 0; k < kBatch; ++k)
            t[k] = j0 + k < nd ? ld_hint(ybkt + ld_hint(a.loc + dp + j0 + k, stream), stream) : T(0);
#pragma unroll
        for (int k = 0; k < kBatch; ++k)
            if (j0 + k < nd) add(t[k], false);
    }
    for (int j0 = 0; j0 < ns; j0 += kBatch) {
        T t[kBatch];
#pragma unroll
        for (int k = 0; k < kBatch; ++k) t[k] = j0 + k < ns ? ld_hint(y + sp + j0 + k, stream) : T(0);
#pragma unroll
        for (int k = 0; k < kBatch; ++k)
            if (j0 + k < ns) add(t[k], true);
    }
    if constexpr (sizeof(T) == 4) acc = A::sub(acc, comp);
    vertex_f<T, VK>(static_cast<T*>(a.du), static_cast<const T*>(a.u), static_cast<const T*>(a.p), v, acc);
}

// Blocks: [medium rows, kBlock per block] [light windows].  Heavy rows are always launched
// separately (launch_rhs with heavy_only).
template <typename T, int VK, int MODE>
__global__ void __launch_bounds__(kBlock, 8) row_phase_kernel(RhsArgs a) {
    __shared__ __align__(16) unsigned char smem[SmemR<T>::kBytes];
    const int nm = (a.n_medium + kBlock - 1) / kBlock;
    const int b = blockIdx.x;
    if (b < nm) medium_rows_r<T, VK>(a, b);
    else window_r<T, VK, MODE>(a, a.n_medium_windows + (b - nm), smem);
}

template <typename T, int VK, int EK>
cudaError_t launch_typed(const RhsArgs& a, cudaStream_t s, int phases) {
    if ((phases & kPhaseEdge) && a.n_chunks > 0)
        edge_phase_kernel<T, VK, EK><<<(unsigned)a.n_chunks, kBlock, 0, s>>>(a);
    const int grid = (a.n_medium + kBlock - 1) / kBlock + (a.n_windows - a.n_medium_windows);
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
