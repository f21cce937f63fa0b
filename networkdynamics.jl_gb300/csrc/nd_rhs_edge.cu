// Two-phase (edge-centric) network right-hand side, for canonical edge lists.
//
// The reference evaluates every edge once (edge g, src/coreloop.jl:76-78), stores both
// outputs in the output buffer (AntiSymmetric: y_src = -y_dst,
// src/component_functions.jl:117-127) and then adds the buffer into each vertex in
// buffer order (SequentialAggregator, src/aggregators.jl:140-151).  The two phases here
// do the same on the GPU:
//   E  one thread per pair of edges, in edge order: y_e = g(u_src, u_dst, p_e), written to
//      y and, grouped by destination, to ybkt (EdgeLayout in nd_internal.h);
//   R  one thread per row: the row's destination-side values (edges (s, v), s < v, in
//      ascending edge id) followed by the negated values of its own source block, which
//      is exactly the order of the vertex's entries in the reference's output buffer, then
//      vertex f.  Rows of degree above kMediumMaxDeg run in the heavy-row kernel of the
//      fused path (nd_rhs.cu) on a side stream.
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
// staging slot, parameter, y) move as 4-, 8- or 16-byte vectors.  The values bound for
// ybkt go to shared memory first, in (bucket, edge) order, and leave the block as one
// contiguous run per bucket: written one by one, the scattered 8-byte stores reached L2
// as separate partial-sector requests and took more than half of the phase's time.
template <typename T, int VK, int EK>
__global__ void __launch_bounds__(kBlock) edge_phase_kernel(RhsArgs a) {
    using P2 = typename Pair<T>::type;
    constexpr int DV = VertexDims<VK>::dim;
    __shared__ T stage[kEdgeChunk];
    __shared__ uint16_t rstart[kBuckets + 1];
    __shared__ int32_t rbase[kBuckets];
    const T* __restrict__ u = static_cast<const T*>(a.u);
    const T* __restrict__ pe = static_cast<const T*>(a.p) + a.nv * VertexDims<VK>::pdim;
    T* __restrict__ y = static_cast<T*>(a.y);
    T* __restrict__ ybkt = static_cast<T*>(a.ybkt);
    const uint64_t keep = policy_evict_last(), stream = policy_evict_first();
    const int64_t chunk = blockIdx.x;
    const int64_t e0 = chunk * kEdgeChunk;  // even: kEdgeChunk is
    const int64_t e1 = min(e0 + (int64_t)kEdgeChunk, a.ne);
    if (threadIdx.x <= kBuckets) rstart[threadIdx.x] = __ldg(a.run_start + chunk * (kBuckets + 1) + threadIdx.x);
    if (threadIdx.x < kBuckets) rbase[threadIdx.x] = __ldg(a.run_base + chunk * kBuckets + threadIdx.x);
    // the parameter block starts after nv * pdim vertex parameters: pairs of it are
    // vector-aligned only when that offset is even
    const bool wvec = EK == ND_E_DIFFUSION_UNIT || (reinterpret_cast<uintptr_t>(pe) % sizeof(P2)) == 0;
    const int64_t npair = (e1 - e0) >> 1;
#pragma unroll 4
    for (int64_t k = threadIdx.x; k < npair; k += kBlock) {
        const int64_t e = e0 + 2 * k;
        const int2 s = ld_hint(reinterpret_cast<const int2*>(a.esrc + e), stream);
        const int2 d = ld_hint(reinterpret_cast<const int2*>(a.edst + e), stream);
        const uint32_t ls = ld_hint(reinterpret_cast<const uint32_t*>(a.lslot + e), stream);
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
        // the outputs stream through L2 ahead of the row phase: evict them first so the
        // gathered u stays resident
        st_hint(reinterpret_cast<P2*>(y + e), yv, stream);
        stage[ls & 0xffffu] = yv.x;
        stage[ls >> 16] = yv.y;
    }
    if (((e1 - e0) & 1) && threadIdx.x == 0) {  // odd tail of the last chunk
        const int64_t e = e1 - 1;
        const int32_t s = ld_hint(a.esrc + e, stream);
        const int32_t d = ld_hint(a.edst + e, stream);
        const T w = edge_param<T, EK>(pe, (int32_t)e, stream);
        const T yv = edge_g_w<T, EK>(ld_hint(u + (int64_t)s * DV, keep), ld_hint(u + (int64_t)d * DV, keep), w);
        y[e] = yv;
        stage[a.lslot[e]] = yv;
    }
    __syncthreads();
    // one bucket run per warp step, its lanes writing consecutive ybkt positions
    const int lane = threadIdx.x & 31;
    for (int b = threadIdx.x >> 5; b < kBuckets; b += kWarpsPerBlock) {
        const int s0 = rstart[b], n = rstart[b + 1] - s0;
        T* __restrict__ dst = ybkt + rbase[b];
        for (int j = lane; j < n; j += 32) st_hint(dst + j, stage[s0 + j], stream);
    }
}

// ---- FP32 rows of many terms: a warp per row ----------------------------------------------
// FP32 rows carry no order to keep: the lanes of a warp add every 32nd term of the row with
// Kahan compensation and a butterfly joins the lane sums (as the FP32 heavy rows and the
// batched path's long FP32 rows do).  Positions and source blocks load coalesced across the
// lanes.  Used for every row of a dense network and for the medium rows of any other.
template <int VK>
__device__ __forceinline__ void warp_row_f32(const RhsArgs& a, int64_t slot) {
    using A = Arith<float>;
    const int lane = threadIdx.x & 31;
    const float* __restrict__ y = static_cast<const float*>(a.y);
    const float* __restrict__ ybkt = static_cast<const float*>(a.ybkt);
    const uint64_t stream = policy_evict_first();
    const int4 rm = ld_hint(a.rmeta + slot, stream);
    const int nd = rm.w & 0xffff;
    const int n = nd + (int)((uint32_t)rm.w >> 16);
    float acc = 0.f, comp = 0.f;
    for (int j = lane; j < n; j += 32) {
        const float term = j < nd ? ld_hint(ybkt + ld_hint(a.locp + rm.y + j, stream), stream)
                                  : -ld_hint(y + (uint32_t)rm.z + (uint32_t)(j - nd), stream);
        const float yk = A::sub(term, comp);
        const float s2 = A::add(acc, yk);
        comp = A::sub(A::sub(s2, acc), yk);
        acc = s2;
    }
    acc = A::sub(acc, comp);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc = A::add(acc, __shfl_xor_sync(kFull, acc, off));
    if (lane == 0)
        vertex_f<float, VK>(static_cast<float*>(a.du), static_cast<const float*>(a.u), static_cast<const float*>(a.p),
                            rm.x, acc);
}

template <int VK>
__global__ void __launch_bounds__(kBlock) dense_warp_row_kernel(RhsArgs a) {
    const int64_t slot = (int64_t)a.n_heavy + (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (slot < a.nv) warp_row_f32<VK>(a, slot);  // warp-uniform
}

// ---- phase R: a thread per row, reading the row's terms from global memory -------------------
// Rows of degree up to kMediumMaxDeg, in slot order: medium rows sorted by degree over all
// of them, light rows sorted by degree inside runs of consecutive vertices, so the 32 rows
// of a warp have nearly equal length and every lane of each add is busy.  Loads are issued
// kBatch terms ahead of the adds; nothing is staged in shared memory.
//   FP64  the sequential sum in the reference's order: destination-side terms added,
//         source-side terms subtracted (x - y == x + (-y), IEEE 754), the reference's zero
//         start folded into the first term (0 + t is t, and both zeros give +0);
//   FP32  the same order with Kahan compensation on rows longer than kLightMaxDeg.
template <typename T, int VK>
// 5 blocks per SM (registers capped at 48) in both precisions.  A/B on BA(1e7, 4), FP64:
// 327 µs against 349 µs at the 64 registers the kernel takes uncapped (4 blocks), 374-390 µs
// with 8-term batches at 5-6 blocks, 351 µs with 16-term batches at 4; FP32: 252 µs against
// 309-451 µs with 8-term batches at 6-8 blocks.
__device__ __forceinline__ void row_thread(const RhsArgs& a, int64_t slot) {
    using A = Arith<T>;
    constexpr int kBatch = 12;
    const T* __restrict__ y = static_cast<const T*>(a.y);
    const T* __restrict__ ybkt = static_cast<const T*>(a.ybkt);
    const uint64_t stream = policy_evict_first();
    const int4 rm = ld_hint(a.rmeta + slot, stream);
    const int64_t v = rm.x;
    const int32_t lp = rm.y;  // multiple of 4
    const uint32_t sp = (uint32_t)rm.z;
    const int nd = rm.w & 0xffff;
    const int ns = (int)((uint32_t)rm.w >> 16);
    const bool kahan = sizeof(T) == 4 && nd + ns > kLightMaxDeg;
    T acc = T(0), comp = T(0);
    auto add = [&](T t, bool src) {
        if constexpr (sizeof(T) == 8) {
            acc = src ? __dsub_rn(acc, t) : __dadd_rn(acc, t);
        } else {
            const T term = src ? -t : t;
            if (kahan) {
                const T yk = A::sub(term, comp);
                const T s2 = A::add(acc, yk);
                comp = A::sub(A::sub(s2, acc), yk);
                acc = s2;
            } else {
                acc = A::add(acc, term);
            }
        }
    };
    // The adds of a batch stop at the longest remaining run in the warp (a warp-uniform
    // bound), so a warp issues no add for batch slots that none of its rows has.
    for (int j0 = 0; j0 < nd; j0 += kBatch) {
        // the batch's positions as 16-byte vectors (the row's run starts on a multiple of 4)
        int li[kBatch];
#pragma unroll
        for (int k4 = 0; k4 < kBatch / 4; ++k4) {
            const int4 q = j0 + 4 * k4 < nd ? ld_hint(reinterpret_cast<const int4*>(a.locp + lp + j0) + k4, stream)
                                            : int4{0, 0, 0, 0};
            li[4 * k4] = q.x;
            li[4 * k4 + 1] = q.y;
            li[4 * k4 + 2] = q.z;
            li[4 * k4 + 3] = q.w;
        }
        T t[kBatch];
#pragma unroll
        for (int k = 0; k < kBatch; ++k) t[k] = j0 + k < nd ? ld_hint(ybkt + li[k], stream) : T(0);
        const int lim = __reduce_max_sync(__activemask(), (unsigned)min(kBatch, nd - j0));
#pragma unroll
        for (int k = 0; k < kBatch; ++k) {
            if (k >= lim) break;
            if (j0 + k >= nd) continue;
            if (sizeof(T) == 8 && k == 0 && j0 == 0) {
                const double t0 = (double)t[0];
                acc = (T)((__double_as_longlong(t0) << 1) == 0 ? 0.0 : t0);
            } else {
                add(t[k], false);
            }
        }
    }
    for (int j0 = 0; j0 < ns; j0 += kBatch) {
        // the source block's values as aligned pairs (y has two padding entries at its end;
        // a pair may hold the neighbouring row's value, which is not used)
        using P2 = typename Pair<T>::type;
        const uint32_t b0 = sp + (uint32_t)j0, off = b0 & 1u;
        const P2* __restrict__ yp = reinterpret_cast<const P2*>(y + (b0 - off));
        const int avail = (int)off + ns - j0;  // entries from the pair base to the block end
        T e[kBatch + 2];
#pragma unroll
        for (int k2 = 0; k2 < kBatch / 2 + 1; ++k2) {
            const P2 v = 2 * k2 < avail ? ld_hint(yp + k2, stream) : P2{T(0), T(0)};
            e[2 * k2] = v.x;
            e[2 * k2 + 1] = v.y;
        }
        T t[kBatch];
#pragma unroll
        for (int k = 0; k < kBatch; ++k) t[k] = off ? e[k + 1] : e[k];
        const int lim = __reduce_max_sync(__activemask(), (unsigned)min(kBatch, ns - j0));
#pragma unroll
        for (int k = 0; k < kBatch; ++k) {
            if (k >= lim) break;
            if (j0 + k < ns) add(t[k], true);
        }
    }
    if constexpr (sizeof(T) == 4) acc = A::sub(acc, comp);
    vertex_f<T, VK>(static_cast<T*>(a.du), static_cast<const T*>(a.u), static_cast<const T*>(a.p), v, acc);
}

template <typename T, int VK>
__global__ void __launch_bounds__(kBlock, 5) row_phase_kernel(RhsArgs a) {
    const int64_t slot = (int64_t)a.n_heavy + (int64_t)blockIdx.x * kBlock + threadIdx.x;
    if (slot < a.nv) row_thread<T, VK>(a, slot);
}

// FP32 row phase when some rows have at least kWarpRowMinF32 terms: those rows (the first
// n_warp_f32 medium slots, sorted by degree) take a warp each in the first blocks, the rest a
// thread each, in one launch.  Per thread, such a row is a chain of one memory round trip per
// 12 terms that outlasts every other row: on BA(1e5, 2) swing (rows up to 935 terms) the row
// phase took 57.8 µs with a thread per row and 9.9 µs with a warp per medium row.  Shorter
// rows keep a thread: giving all 170K medium rows of BA(1e7, 4) a warp each (most have 33 to
// 100 terms) made its row phase 302 µs against 250.
template <int VK>
__global__ void __launch_bounds__(kBlock, 5) row_phase_f32_kernel(RhsArgs a) {
    const int64_t nb_w = ((int64_t)a.n_warp_f32 + kWarpsPerBlock - 1) / kWarpsPerBlock;
    if ((int64_t)blockIdx.x < nb_w) {
        const int64_t r = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
        if (r < a.n_warp_f32) warp_row_f32<VK>(a, a.n_heavy + r);  // warp-uniform
        return;
    }
    const int64_t slot = (int64_t)a.n_heavy + a.n_warp_f32 + ((int64_t)blockIdx.x - nb_w) * kBlock + threadIdx.x;
    if (slot < a.nv) row_thread<float, VK>(a, slot);
}

// ---- phase R on dense networks: rows of hundreds of terms ------------------------------------
// When the medium rows carry most of the incidences (dense graphs such as the reference's
// diffusion benchmark on WS(3000, 1500)), there are few rows and each is a long serial chain:
// 3000 rows fill 94 warps, and a row waits one memory round trip per batch of terms.  Here a
// thread still sums one row in the same order (the same bits), but its terms come in batches
// of 32, with the values of the next batch and the destination-side positions of the one
// after that in flight while the current batch is added, and one-warp blocks spread the few
// warps over as many SMs as there are warps.
constexpr int kDenseBlock = 32;

// Sequential sum of n terms in batches of KB, the next batch's loads in flight while the
// current one is added.  load(j0, t) fills t with terms j0 .. j0 + KB - 1 (0 past the end);
// add(t) adds one term.  The adds of a batch stop at the longest remaining run in the warp.
template <typename T, int KB, typename Load, typename Add>
__device__ __forceinline__ void pipelined_sum(int n, Load&& load, Add&& add) {
    T cur[KB], nxt[KB];
    load(0, cur);
    for (int j0 = 0; j0 < n; j0 += KB) {
        load(j0 + KB, nxt);
        const int lim = __reduce_max_sync(__activemask(), (unsigned)min(KB, n - j0));
#pragma unroll
        for (int k = 0; k < KB; ++k) {
            if (k >= lim) break;
            if (j0 + k < n) add(j0 + k, cur[k]);
        }
#pragma unroll
        for (int k = 0; k < KB; ++k) cur[k] = nxt[k];
    }
}

template <typename T, int VK>
__global__ void __launch_bounds__(kDenseBlock) dense_row_kernel(RhsArgs a) {
    using A = Arith<T>;
    constexpr int KB = 32;
    const int64_t slot = (int64_t)a.n_heavy + (int64_t)blockIdx.x * kDenseBlock + threadIdx.x;
    if (slot >= a.nv) return;
    const T* __restrict__ y = static_cast<const T*>(a.y);
    const T* __restrict__ ybkt = static_cast<const T*>(a.ybkt);
    const uint64_t stream = policy_evict_first();
    const int4 rm = ld_hint(a.rmeta + slot, stream);
    const int64_t v = rm.x;
    const int32_t lp = rm.y;  // multiple of 4
    const uint32_t sp = (uint32_t)rm.z;
    const int nd = rm.w & 0xffff;
    const int ns = (int)((uint32_t)rm.w >> 16);
    const bool kahan = sizeof(T) == 4 && nd + ns > kLightMaxDeg;
    T acc = T(0), comp = T(0);
    auto add = [&](T term) {
        if (kahan) {
            const T yk = A::sub(term, comp);
            const T s2 = A::add(acc, yk);
            comp = A::sub(A::sub(s2, acc), yk);
            acc = s2;
        } else {
            acc = A::add(acc, term);
        }
    };
    // destination side: positions in locp, values in ybkt
    {
        int pos[KB];
        auto load_pos = [&](int j0) {
#pragma unroll
            for (int k4 = 0; k4 < KB / 4; ++k4) {
                const int4 q = j0 + 4 * k4 < nd
                                   ? ld_hint(reinterpret_cast<const int4*>(a.locp + lp + j0) + k4, stream)
                                   : int4{0, 0, 0, 0};
                pos[4 * k4] = q.x;
                pos[4 * k4 + 1] = q.y;
                pos[4 * k4 + 2] = q.z;
                pos[4 * k4 + 3] = q.w;
            }
        };
        load_pos(0);
        pipelined_sum<T, KB>(
            nd,
            [&](int j0, T (&t)[KB]) {
#pragma unroll
                for (int k = 0; k < KB; ++k) t[k] = j0 + k < nd ? ld_hint(ybkt + pos[k], stream) : T(0);
                load_pos(j0 + KB);  // the positions of the batch after
            },
            [&](int j, T t) {
                if constexpr (sizeof(T) == 8) {
                    if (j == 0) acc = (T)((__double_as_longlong((double)t) << 1) == 0 ? 0.0 : (double)t);
                    else acc = __dadd_rn(acc, t);
                } else {
                    add(t);
                }
            });
    }
    // source side: the row's own block of y
    pipelined_sum<T, KB>(
        ns,
        [&](int j0, T (&t)[KB]) {
#pragma unroll
            for (int k = 0; k < KB; ++k) t[k] = j0 + k < ns ? ld_hint(y + sp + (uint32_t)(j0 + k), stream) : T(0);
        },
        [&](int, T t) {
            if constexpr (sizeof(T) == 8) acc = __dsub_rn(acc, t);
            else add(-t);
        });
    if constexpr (sizeof(T) == 4) acc = A::sub(acc, comp);
    vertex_f<T, VK>(static_cast<T*>(a.du), static_cast<const T*>(a.u), static_cast<const T*>(a.p), v, acc);
}

template <typename T, int VK, int EK>
cudaError_t launch_typed(const RhsArgs& a, cudaStream_t s, int phases) {
    if ((phases & kPhaseEdge) && a.n_chunks > 0)
        edge_phase_kernel<T, VK, EK><<<(unsigned)a.n_chunks, kBlock, 0, s>>>(a);
    // rows below the heavy ones; every summation order adds them sequentially
    const int64_t rows = a.nv - a.n_heavy;
    if (!(phases & kPhaseRow) || rows <= 0) return cudaGetLastError();
    if (a.dense_rows && sizeof(T) == 4)
        dense_warp_row_kernel<VK><<<(unsigned)((rows + kWarpsPerBlock - 1) / kWarpsPerBlock), kBlock, 0, s>>>(a);
    else if (a.dense_rows)
        dense_row_kernel<T, VK><<<(unsigned)((rows + kDenseBlock - 1) / kDenseBlock), kDenseBlock, 0, s>>>(a);
    else if (sizeof(T) == 4 && a.n_warp_f32 > 0)
        row_phase_f32_kernel<VK><<<(unsigned)((a.n_warp_f32 + kWarpsPerBlock - 1) / kWarpsPerBlock +
                                              (rows - a.n_warp_f32 + kBlock - 1) / kBlock),
                                   kBlock, 0, s>>>(a);
    else
        row_phase_kernel<T, VK><<<(unsigned)((rows + kBlock - 1) / kBlock), kBlock, 0, s>>>(a);
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
