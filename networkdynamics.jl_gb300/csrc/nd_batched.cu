// Batched (heterogeneous) networks: several vertex and edge batches, ODE edges and the
// Symmetric / Directed / Fiducial output wrappers.
//
// The reference builds one batch per group of identical components
// (src/construction.jl:155-195), lays the flat vectors out batch by batch
// (src/network_structure.jl:224-258) and runs its core loop per batch
// (src/coreloop.jl:111-155): vertex g, edge g / f, aggregation in output-buffer order
// (SequentialAggregator, src/aggregators.jl:140-151), vertex f.  The GPU path needs two
// launches for any number of batches:
//   edges  one thread per edge position: the batch is found in a small table, the edge
//          function of its kind runs (static g with its coupling, or the ODE edge's f,
//          writing du of the edge states, and its StateMask outputs), and the pair
//          (y_src, y_dst) is stored as one vector at y2[2k], the reference's output
//          buffer order;
//   rows   every vertex sums the y2 entries of its terms in ascending index order (the
//          sequential aggregation order), then runs the vertex f of its batch.  Long rows
//          take a warp each (FP64: the windowed exact scan, the same bits as the sequential
//          sum), shorter rows a thread each, sorted by degree so the lanes of a warp do
//          equal work.
// Homogeneous networks of the static AntiSymmetric kinds keep the two-phase kernels of
// nd_rhs_edge.cu; this path covers everything else in the library.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "nd_components.cuh"
#include "nd_exact.cuh"
#include "nd_internal.h"
#include "nd_scan.cuh"

namespace nd {

namespace {

using namespace dev;

template <typename T>
struct Vec2;
template <>
struct Vec2<double> {
    using type = double2;
};
template <>
struct Vec2<float> {
    using type = float2;
};

struct BatchedKArgs {
    void* du;
    const void* u;
    const void* p;
    int64_t nv, ne, n_warp_rows;
    BatchTableDev vb, eb;  // the batch tables (device arrays)
    const int2* eu;
    const uint32_t* tptr;
    const int32_t* tidx;
    const int32_t* slot_vpos;
    void* y2;
    int32_t mode;
};

template <typename T>
__device__ __forceinline__ T static_edge_g(int kind, T vs, T vd, T w) {
    if (kind == ND_E_DIFFUSION) return edge_g_w<T, ND_E_DIFFUSION>(vs, vd, w);
    if (kind == ND_E_DIFFUSION_UNIT) return edge_g_w<T, ND_E_DIFFUSION_UNIT>(vs, vd, w);
    return edge_g_w<T, ND_E_KURAMOTO>(vs, vd, w);
}

template <typename T>
__global__ void __launch_bounds__(kBlock) batched_edge_kernel(BatchedKArgs a) {
    using A = Arith<T>;
    using V2 = typename Vec2<T>::type;
    const T* __restrict__ u = static_cast<const T*>(a.u);
    const T* __restrict__ p = static_cast<const T*>(a.p);
    T* __restrict__ du = static_cast<T*>(a.du);
    V2* __restrict__ y2 = static_cast<V2*>(a.y2);
    for (int64_t k = (int64_t)blockIdx.x * kBlock + threadIdx.x; k < a.ne; k += (int64_t)gridDim.x * kBlock) {
        const int b = find_batch(a.eb, k);
        const int kind = __ldg(a.eb.kind + b);
        const int64_t r = k - __ldg(a.eb.pos0 + b);
        const int2 uv = __ldg(a.eu + k);
        const T vs = __ldg(u + uv.x), vd = __ldg(u + uv.y);  // vertex outputs: StateMask(1)
        V2 y;
        if (kind == ND_E_DIFFUSION_ODE || kind == ND_E_DIFFUSION_ODE_FIXED) {
            const int64_t s = __ldg(a.eb.s0 + b) + 2 * r;
            const T e1 = __ldg(u + s), e2 = __ldg(u + s + 1);
            const T rate = kind == ND_E_DIFFUSION_ODE ? A::div(T(1), __ldg(p + __ldg(a.eb.p0 + b) + r)) : T(100);
            T d1, d2;
            ode_edge_f<T>(rate, vs, vd, e1, e2, d1, d2);
            du[s] = d1;
            du[s + 1] = d2;
            y.x = e2;  // Fiducial(dst=1:1, src=2:2): y_src = e2, y_dst = e1
            y.y = e1;
        } else {
            const T w = kind == ND_E_DIFFUSION_UNIT ? T(0) : __ldg(p + __ldg(a.eb.p0 + b) + r);
            const T yd = static_edge_g<T>(kind, vs, vd, w);
            const int c = __ldg(a.eb.coupling + b);
            // AntiSymmetric and the two-sided diffusionedge_fid!: y_src = -y_dst (a sign
            // flip); Symmetric: y_src = y_dst; Directed: y_src = +0 (fill! with zero)
            y.x = c == ND_SYMMETRIC ? yd : (c == ND_DIRECTED ? T(0) : -yd);
            y.y = yd;
        }
        y2[k] = y;
    }
}

// Rows with at least this many terms take a warp each; shorter rows a thread each.  FP64
// keeps the sequential sum, whose running sum changes binade often on rows of mixed-sign
// terms; there a thread per row (32 rows in step per warp) beats the warp scan up to the
// length at which the homogeneous path also moves rows to the exact scan.  FP32 rows are
// compensated sums with no order to keep, which a warp splits across its lanes.
constexpr int kWarpRowMinDegF64 = kMediumMaxDeg + 1;
constexpr int kWarpRowMinDegF32 = 2 * kLightMaxDeg + 1;
// Terms per warp tile in shared memory (FP64 warp rows): 16 per lane.
constexpr int kWarpTile = 512;

// Sum of a row's n terms (y2 indices idx[0..n)) by one thread, in order.  The terms come in
// batches of kB; the loads of batch k + 1 are issued before the adds of batch k, so on long
// rows the gathers overlap the chain of dependent adds.  The adds of a batch stop at the
// longest remaining row in the warp (a warp-uniform bound), so no add is issued for batch
// slots no lane has.
//   FP64  the sequential sum with the reference's zero start folded into the first term
//         (0 + t is t; -0 gives +0);
//   FP32  the same order, Kahan-compensated on rows longer than kLightMaxDeg.
template <typename T>
__device__ __forceinline__ T thread_row_sum(const T* __restrict__ y2, const int32_t* __restrict__ idx, int n) {
    using A = Arith<T>;
    constexpr int kB = 12;
    const bool kahan = sizeof(T) == 4 && n > kLightMaxDeg;
    T acc = T(0), comp = T(0);
    T cur[kB], nxt[kB];
#pragma unroll
    for (int k = 0; k < kB; ++k) cur[k] = k < n ? __ldg(y2 + __ldg(idx + k)) : T(0);
    for (int j0 = 0; j0 < n; j0 += kB) {
        const int j1 = j0 + kB;
#pragma unroll
        for (int k = 0; k < kB; ++k) nxt[k] = j1 + k < n ? __ldg(y2 + __ldg(idx + j1 + k)) : T(0);
        const int lim = __reduce_max_sync(__activemask(), (unsigned)min(kB, n - j0));
#pragma unroll
        for (int k = 0; k < kB; ++k) {
            if (k >= lim) break;
            if (j0 + k >= n) continue;
            if (sizeof(T) == 8 && j0 + k == 0) {
                const double t0 = (double)cur[0];
                acc = (T)((__double_as_longlong(t0) << 1) == 0 ? 0.0 : t0);
            } else if (kahan) {
                const T yk = A::sub(cur[k], comp);
                const T s2 = A::add(acc, yk);
                comp = A::sub(A::sub(s2, acc), yk);
                acc = s2;
            } else {
                acc = A::add(acc, cur[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < kB; ++k) cur[k] = nxt[k];
    }
    return sizeof(T) == 4 ? A::sub(acc, comp) : acc;
}

// The same sum for the long thread rows of dense networks (FP64): batches of 32 terms, the
// next batch's values and the term indices of the one after that in flight while the current
// batch is added.  Dense graphs have few rows, each a long serial chain, so every exposed
// round trip lengthens the whole row phase; the extra registers cost no occupancy there.
template <typename T>
__device__ __forceinline__ T thread_row_sum_deep(const T* __restrict__ y2, const int32_t* __restrict__ idx, int n) {
    using A = Arith<T>;
    constexpr int kB = 32;
    const bool kahan = sizeof(T) == 4 && n > kLightMaxDeg;
    T acc = T(0), comp = T(0);
    int ia[kB], ib[kB];
    T cur[kB], nxt[kB];
    auto load_idx = [&](int j0, int (&ix)[kB]) {
#pragma unroll
        for (int k = 0; k < kB; ++k) ix[k] = j0 + k < n ? __ldg(idx + j0 + k) : 0;
    };
    auto load_val = [&](int j0, const int (&ix)[kB], T (&t)[kB]) {
#pragma unroll
        for (int k = 0; k < kB; ++k) t[k] = j0 + k < n ? __ldg(y2 + ix[k]) : T(0);
    };
    load_idx(0, ia);
    load_val(0, ia, cur);
    load_idx(kB, ib);
    for (int j0 = 0; j0 < n; j0 += kB) {
        load_val(j0 + kB, ib, nxt);
        load_idx(j0 + 2 * kB, ia);
        const int lim = __reduce_max_sync(__activemask(), (unsigned)min(kB, n - j0));
#pragma unroll
        for (int k = 0; k < kB; ++k) {
            if (k >= lim) break;
            if (j0 + k >= n) continue;
            if (sizeof(T) == 8 && j0 + k == 0) {
                const double t0 = (double)cur[0];
                acc = (T)((__double_as_longlong(t0) << 1) == 0 ? 0.0 : t0);
            } else if (kahan) {
                const T yk = A::sub(cur[k], comp);
                const T s2 = A::add(acc, yk);
                comp = A::sub(A::sub(s2, acc), yk);
                acc = s2;
            } else {
                acc = A::add(acc, cur[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < kB; ++k) {
            cur[k] = nxt[k];
            ib[k] = ia[k];
        }
    }
    return sizeof(T) == 4 ? A::sub(acc, comp) : acc;
}

// Sum of a row's n terms by one warp (the result is valid in every lane).
//   FP64 exact   the sequential sum, bit for bit: the terms are gathered tile by tile into
//                shared memory and added by the windowed exact scan (256 terms per warp
//                step while the running sum keeps its binade)
//   FP64 native  the sequential sum with hardware adds (lane 0 walks the tile)
//   FP64 tree    lane partial sums and a butterfly (deterministic, not the sequential bits)
//   FP32         Kahan-compensated lane partial sums and a butterfly
template <typename T>
__device__ __forceinline__ T warp_row_sum(const T* __restrict__ y2, const int32_t* __restrict__ idx, int n, int lane,
                                          int mode, double* __restrict__ tile) {
    if constexpr (sizeof(T) == 8) {
        constexpr int kPer = kWarpTile / 32;
        double S = 0.0, part = 0.0;
        for (int c = 0; c < n; c += kWarpTile) {
            const int m = min(kWarpTile, n - c);
            double r[kPer];
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                const int j = lane + 32 * k;
                r[k] = j < m ? __ldg(y2 + __ldg(idx + c + j)) : 0.0;
            }
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                const int j = lane + 32 * k;
                if (j < m) tile[j] = r[k];
            }
            __syncwarp();
            if (mode == kModeExact) {
                S = exact_scan_wide(S, tile, m, lane);
            } else if (mode == kModeNative) {
                if (lane == 0)
                    for (int i = 0; i < m; ++i) S = __dadd_rn(S, tile[i]);
                S = __shfl_sync(kFull, S, 0);
            } else {
#pragma unroll
                for (int k = 0; k < kPer; ++k) part = __dadd_rn(part, r[k]);
            }
            __syncwarp();
        }
        if (mode == kModeTree) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) part = __dadd_rn(part, __shfl_xor_sync(kFull, part, off));
            S = part;
        }
        return (T)S;
    } else {
        float s = 0.f, comp = 0.f;
        for (int j = lane; j < n; j += 32) {
            const float yk = __fsub_rn(__ldg(y2 + __ldg(idx + j)), comp);
            const float s2 = __fadd_rn(s, yk);
            comp = __fsub_rn(__fsub_rn(s2, s), yk);
            s = s2;
        }
        s = __fsub_rn(s, comp);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s = __fadd_rn(s, __shfl_xor_sync(kFull, s, off));
        return (T)s;
    }
}

template <typename T>
__device__ __forceinline__ void batched_vertex_f(const BatchedKArgs& a, int64_t pos, T acc) {
    const int b = find_batch(a.vb, pos);
    const int kind = __ldg(a.vb.kind + b);
    const int64_t r = pos - __ldg(a.vb.pos0 + b);
    const int64_t s0 = __ldg(a.vb.s0 + b), q0 = __ldg(a.vb.p0 + b);
    T* du = static_cast<T*>(a.du);
    const T* u = static_cast<const T*>(a.u);
    const T* p = static_cast<const T*>(a.p);
    switch (kind) {
        case ND_V_DIFFUSION:
            vertex_f_at<T, ND_V_DIFFUSION>(du, u, p, s0 + r, q0, acc);
            break;
        case ND_V_KURAMOTO:
            vertex_f_at<T, ND_V_KURAMOTO>(du, u, p, s0 + r, q0 + r, acc);
            break;
        case ND_V_SWING:
            vertex_f_at<T, ND_V_SWING>(du, u, p, s0 + 2 * r, q0 + 3 * r, acc);
            break;
        default:
            vertex_f_at<T, ND_V_SWING_UNIT>(du, u, p, s0 + 2 * r, q0 + r, acc);
            break;
    }
}

// Rows: blocks [0, n_warp_blocks) take the long rows a warp each, the rest one row per
// thread.  Blocks are small (kRowBlock threads) so that networks with few rows -- dense
// graphs, whose long per-thread chains are the whole cost -- still spread over every SM.
constexpr int kRowBlock = 64;
template <typename T, bool kDense, int NT>
__global__ void __launch_bounds__(NT) batched_row_kernel(BatchedKArgs a, int64_t n_warp_blocks) {
    constexpr int kWarps = NT / 32;
    const T* __restrict__ y2 = static_cast<const T*>(a.y2);
    if ((int64_t)blockIdx.x < n_warp_blocks) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const int64_t slot = (int64_t)blockIdx.x * kWarps + warp;
        if (slot >= a.n_warp_rows) return;  // warp-uniform
        const uint32_t t0 = __ldg(a.tptr + slot);
        const int n = (int)(__ldg(a.tptr + slot + 1) - t0);
        T acc;
        if constexpr (sizeof(T) == 8) {
            __shared__ double tiles[kWarps][kWarpTile];
            acc = warp_row_sum<T>(y2, a.tidx + t0, n, lane, a.mode, tiles[warp]);
        } else {
            acc = warp_row_sum<T>(y2, a.tidx + t0, n, lane, a.mode, nullptr);
        }
        if (lane == 0) batched_vertex_f<T>(a, __ldg(a.slot_vpos + slot), acc);
    } else {
        const int64_t slot = a.n_warp_rows + ((int64_t)blockIdx.x - n_warp_blocks) * NT + threadIdx.x;
        if (slot >= a.nv) return;
        const uint32_t t0 = __ldg(a.tptr + slot);
        const int n = (int)(__ldg(a.tptr + slot + 1) - t0);
        const T acc = kDense ? thread_row_sum_deep<T>(y2, a.tidx + t0, n) : thread_row_sum<T>(y2, a.tidx + t0, n);
        batched_vertex_f<T>(a, __ldg(a.slot_vpos + slot), acc);
    }
}

// ---- output dimension 2: the power-grid networks (complex voltages and currents) ----------
// The same two launches with complex values: y2 holds (y_src, y_dst) as two complex numbers
// per edge position, a term index t names the complex number y2[t], and a row's real and
// imaginary parts are summed side by side in the sequential order, one thread per row.
template <typename T>
__global__ void __launch_bounds__(kBlock) batched_edge_kernel2(BatchedKArgs a) {
    using V2 = typename Vec2<T>::type;
    const T* __restrict__ u = static_cast<const T*>(a.u);
    const T* __restrict__ p = static_cast<const T*>(a.p);
    V2* __restrict__ y2 = static_cast<V2*>(a.y2);
    for (int64_t k = (int64_t)blockIdx.x * kBlock + threadIdx.x; k < a.ne; k += (int64_t)gridDim.x * kBlock) {
        const int b = find_batch(a.eb, k);  // every edge batch is a pi-line batch
        const int64_t q = __ldg(a.eb.p0 + b) + 4 * (k - __ldg(a.eb.pos0 + b));
        const int2 uv = __ldg(a.eu + k);
        const Cx<T> vs = {__ldg(u + uv.x), __ldg(u + uv.x + 1)}, vd = {__ldg(u + uv.y), __ldg(u + uv.y + 1)};
        Cx<T> ys, yd;
        piline_g<T>(vs, vd, __ldg(p + q), __ldg(p + q + 1), __ldg(p + q + 2), __ldg(p + q + 3), ys, yd);
        V2 a0, a1;
        a0.x = ys.r;
        a0.y = ys.i;
        a1.x = yd.r;
        a1.y = yd.i;
        y2[2 * k] = a0;
        y2[2 * k + 1] = a1;
    }
}

template <typename T>
__global__ void __launch_bounds__(kRowBlock) batched_row_kernel2(BatchedKArgs a) {
    using A = Arith<T>;
    using V2 = typename Vec2<T>::type;
    const V2* __restrict__ y2 = static_cast<const V2*>(a.y2);
    const int64_t slot = (int64_t)blockIdx.x * kRowBlock + threadIdx.x;
    if (slot >= a.nv) return;
    const uint32_t t0 = __ldg(a.tptr + slot);
    const int n = (int)(__ldg(a.tptr + slot + 1) - t0);
    T re = T(0), im = T(0);
    for (int j = 0; j < n; ++j) {
        const V2 t = y2[__ldg(a.tidx + t0 + j)];
        if (j == 0) {  // the reference's zero start folded into the first term (0 + t is t)
            re = A::add(T(0), t.x);
            im = A::add(T(0), t.y);
        } else {
            re = A::add(re, t.x);
            im = A::add(im, t.y);
        }
    }
    const int64_t pos = __ldg(a.slot_vpos + slot);
    const int b = find_batch(a.vb, pos);
    const int64_t r = pos - __ldg(a.vb.pos0 + b);
    const int64_t s0 = __ldg(a.vb.s0 + b), q0 = __ldg(a.vb.p0 + b);
    T* du = static_cast<T*>(a.du);
    const T* u = static_cast<const T*>(a.u);
    const T* p = static_cast<const T*>(a.p);
    const int kind = __ldg(a.vb.kind + b);
    if (kind == ND_V_PQ) {
        vertex_f2_at<T, ND_V_PQ>(du, u, p, s0 + 2 * r, q0 + 2 * r, {re, im});
    } else if (kind == ND_V_PQ_CONST) {  // P, Q are the batch's constants
        const Cx<T> uc = cdiv<T>({(T)__ldg(a.vb.consts + kBatchConstants * b),
                                  (T)__ldg(a.vb.consts + kBatchConstants * b + 1)},
                                 {re, -im});
        du[s0 + 2 * r] = uc.r;
        du[s0 + 2 * r + 1] = uc.i;
    } else {
        vertex_f2_at<T, ND_V_GENERATOR>(du, u, p, s0 + 4 * r, q0 + 11 * r, {re, im});
    }
}

template <typename T>
cudaError_t launch_typed(const BatchedNet& b, void* du, const void* u, const void* p, int mode, cudaStream_t s,
                         int phases) {
    BatchedKArgs a;
    a.du = du;
    a.u = u;
    a.p = p;
    a.nv = b.nv;
    a.ne = b.ne;
    a.n_warp_rows = b.n_warp_rows;
    a.vb = b.dvb;
    a.eb = b.deb;
    a.eu = b.eu;
    a.tptr = b.tptr;
    a.tidx = b.tidx;
    a.slot_vpos = b.slot_vpos;
    a.y2 = b.y2;
    a.mode = mode;
    if (b.depth == 2) {
        if ((phases & kPhaseEdge) && b.ne > 0) {
            const int64_t blocks = std::min<int64_t>((b.ne + kBlock - 1) / kBlock, int64_t(1) << 20);
            batched_edge_kernel2<T><<<(unsigned)blocks, kBlock, 0, s>>>(a);
        }
        if (phases & kPhaseRow)
            batched_row_kernel2<T><<<(unsigned)((b.nv + kRowBlock - 1) / kRowBlock), kRowBlock, 0, s>>>(a);
        return cudaGetLastError();
    }
    if ((phases & kPhaseEdge) && b.ne > 0) {
        const int64_t blocks = std::min<int64_t>((b.ne + kBlock - 1) / kBlock, int64_t(1) << 20);
        batched_edge_kernel<T><<<(unsigned)blocks, kBlock, 0, s>>>(a);
    }
    if (phases & kPhaseRow) {
        // dense networks: one-warp blocks, so that their few row warps reach as many SMs
        const int nt = b.dense_rows ? 32 : kRowBlock;
        const int64_t wb = (b.n_warp_rows + nt / 32 - 1) / (nt / 32);
        const int64_t tb = (b.nv - b.n_warp_rows + nt - 1) / nt;
        if (wb + tb > 0) {
            if (b.dense_rows) batched_row_kernel<T, true, 32><<<(unsigned)(wb + tb), 32, 0, s>>>(a, wb);
            else batched_row_kernel<T, false, kRowBlock><<<(unsigned)(wb + tb), kRowBlock, 0, s>>>(a, wb);
        }
    }
    return cudaGetLastError();
}

bool static_kind(int ek) { return ek >= ND_E_DIFFUSION && ek <= ND_E_KURAMOTO; }
bool ode_kind(int ek) { return ek == ND_E_DIFFUSION_ODE || ek == ND_E_DIFFUSION_ODE_FIXED; }

}  // namespace

// Is (kind, coupling) an edge component of the library?
int check_edge_component(int ek, int coupling) {
    if (!static_kind(ek) && !ode_kind(ek) && ek != ND_E_PILINE)
        return fail(ND_ERR_UNSUPPORTED_COMPONENT,
                    "edge model is not in the GB300 component library (diffusion, unit diffusion, kuramoto / "
                    "static line, diffusion ODE edge, pi-line); no CPU fallback exists");
    if (ek == ND_E_PILINE && coupling != ND_FIDUCIAL)
        return fail(ND_ERR_UNSUPPORTED_COMPONENT, "the pi-line edge has a two-sided output function (ND_FIDUCIAL)");
    if (ode_kind(ek) && coupling != ND_FIDUCIAL)
        return fail(ND_ERR_UNSUPPORTED_COMPONENT, "the diffusion ODE edges have Fiducial(dst=1, src=2) outputs");
    if (static_kind(ek) && coupling != ND_ANTISYMMETRIC && coupling != ND_SYMMETRIC && coupling != ND_DIRECTED &&
        !(coupling == ND_FIDUCIAL && ek == ND_E_DIFFUSION))
        return fail(ND_ERR_UNSUPPORTED_COMPONENT,
                    "edge coupling is not in the GB300 library for this edge kind (AntiSymmetric, Symmetric, "
                    "Directed; Fiducial only for diffusionedge_fid!)");
    return ND_OK;
}

// Both batch tables in one device allocation, and their device views.
static cudaError_t upload_tables(BatchedNet& bn) {
    auto bytes_of = [](const BatchTable& t) {
        return (size_t)t.n * (2 * sizeof(int32_t) + 2 * sizeof(int64_t) + kBatchConstants * sizeof(double)) +
               ((size_t)t.n + 1) * sizeof(int64_t);
    };
    const size_t total = bytes_of(bn.vb) + bytes_of(bn.eb) + 256;
    cudaError_t err = cudaMalloc(&bn.table_mem, total);
    if (err != cudaSuccess) return err;
    std::vector<unsigned char> host(total, 0);
    size_t off = 0;
    auto place = [&](const void* src, size_t n) -> size_t {
        off = (off + 7) & ~size_t(7);
        const size_t at = off;
        if (n) std::memcpy(host.data() + at, src, n);
        off += n;
        return at;
    };
    auto build = [&](const BatchTable& t, BatchTableDev& d) {
        const unsigned char* base = static_cast<unsigned char*>(bn.table_mem);
        d.n = t.n;
        d.kind = reinterpret_cast<const int32_t*>(base + place(t.kind.data(), t.n * sizeof(int32_t)));
        d.coupling = reinterpret_cast<const int32_t*>(base + place(t.coupling.data(), t.n * sizeof(int32_t)));
        d.pos0 = reinterpret_cast<const int64_t*>(base + place(t.pos0.data(), (t.n + 1) * sizeof(int64_t)));
        d.s0 = reinterpret_cast<const int64_t*>(base + place(t.s0.data(), t.n * sizeof(int64_t)));
        d.p0 = reinterpret_cast<const int64_t*>(base + place(t.p0.data(), t.n * sizeof(int64_t)));
        d.consts = t.consts.empty() ? nullptr
                                    : reinterpret_cast<const double*>(
                                          base + place(t.consts.data(), t.consts.size() * sizeof(double)));
    };
    build(bn.vb, bn.dvb);
    build(bn.eb, bn.deb);
    return cudaMemcpy(bn.table_mem, host.data(), off, cudaMemcpyHostToDevice);
}

void free_batched(BatchedNet* b) {
    cudaFree(b->table_mem);
    cudaFree(b->eu);
    cudaFree(b->tptr);
    cudaFree(b->tidx);
    cudaFree(b->slot_vpos);
    cudaFree(b->y2);
    *b = BatchedNet{};
}

// Every check on a description, on the host: no device resource is touched before it passes.
int validate_batched(const nd_batched_network_desc* d) {
    const int64_t nv = d->nv, ne = d->ne;
    const int nvb = d->n_vertex_batches, neb = d->n_edge_batches;
    if (nv <= 0) return fail(ND_ERR_ARG, "network has no vertices");
    if (ne < 0) return fail(ND_ERR_ARG, "negative edge count");
    if (d->flags != 0) return fail(ND_ERR_ARG, "nd_batched_network_desc.flags must be 0");
    if (nvb < 1 || nvb > kMaxBatches) return fail(ND_ERR_ARG, "n_vertex_batches must be in 1..ND_MAX_BATCHES");
    if (neb < 0 || neb > kMaxBatches || (ne > 0 && neb == 0))
        return fail(ND_ERR_ARG, "n_edge_batches must be in 1..ND_MAX_BATCHES (0 only without edges)");
    if (!d->vertex_batches || !d->vertex_batch || (neb > 0 && !d->edge_batches) ||
        (ne > 0 && (!d->src || !d->dst || !d->edge_batch)))
        return fail(ND_ERR_ARG, "nd_batched_network_desc: NULL array");
    if (nv > INT32_MAX - 1) return fail(ND_ERR_UNSUPPORTED, "more than 2^31-2 vertices");
    if (2 * ne > (int64_t)INT32_MAX) return fail(ND_ERR_UNSUPPORTED, "more than 2^30-1 edges in a batched network");
    for (int b = 0; b < nvb; ++b) {
        const nd_batch& vb = d->vertex_batches[b];
        if (vb.kind < ND_V_DIFFUSION || vb.kind > ND_V_PQ_CONST)
            return fail(ND_ERR_UNSUPPORTED_COMPONENT,
                        "vertex model is not in the GB300 component library (diffusion, kuramoto first order, "
                        "swing, benchmark swing, PQ bus, generator); no CPU fallback exists");
        if (vb.coupling != 0) return fail(ND_ERR_ARG, "vertex batches take coupling 0");
        if (vb.kind == ND_V_PQ_CONST && !d->vertex_constants)
            return fail(ND_ERR_ARG, "the PQ bus with its own P, Q needs vertex_constants");
    }
    for (int b = 0; b < neb; ++b) {
        const int rc = check_edge_component(d->edge_batches[b].kind, d->edge_batches[b].coupling);
        if (rc != ND_OK) return rc;
    }
    // one output dimension for all vertex models and all edge models (src/construction.jl:98-106)
    const int depth = vertex_outdim(d->vertex_batches[0].kind);
    for (int b = 0; b < nvb; ++b)
        if (vertex_outdim(d->vertex_batches[b].kind) != depth)
            return fail(ND_ERR_ARG, "All vertex models must have the same output dimension!");
    for (int b = 0; b < neb; ++b)
        if (edge_outdim(d->edge_batches[b].kind) != depth)
            return fail(ND_ERR_ARG, "All edge models must have the same output dimension as the vertex models!");
    for (int64_t v = 0; v < nv; ++v) {
        const int32_t b = d->vertex_batch[v];
        if (b < 0 || b >= nvb) return fail(ND_ERR_ARG, "vertex " + std::to_string(v) + " has no valid batch");
    }
    int64_t states = 0, params = 0;
    for (int64_t v = 0; v < nv; ++v) {
        const int k = d->vertex_batches[d->vertex_batch[v]].kind;
        states += vertex_dim(k);
        params += vertex_pdim(k);
    }
    for (int64_t e = 0; e < ne; ++e) {
        const int32_t b = d->edge_batch[e];
        if (b < 0 || b >= neb) return fail(ND_ERR_ARG, "edge " + std::to_string(e) + " has no valid batch");
        const int64_t s = d->src[e], t = d->dst[e];
        if (s < 0 || s >= nv || t < 0 || t >= nv)
            return fail(ND_ERR_ARG, "edge " + std::to_string(e) + " has endpoint out of range");
        states += edge_dim(d->edge_batches[b].kind);
        params += edge_pdim(d->edge_batches[b].kind);
    }
    // the kernels index states and parameters with 32-bit offsets
    if (states > (int64_t)INT32_MAX) return fail(ND_ERR_UNSUPPORTED, "more than 2^31-1 states in a batched network");
    if (params > (int64_t)INT32_MAX)
        return fail(ND_ERR_UNSUPPORTED, "more than 2^31-1 parameters in a batched network");
    return ND_OK;
}

int build_batched(const nd_batched_network_desc* d, int elem, BatchedNet* out) {
    const int rc0 = validate_batched(d);
    if (rc0 != ND_OK) return rc0;
    const int64_t nv = d->nv, ne = d->ne;
    const int nvb = d->n_vertex_batches, neb = d->n_edge_batches;
    const int depth = vertex_outdim(d->vertex_batches[0].kind);
    std::vector<int64_t> vcount(nvb, 0), ecount(std::max(neb, 1), 0);
    for (int64_t v = 0; v < nv; ++v) vcount[d->vertex_batch[v]]++;
    for (int64_t e = 0; e < ne; ++e) ecount[d->edge_batch[e]]++;
    // Batch tables: vertex batches first (register_vertices!), then edge batches whose
    // states follow every vertex state and whose parameters follow every vertex parameter
    // (register_edges!, src/network_structure.jl:224-258).
    BatchTable vb, eb;
    int64_t pos = 0, st = 0, par = 0;
    vb.n = nvb;
    vb.kind.resize(nvb);
    vb.coupling.assign(nvb, 0);
    vb.pos0.resize(nvb + 1);
    vb.s0.resize(nvb);
    vb.p0.resize(nvb);
    vb.consts.assign((size_t)nvb * kBatchConstants, 0.0);
    for (int b = 0; b < nvb; ++b) {
        const int k = d->vertex_batches[b].kind;
        vb.kind[b] = k;
        vb.pos0[b] = pos;
        vb.s0[b] = st;
        vb.p0[b] = par;
        if (d->vertex_constants)
            for (int c = 0; c < kBatchConstants; ++c)
                vb.consts[(size_t)b * kBatchConstants + c] = d->vertex_constants[(size_t)b * kBatchConstants + c];
        pos += vcount[b];
        st += vcount[b] * vertex_dim(k);
        par += vcount[b] * vertex_pdim(k);
    }
    vb.pos0[nvb] = pos;
    const int64_t vdim_total = st;
    eb.n = neb;
    eb.kind.resize(neb);
    eb.coupling.resize(neb);
    eb.pos0.resize(neb + 1);
    eb.s0.resize(neb);
    eb.p0.resize(neb);
    pos = 0;
    for (int b = 0; b < neb; ++b) {
        const int k = d->edge_batches[b].kind;
        eb.kind[b] = k;
        eb.coupling[b] = d->edge_batches[b].coupling;
        eb.pos0[b] = pos;
        eb.s0[b] = st;
        eb.p0[b] = par;
        pos += ecount[b];
        st += ecount[b] * edge_dim(k);
        par += ecount[b] * edge_pdim(k);
    }
    eb.pos0[neb] = pos;
    (void)vdim_total;  // states and parameters fit 32-bit offsets: checked by validate_batched

    // vertex positions and the u index of every vertex output (its first state)
    std::vector<int64_t> fill(vb.pos0.begin(), vb.pos0.begin() + nvb);
    std::vector<int32_t> vpos(nv), vdata(nv);
    for (int64_t v = 0; v < nv; ++v) {
        const int b = d->vertex_batch[v];
        const int64_t k = fill[b]++;
        vpos[v] = (int32_t)k;
        vdata[v] = (int32_t)(vb.s0[b] + (k - vb.pos0[b]) * vertex_dim(vb.kind[b]));
    }
    // edge positions
    std::vector<int64_t> efill(eb.pos0.begin(), eb.pos0.begin() + neb);
    std::vector<int64_t> order(ne);
    for (int64_t e = 0; e < ne; ++e) order[efill[d->edge_batch[e]]++] = e;
    std::vector<int2> eu(ne);
    std::vector<uint32_t> deg(nv, 0);
    for (int64_t k = 0; k < ne; ++k) {
        const int64_t e = order[k];
        eu[k] = make_int2(vdata[d->src[e]], vdata[d->dst[e]]);
        deg[d->src[e]]++;
        deg[d->dst[e]]++;
    }
    // every vertex's terms in ascending output order: for each edge position, the source's
    // entry 2k before the destination's 2k+1
    std::vector<uint32_t> vptr(nv + 1, 0);
    for (int64_t v = 0; v < nv; ++v) vptr[v + 1] = vptr[v] + deg[v];
    std::vector<int32_t> vterms((size_t)2 * ne);
    {
        std::vector<uint32_t> f(vptr.begin(), vptr.end() - 1);
        for (int64_t k = 0; k < ne; ++k) {
            const int64_t e = order[k];
            vterms[f[d->src[e]]++] = (int32_t)(2 * k);
            vterms[f[d->dst[e]]++] = (int32_t)(2 * k + 1);
        }
    }
    // slot order: long rows by degree (descending), then short rows in runs of kLightRun
    // vertex positions, by degree inside a run
    std::vector<int32_t> by_pos(nv);
    for (int64_t v = 0; v < nv; ++v) by_pos[vpos[v]] = (int32_t)v;
    std::vector<int32_t> longr, shortr;
    const int warp_min = elem == 8 ? kWarpRowMinDegF64 : kWarpRowMinDegF32;
    for (int64_t k = 0; k < nv; ++k) {
        const int32_t v = by_pos[k];
        (deg[v] >= (uint32_t)warp_min ? longr : shortr).push_back(v);
    }
    auto by_degree = [&](int32_t x, int32_t y) { return deg[x] > deg[y]; };
    std::stable_sort(longr.begin(), longr.end(), by_degree);
    for (size_t r0 = 0; r0 < shortr.size(); r0 += (size_t)kLightRun)
        std::stable_sort(shortr.begin() + r0, shortr.begin() + std::min(shortr.size(), r0 + (size_t)kLightRun),
                         by_degree);
    std::vector<int32_t> slots;
    slots.reserve(nv);
    slots.insert(slots.end(), longr.begin(), longr.end());
    slots.insert(slots.end(), shortr.begin(), shortr.end());
    std::vector<uint32_t> tptr(nv + 1, 0);
    std::vector<int32_t> tidx((size_t)2 * ne), slot_vpos(nv);
    uint32_t maxdeg = 0;
    for (int64_t s = 0; s < nv; ++s) {
        const int32_t v = slots[s];
        std::copy(vterms.begin() + vptr[v], vterms.begin() + vptr[v + 1], tidx.begin() + tptr[s]);
        tptr[s + 1] = tptr[s] + deg[v];
        slot_vpos[s] = vpos[v];
        maxdeg = std::max(maxdeg, deg[v]);
    }

    BatchedNet bn;
    bn.vb = vb;
    bn.eb = eb;
    bn.nv = nv;
    bn.ne = ne;
    bn.dim = st;
    bn.pdim = par;
    bn.max_degree = (int32_t)maxdeg;
    bn.depth = depth;
    bn.n_warp_rows = (int64_t)longr.size();
    {
        // FP64 thread rows longer than kLightMaxDeg carrying most of the thread-row terms: a
        // dense network, whose row kernel takes the deep batches of thread_row_sum_deep
        int64_t inc_long = 0, inc_short = 0;
        for (int32_t v : shortr) (deg[v] > (uint32_t)kLightMaxDeg ? inc_long : inc_short) += deg[v];
        bn.dense_rows = elem == 8 && inc_long > inc_short;
    }
    auto upload = [&](void** dptr, const void* hptr, size_t bytes) -> cudaError_t {
        cudaError_t err = cudaMalloc(dptr, std::max<size_t>(bytes, 16));
        if (err != cudaSuccess) return err;
        if (bytes) err = cudaMemcpy(*dptr, hptr, bytes, cudaMemcpyHostToDevice);
        return err;
    };
    cudaError_t err;
    if ((err = upload_tables(bn)) != cudaSuccess ||
        (err = upload((void**)&bn.eu, eu.data(), eu.size() * sizeof(int2))) != cudaSuccess ||
        (err = upload((void**)&bn.tptr, tptr.data(), tptr.size() * sizeof(uint32_t))) != cudaSuccess ||
        (err = upload((void**)&bn.tidx, tidx.data(), tidx.size() * sizeof(int32_t))) != cudaSuccess ||
        (err = upload((void**)&bn.slot_vpos, slot_vpos.data(), slot_vpos.size() * sizeof(int32_t))) != cudaSuccess ||
        (elem > 0 && (err = cudaMalloc(&bn.y2, std::max<size_t>((size_t)2 * depth * ne * elem, 16))) != cudaSuccess)) {
        free_batched(&bn);
        return cuda_fail(err, "upload of the batched network");
    }
    bn.enabled = true;
    *out = bn;
    return ND_OK;
}

cudaError_t launch_batched(int dtype, const BatchedNet& b, void* du, const void* u, const void* p, int mode,
                           cudaStream_t s, int phases) {
    return dtype == ND_F64 ? launch_typed<double>(b, du, u, p, mode, s, phases)
                           : launch_typed<float>(b, du, u, p, mode, s, phases);
}

}  // namespace nd
