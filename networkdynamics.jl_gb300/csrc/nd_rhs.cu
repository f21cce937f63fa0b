// Fused network right-hand side over the destination-sorted CSR.
//
// One RHS replaces the reference's phased core loop (src/coreloop.jl:22-101): vertex g,
// edge g/f, the gather of vertex outputs into edge inputs (src/gbufs.jl:7-25), the
// aggregation (src/aggregators.jl:133-151) and vertex f.  Vertex outputs are the first
// state (StateMask(1)), so edges read u directly; edge values live in registers or shared
// memory; each row is summed in ascending edge id, the SequentialAggregator order; du is
// written once.  There are no output, gather or aggregation buffers.
//
// One launch, two roles chosen per block (degree buckets and slot order: nd_internal.h):
//   heavy   a block per row: the terms of kTile incidences at a time go to shared memory
//           and warp 0 adds them in order with the exact scan (FP64), or the block sums
//           thread-strided slices in a fixed tree (FP32 with Kahan, FP64 tree mode);
//   window  a block per window of rows: phase A evaluates the window's edge terms, one
//           incidence per thread (coalesced incidence loads, independent gathers and FP64
//           operations in flight) into shared memory; phase B sums one row per thread.
// Heavy blocks come first so the long rows start early.
//
// Cache policy: u is gathered at random and is re-read by every incidence, so its loads
// ask L2 to keep the lines (evict_last); the incidence stream and the edge parameters are
// read once per side and ask to be evicted first.
//
// FP64 on GB300 retires ~2 lanes/clock/SM and a DADD holds its sub-partition's FP64 pipe
// for a full warp even with one lane active.  Window rows (at most kMediumMaxDeg long)
// add with hardware DADDs, all lanes busy on rows of similar length.  A hub's sum would
// be a chain of thousands of DADDs on one sub-partition, so it runs on the integer pipes:
//   * the heavy rows' warp sums use an exact scan: while the running sum S stays inside one binade,
//     RN(S + t) = S + RN(t / ulp(S)) ulp(S), so a run of additions becomes an integer
//     prefix sum of the terms scaled to S's ulp.  A lane whose prefix leaves the binade
//     (or whose scaled term is a tie) ends the run; that one step is done with the exact
//     adder and the scan resumes.  The result equals the sequential sum bit for bit.

#include "nd_components.cuh"
#include "nd_exact.cuh"
#include "nd_internal.h"
#include "nd_scan.cuh"

namespace nd {

namespace {

using namespace dev;

// Shared memory of one block, sized for the largest role (light windows in FP64).
template <typename T>
struct Smem {
    static constexpr int kWin = (kWindowIncidences + kWindow) * (int)sizeof(T) + kWindowIncidences;
    static constexpr int kHeavy = kTile * (int)sizeof(double);
    static constexpr int kBytes = kWin > kHeavy ? kWin : kHeavy;
};

// ---- heavy: a block per row ---------------------------------------------------------------
template <typename T, int VK, int EK, int MODE>
__device__ __forceinline__ void block_row(const RhsArgs& a, int slot, unsigned char* smem) {
    using A = Arith<T>;
    constexpr int DV = VertexDims<VK>::dim;
    const T* __restrict__ u = static_cast<const T*>(a.u);
    const T* __restrict__ p = static_cast<const T*>(a.p);
    const T* __restrict__ pe = p + a.nv * VertexDims<VK>::pdim;
    const int2* __restrict__ incid = reinterpret_cast<const int2*>(a.incid);
    const uint64_t keep = policy_evict_last(), stream = policy_evict_first();
    const int64_t v = __ldg(a.slot_vertex + slot);
    const uint32_t beg = __ldg(a.slot_ptr + slot), end = __ldg(a.slot_ptr + slot + 1);
    const T uv = __ldg(u + v * DV);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if constexpr (sizeof(T) == 8 && MODE != kModeTree) {
        double* tile = reinterpret_cast<double*>(smem);
        double S = 0.0;
        for (uint32_t base = beg; base < end; base += kTile) {
            const int n = (int)min((uint32_t)kTile, end - base);
#pragma unroll 4
            for (int i = tid; i < n; i += kBlock) {
                const int2 inc = ld_hint(incid + base + i, stream);
                const T un = ld_hint(u + (int64_t)inc.x * DV, keep);
                const T w = edge_param<T, EK>(pe, inc.y & 0x7fffffff, stream);
                tile[i] = incidence_term_w<T, EK>(uv, un, w, inc.y < 0);
            }
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
        for (uint32_t k = beg + tid; k < end; k += kBlock) {
            const int2 inc = ld_hint(incid + k, stream);
            const T un = ld_hint(u + (int64_t)inc.x * DV, keep);
            const T w = edge_param<T, EK>(pe, inc.y & 0x7fffffff, stream);
            const T term = incidence_term_w<T, EK>(uv, un, w, inc.y < 0);
            if constexpr (sizeof(T) == 4) {
                const T y = A::sub(term, comp);
                const T s = A::add(acc, y);
                comp = A::sub(A::sub(s, acc), y);
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

// ---- windows: a block per window of rows ----------------------------------------------------
template <typename T, int VK, int EK, int MODE>
__device__ __forceinline__ void window_block(const RhsArgs& a, int win, unsigned char* smem) {
    using A = Arith<T>;
    constexpr int DV = VertexDims<VK>::dim;
    const T* __restrict__ u = static_cast<const T*>(a.u);
    const T* __restrict__ p = static_cast<const T*>(a.p);
    const T* __restrict__ pe = p + a.nv * VertexDims<VK>::pdim;
    const int2* __restrict__ incid = reinterpret_cast<const int2*>(a.incid);
    T* s_term = reinterpret_cast<T*>(smem);                        // [kWindowIncidences]
    T* s_uv = s_term + kWindowIncidences;                          // [kWindow]
    uint8_t* s_owner = reinterpret_cast<uint8_t*>(s_uv + kWindow);  // [kWindowIncidences]
    const uint64_t keep = policy_evict_last(), stream = policy_evict_first();
    const int first = a.n_heavy;
    const int slot0 = first + __ldg(a.win_ptr + win), slot1 = first + __ldg(a.win_ptr + win + 1);
    const uint32_t i0 = __ldg(a.slot_ptr + slot0), i1 = __ldg(a.slot_ptr + slot1);
    const int n = (int)(i1 - i0);  // <= kWindowIncidences
    const int tid = threadIdx.x;
    // phase 0: each row's vertex value and the owner (row) of each incidence
    const int s = slot0 + tid;
    const bool has_row = s < slot1;
    int64_t v = 0;
    int beg = 0, end = 0;
    if (has_row) {
        v = __ldg(a.slot_vertex + s);
        beg = (int)(__ldg(a.slot_ptr + s) - i0);
        end = (int)(__ldg(a.slot_ptr + s + 1) - i0);
        s_uv[tid] = ld_hint(u + v * DV, keep);
        for (int j = beg; j < end; ++j) s_owner[j] = (uint8_t)tid;
    }
    __syncthreads();
    // phase A: the edge terms, one incidence per thread: coalesced incidence loads, many
    // independent gathers and FP64 operations in flight
#pragma unroll 4
    for (int k = tid; k < n; k += kBlock) {
        const int2 inc = ld_hint(incid + i0 + k, stream);
        const T un = ld_hint(u + (int64_t)inc.x * DV, keep);
        const T w = edge_param<T, EK>(pe, inc.y & 0x7fffffff, stream);
        s_term[k] = incidence_term_w<T, EK>(s_uv[s_owner[k]], un, w, inc.y < 0);
    }
    __syncthreads();
    // phase B: one row per thread, in edge order.  FP64: hardware adds (a row is at most
    // kMediumMaxDeg long; one DADD per term is cheaper than the ~100 integer operations
    // of an emulated add).  FP32: compensated sums on the rows above kLightMaxDeg.
    if (!has_row) return;
    T acc = T(0);
    if constexpr (sizeof(T) == 8) {
        for (int j = beg; j < end; ++j) acc = __dadd_rn(acc, s_term[j]);
    } else {
        if (end - beg > kLightMaxDeg) {
            T comp = T(0);
            for (int j = beg; j < end; ++j) {
                const T y = A::sub(s_term[j], comp);
                const T t = A::add(acc, y);
                comp = A::sub(A::sub(t, acc), y);
                acc = t;
            }
            acc = A::sub(acc, comp);
        } else {
            for (int j = beg; j < end; ++j) acc = A::add(acc, s_term[j]);
        }
    }
    vertex_f<T, VK>(static_cast<T*>(a.du), u, p, v, acc);
}

template <typename T, int VK, int EK, int MODE>
__global__ void __launch_bounds__(kBlock, 8) rhs_kernel(RhsArgs a) {
    __shared__ __align__(16) unsigned char smem[Smem<T>::kBytes];
    const int nh = a.heavy_separate ? 0 : a.n_heavy;
    const int b = blockIdx.x;
    if (b < nh) {
        block_row<T, VK, EK, MODE>(a, b, smem);
    } else {
        window_block<T, VK, EK, MODE>(a, b - nh, smem);
    }
}

// Heavy rows alone, a block per row.  The FP32 and tree rows ask for most of an SM's shared
// memory, which keeps all but four other blocks off the SM: the row's summation chain is
// serial, and on a crowded SM each of its steps waits for other blocks' instructions.
constexpr int kHeavySoloSmem = 160 * 1024;

// FP64 sequential sum of a heavy row in the solo kernel, in tiles of TILE terms: warp 0
// adds tile k of the row's terms (exact scan, or the hardware DADD chain in the native
// mode) while warps 1..7 evaluate tile k + 1 into the other half of a double buffer, so the
// serial chain never waits for its terms after the first tile.
constexpr int kSoloTile = 8192;

template <int VK, int EK, int MODE, int TILE>
__device__ __forceinline__ void solo_row_fp64(const RhsArgs& a, int slot, double* buf) {
    constexpr int DV = VertexDims<VK>::dim;
    const double* __restrict__ u = static_cast<const double*>(a.u);
    const double* __restrict__ p = static_cast<const double*>(a.p);
    const double* __restrict__ pe = p + a.nv * VertexDims<VK>::pdim;
    const int2* __restrict__ incid = reinterpret_cast<const int2*>(a.incid);
    const uint64_t keep = policy_evict_last(), stream = policy_evict_first();
    const int64_t v = __ldg(a.slot_vertex + slot);
    const uint32_t beg = __ldg(a.slot_ptr + slot), end = __ldg(a.slot_ptr + slot + 1);
    const double uv = __ldg(u + v * DV);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ntiles = (int)((end - beg + TILE - 1) / TILE);
    auto load = [&](int k, int first, int stride) {
        const uint32_t base = beg + (uint32_t)k * TILE;
        const int n = (int)min((uint32_t)TILE, end - base);
        double* dst = buf + (k & 1) * TILE;
#pragma unroll 4
        for (int i = first; i < n; i += stride) {
            const int2 inc = ld_hint(incid + base + i, stream);
            const double un = ld_hint(u + (int64_t)inc.x * DV, keep);
            const double w = edge_param<double, EK>(pe, inc.y & 0x7fffffff, stream);
            dst[i] = incidence_term_w<double, EK>(uv, un, w, inc.y < 0);
        }
    };
    if (ntiles > 0) load(0, tid, kBlock);
    __syncthreads();
    double S = 0.0;
    for (int k = 0; k < ntiles; ++k) {
        if (warp == 0) {
            const double* cur = buf + (k & 1) * TILE;
            const int n = (int)min((uint32_t)TILE, end - (beg + (uint32_t)k * TILE));
            if constexpr (MODE == kModeNative) {
                if (lane == 0)
                    for (int i = 0; i < n; ++i) S = __dadd_rn(S, cur[i]);
            } else {
                S = exact_scan_wide(S, cur, n, lane);
            }
        } else if (k + 1 < ntiles) {
            load(k + 1, tid - 32, kBlock - 32);
        }
        __syncthreads();
    }
    if (tid == 0) vertex_f<double, VK>(static_cast<double*>(a.du), u, p, v, S);
}

template <typename T, int VK, int EK, int MODE, int TILE>
__global__ void __launch_bounds__(kBlock, 1) heavy_solo_kernel(RhsArgs a) {
    extern __shared__ __align__(16) unsigned char smem_dyn[];
    if constexpr (sizeof(T) == 8 && MODE != kModeTree) {
        static_assert(2 * TILE * sizeof(double) <= kHeavySoloSmem, "solo double buffer");
        solo_row_fp64<VK, EK, MODE, TILE>(a, blockIdx.x, reinterpret_cast<double*>(smem_dyn));
    } else {
        block_row<T, VK, EK, MODE>(a, blockIdx.x, smem_dyn);
    }
}

template <typename T, int VK, int EK, int MODE, int TILE>
cudaError_t launch_heavy_solo_t(const RhsArgs& a, cudaStream_t s, int smem) {
    static int attr_set = 0;  // per instantiation; the attribute is per function
    if (attr_set < smem) {
        cudaError_t err = cudaFuncSetAttribute(heavy_solo_kernel<T, VK, EK, MODE, TILE>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (err != cudaSuccess) return err;
        attr_set = smem;
    }
    heavy_solo_kernel<T, VK, EK, MODE, TILE><<<a.n_heavy, kBlock, smem, s>>>(a);
    return cudaGetLastError();
}

// The FP64 sequential sums (exact scan and hardware chains) use tiles of kSoloTileShared
// terms: 32 KB of shared memory, so that a heavy-row block also fits on an SM that already
// holds seven edge-phase blocks.  With the whole-SM request a heavy block could start only
// on an SM holding at most four, and when the edge phase had filled the GPU first the heavy
// rows waited for its end and outlasted the row phase: stretches of calls at 776-793 µs
// instead of 755 µs on BA(1e7, 4).  With the small tiles and the handle's high-priority
// side stream (FP64 handles) the step took 747-753 µs in every stretch.  The FP32 and tree
// heavy rows keep the whole-SM request: with small tiles they took 515 µs against 476 µs.
constexpr int kSoloTileShared = 2048;

template <typename T, int VK, int EK, int MODE>
cudaError_t launch_heavy_solo(const RhsArgs& a, cudaStream_t s) {
    if constexpr (sizeof(T) == 8 && MODE != kModeTree) {
        constexpr int smem = (int)(2 * kSoloTileShared * sizeof(double));
        return launch_heavy_solo_t<T, VK, EK, MODE, kSoloTileShared>(a, s, smem);
    } else {
        return launch_heavy_solo_t<T, VK, EK, MODE, kSoloTile>(a, s, kHeavySoloSmem);
    }
}

template <typename T, int VK, int EK>
cudaError_t launch_heavy_typed(const RhsArgs& a, cudaStream_t s) {
    if (a.n_heavy == 0) return cudaSuccess;
    if constexpr (sizeof(T) == 4) {
        return launch_heavy_solo<T, VK, EK, kModeTree>(a, s);
    } else {
        switch (a.mode) {
            case kModeNative: return launch_heavy_solo<T, VK, EK, kModeNative>(a, s);
            case kModeTree: return launch_heavy_solo<T, VK, EK, kModeTree>(a, s);
            default: return launch_heavy_solo<T, VK, EK, kModeExact>(a, s);
        }
    }
}

template <typename T, int VK, int EK>
cudaError_t launch_typed(const RhsArgs& a, cudaStream_t s) {
    if (a.heavy_only) return launch_heavy_typed<T, VK, EK>(a, s);
    const int grid = (a.heavy_separate ? 0 : a.n_heavy) + a.n_windows;
    if (grid == 0) return cudaSuccess;
    if constexpr (sizeof(T) == 4) {
        rhs_kernel<T, VK, EK, kModeTree><<<grid, kBlock, 0, s>>>(a);
    } else {
        switch (a.mode) {
            case kModeNative:
                rhs_kernel<T, VK, EK, kModeNative><<<grid, kBlock, 0, s>>>(a);
                break;
            case kModeTree:
                rhs_kernel<T, VK, EK, kModeTree><<<grid, kBlock, 0, s>>>(a);
                break;
            default:
                rhs_kernel<T, VK, EK, kModeExact><<<grid, kBlock, 0, s>>>(a);
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

// Self-test of the integer-exact adder.
__global__ void exact_add_selftest_kernel(const double* a, const double* b, double* out, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = exact::add_rn(a[i], b[i]);
}

// Self-test of the exact scans: one block per segment; odd segments use the 32-term warp
// scan on registers, even segments shared-memory tiles with the 32-term scan (w % 4 == 2)
// or the sliding 256-term scan of the heavy rows' path (w % 4 == 0).
__global__ void exact_scan_selftest_kernel(const double* terms, const int64_t* seg, const double* s0, double* out,
                                           int64_t nseg) {
    __shared__ double tile[kTile];
    const int64_t w = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double S = s0[w];
    if (w & 1) {
        if (warp == 0) {
            for (int64_t c = seg[w]; c < seg[w + 1]; c += 32) {
                const int64_t k = c + lane;
                const double t = k < seg[w + 1] ? terms[k] : 0.0;
                const int n = (int)min((int64_t)32, seg[w + 1] - c);
                S = exact_scan_add(S, t, n, lane);
            }
        }
    } else {
        for (int64_t base = seg[w]; base < seg[w + 1]; base += kTile) {
            const int n = (int)min((int64_t)kTile, seg[w + 1] - base);
            for (int i = threadIdx.x; i < n; i += blockDim.x) tile[i] = terms[base + i];
            __syncthreads();
            if (warp == 0) S = (w & 2) ? exact_scan_smem(S, tile, n, lane) : exact_scan_wide(S, tile, n, lane);
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) out[w] = S;
}

}  // namespace

cudaError_t launch_rhs(int dtype, const RhsArgs& a, cudaStream_t s) {
    return dtype == ND_F64 ? launch_dtype<double>(a, s) : launch_dtype<float>(a, s);
}

cudaError_t launch_exact_selftest(const double* a, const double* b, double* out, int64_t n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    exact_add_selftest_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, b, out, n);
    return cudaGetLastError();
}

cudaError_t launch_scan_selftest(const double* terms, const int64_t* seg, const double* s0, double* out, int64_t nseg,
                                 cudaStream_t s) {
    if (nseg <= 0) return cudaSuccess;
    exact_scan_selftest_kernel<<<(unsigned)nseg, kBlock, 0, s>>>(terms, seg, s0, out, nseg);
    return cudaGetLastError();
}

}  // namespace nd
