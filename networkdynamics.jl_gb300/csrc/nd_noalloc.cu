// Allocation-free RHS entry point: nd_rhs_static_scratch (include/nd_gb300.h).
//
// Who needs it: a caller that must not allocate device memory while it runs the RHS,
// for example a process whose device memory is owned by a caching allocator (CUDA.jl's
// or PyTorch's pool), where a library's own cudaMalloc can fail once the pool holds the
// memory or fragment it, or a host program with a fixed device-memory budget that it
// allocates once up front.  nd_create allocates the network's topology and its scratch;
// this entry point allocates nothing: the caller passes the topology arrays and the input /
// output buffers, and the scratch comes from one file-scope __device__ array of fixed size.
//
// The computation is the two-phase RHS of nd_rhs_edge.cu in its simplest form: phase E
// writes each edge's value y_e = g(u_src, u_dst, p_e) to the scratch array, phase R sums
// every vertex's destination-side values (ascending edge id) and then the negated values
// of its source block with hardware adds, in the reference's order, and applies vertex f.
// Phase E writes every scratch entry phase R reads, so nothing needs clearing between
// calls.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>

#include "nd_components.cuh"
#include "nd_internal.h"

namespace nd {

namespace {

// The scratch: every GPU that loads this library holds it until the process exits.
constexpr size_t kStaticScratchBytes = 64ull << 20;  // 64 MiB: 8 Mi FP64 / 16 Mi FP32 edge values
__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void* g_scratch_ptr[kMaxDevices] = {};
void* g_scratch_ctx[kMaxDevices] = {};  // the context the cached address belongs to

// The current driver context (cuCtxGetCurrent through the runtime's entry-point query, so
// the library needs no link to libcuda); nullptr when the query is unavailable.
void* current_context() {
    using GetCurrent = int (*)(void**);
    static GetCurrent fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<GetCurrent>(f);
    }();
    void* ctx = nullptr;
    if (fn && fn(&ctx) != 0) ctx = nullptr;
    return ctx;
}

// Device address of the scratch on the current device.  The set-up (cudaGetSymbolAddress
// with the device current) runs on the first call on a device, and again only if that
// device's context was replaced since (cudaDeviceReset), which reloads the module.
cudaError_t scratch_address(void** out) {
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    void* ctx = g_scratch_ptr[dev] ? current_context() : nullptr;
    if (!g_scratch_ptr[dev] || ctx != g_scratch_ctx[dev]) {
        void* p = nullptr;
        err = cudaGetSymbolAddress(&p, g_static_scratch);
        if (err != cudaSuccess) return err;
        g_scratch_ptr[dev] = p;
        g_scratch_ctx[dev] = current_context();
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

// ---- device checks (nd_set_device_checks) ----------------------------------------------------
// With checks on, the kernels test every index they read from the caller's topology
// arrays before using it.  An index out of range is not dereferenced: its term counts as
// zero.  The first finding goes to a status pair on the device, {kind << 48 | position,
// value}, which the host call reads back; nothing traps.
enum CheckKind : uint64_t {
    kChkSrcRange = 1,    // src[e] outside [0, nv)
    kChkDstRange = 2,    // dst[e] outside [0, nv)
    kChkSrcPtr = 3,      // src_ptr[v] > src_ptr[v + 1] or src_ptr[v + 1] > ne
    kChkDstPtr = 4,      // dst_ptr[v] > dst_ptr[v + 1] or dst_ptr[v + 1] > ne
    kChkDstEid = 5,      // dst_eid[k] outside [0, ne)
    kChkOrder = 6,       // edge e not canonical: src[e] >= dst[e] or src[e - 1] > src[e]
    kChkSrcBlock = 7,    // edge e in vertex v's source block has src[e] != v
    kChkDstBlock = 8,    // dst_eid[k] = e in vertex v's destination list has dst[e] != v
    kChkDstEidOrder = 9  // dst_eid not ascending within vertex v's destination list
};
__device__ unsigned long long g_check_status[2];
std::atomic<bool> g_device_checks{false};

__device__ void check_report(uint64_t kind, int64_t pos, int64_t value) {
    const unsigned long long code = (unsigned long long)(kind << 48) | (unsigned long long)(pos & 0xffffffffffffll);
    if (atomicCAS(&g_check_status[0], 0ull, code) == 0ull) g_check_status[1] = (unsigned long long)value;
}

template <typename T, int VK, int EK, bool CHECK>
__global__ void static_edge_kernel(int64_t nv, int64_t ne, const int32_t* __restrict__ src,
                                   const int32_t* __restrict__ dst, const T* __restrict__ u,
                                   const T* __restrict__ p, T* __restrict__ y) {
    constexpr int DV = VertexDims<VK>::dim;
    const T* __restrict__ pe = p + nv * VertexDims<VK>::pdim;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t se = src[e], de = dst[e];
        if constexpr (CHECK) {
            const bool bad_s = se < 0 || se >= nv, bad_d = de < 0 || de >= nv;
            if (bad_s) check_report(kChkSrcRange, e, se);
            if (bad_d) check_report(kChkDstRange, e, de);
            if (bad_s || bad_d) {
                y[e] = T(0);
                continue;
            }
            if (se >= de || (e > 0 && src[e - 1] > se)) check_report(kChkOrder, e, se);
        }
        const T us = __ldg(u + (int64_t)se * DV), ud = __ldg(u + (int64_t)de * DV);
        const T w = EK == ND_E_DIFFUSION_UNIT ? T(0) : __ldg(pe + e);
        y[e] = edge_g_w<T, EK>(us, ud, w);
    }
}

template <typename T, int VK, int EK, bool CHECK>
__global__ void static_row_kernel(int64_t nv, int64_t ne, const int32_t* __restrict__ src,
                                  const int32_t* __restrict__ dst, const uint32_t* __restrict__ src_ptr,
                                  const uint32_t* __restrict__ dst_ptr, const int32_t* __restrict__ dst_eid,
                                  const T* __restrict__ y, const T* __restrict__ u, const T* __restrict__ p,
                                  T* __restrict__ du) {
    using A = Arith<T>;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
        uint32_t d0 = dst_ptr[v], d1 = dst_ptr[v + 1], s0 = src_ptr[v], s1 = src_ptr[v + 1];
        if constexpr (CHECK) {
            if (d0 > d1 || d1 > (uint64_t)ne) {
                check_report(kChkDstPtr, v, d1);
                d1 = d0;
            }
            if (s0 > s1 || s1 > (uint64_t)ne) {
                check_report(kChkSrcPtr, v, s1);
                s1 = s0;
            }
        }
        // FP32 rows longer than kLightMaxDeg add with Kahan compensation, as the row phase of
        // nd_rhs does: both give the same bits on every row of degree <= kMediumMaxDeg
        const bool kahan = sizeof(T) == 4 && (d1 - d0) + (s1 - s0) > (uint32_t)kLightMaxDeg;
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
        [[maybe_unused]] int32_t prev = -1;
        for (uint32_t k = d0; k < d1; ++k) {
            const int32_t e = dst_eid[k];
            if constexpr (CHECK) {
                if (e < 0 || e >= ne) {
                    check_report(kChkDstEid, k, e);
                    continue;
                }
                if (dst[e] != v) check_report(kChkDstBlock, k, e);
                if (e <= prev) check_report(kChkDstEidOrder, k, e);
                prev = e;
            }
            add(y[e]);
        }
        for (uint32_t e = s0; e < s1; ++e) {
            if constexpr (CHECK) {
                if (src[e] != v) check_report(kChkSrcBlock, e, src[e]);
            }
            add(-y[e]);
        }
        if constexpr (sizeof(T) == 4) acc = A::sub(acc, comp);
        vertex_f<T, VK>(du, u, p, v, acc);
    }
}

template <typename T, int VK, int EK, bool CHECK>
cudaError_t launch_static(int64_t nv, int64_t ne, const int32_t* src, const int32_t* dst, const uint32_t* src_ptr,
                          const uint32_t* dst_ptr, const int32_t* dst_eid, void* du, const void* u, const void* p,
                          void* scratch, cudaStream_t s) {
    // grid-stride kernels: at most 16 blocks per SM of the current device
    const int block = 256;
    int dev = 0, sms = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err == cudaSuccess) err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (err != cudaSuccess) return err;
    const int64_t cap = 16 * (int64_t)std::max(sms, 1);
    const unsigned ge = (unsigned)std::min<int64_t>((ne + block - 1) / block, cap);
    const unsigned gv = (unsigned)std::min<int64_t>((nv + block - 1) / block, cap);
    T* y = static_cast<T*>(scratch);
    if (ne > 0)
        static_edge_kernel<T, VK, EK, CHECK><<<ge, block, 0, s>>>(nv, ne, src, dst, static_cast<const T*>(u),
                                                                  static_cast<const T*>(p), y);
    static_row_kernel<T, VK, EK, CHECK><<<gv, block, 0, s>>>(nv, ne, src, dst, src_ptr, dst_ptr, dst_eid, y,
                                                             static_cast<const T*>(u), static_cast<const T*>(p),
                                                             static_cast<T*>(du));
    return cudaGetLastError();
}

template <typename T, bool CHECK>
cudaError_t launch_static_dtype(int vk, int ek, int64_t nv, int64_t ne, const int32_t* src, const int32_t* dst,
                                const uint32_t* src_ptr, const uint32_t* dst_ptr, const int32_t* dst_eid, void* du,
                                const void* u, const void* p, void* scratch, cudaStream_t s) {
#define ND_CASE(VK, EK)            \
    if (vk == VK && ek == EK)      \
        return launch_static<T, VK, EK, CHECK>(nv, ne, src, dst, src_ptr, dst_ptr, dst_eid, du, u, p, scratch, s);
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

extern "C" int nd_rhs_static_scratch(int dtype, int vertex_kind, int edge_kind, int64_t nv, int64_t ne,
                                     const int32_t* src, const int32_t* dst, const uint32_t* src_ptr,
                                     const uint32_t* dst_ptr, const int32_t* dst_eid, void* du, const void* u,
                                     const void* p, void* stream) {
    clear_error();
    ND_NVTX("nd_rhs_static_scratch");
    if (dtype != ND_F32 && dtype != ND_F64) return fail(ND_ERR_DTYPE, "nd_rhs_static_scratch: dtype must be ND_F32 or ND_F64");
    if (vertex_kind < ND_V_DIFFUSION || vertex_kind > ND_V_SWING || edge_kind < ND_E_DIFFUSION ||
        edge_kind > ND_E_KURAMOTO)
        return fail(ND_ERR_UNSUPPORTED_COMPONENT, "nd_rhs_static_scratch: component not in the GB300 library");
    if (nv <= 0 || ne < 0) return fail(ND_ERR_ARG, "nd_rhs_static_scratch: nv must be > 0 and ne >= 0");
    const size_t elem = dtype == ND_F64 ? 8 : 4;
    const int64_t max_edges = (int64_t)(kStaticScratchBytes / elem);
    if (ne > max_edges)
        return fail(ND_ERR_ARG, "nd_rhs_static_scratch: " + std::to_string(ne) + " edges exceed the static scratch (" +
                                    std::to_string(max_edges) + " edges of this precision, " +
                                    std::to_string(kStaticScratchBytes >> 20) + " MiB); use nd_create / nd_rhs");
    if (nv > INT32_MAX) return fail(ND_ERR_ARG, "nd_rhs_static_scratch: more than 2^31-1 vertices");
    if (!du || !u || !src_ptr || !dst_ptr || (ne > 0 && (!src || !dst || !dst_eid)))
        return fail(ND_ERR_ARG, "nd_rhs_static_scratch: NULL buffer");
    const int pdim_v = vertex_pdim(vertex_kind), pdim_e = edge_pdim(edge_kind);
    if ((pdim_v > 0 || (pdim_e > 0 && ne > 0)) && !p) return fail(ND_ERR_ARG, "nd_rhs_static_scratch: p is NULL");
    void* scratch = nullptr;
    cudaError_t err = scratch_address(&scratch);
    if (err != cudaSuccess) return cuda_fail(err, "nd_rhs_static_scratch: cudaGetSymbolAddress");
    cudaStream_t s = (cudaStream_t)stream;
    if (!g_device_checks.load()) {
        err = dtype == ND_F64 ? launch_static_dtype<double, false>(vertex_kind, edge_kind, nv, ne, src, dst, src_ptr,
                                                                   dst_ptr, dst_eid, du, u, p, scratch, s)
                              : launch_static_dtype<float, false>(vertex_kind, edge_kind, nv, ne, src, dst, src_ptr,
                                                                  dst_ptr, dst_eid, du, u, p, scratch, s);
        if (err != cudaSuccess) return cuda_fail(err, "nd_rhs_static_scratch kernel launch");
        return ND_OK;
    }
    // checked call: clear the status, run the checking kernels, read the status back
    void* status = nullptr;
    err = cudaGetSymbolAddress(&status, g_check_status);
    if (err != cudaSuccess) return cuda_fail(err, "nd_rhs_static_scratch: device check status");
    err = cudaMemsetAsync(status, 0, sizeof(unsigned long long) * 2, s);
    if (err != cudaSuccess) return cuda_fail(err, "nd_rhs_static_scratch: clearing the device check status");
    err = dtype == ND_F64 ? launch_static_dtype<double, true>(vertex_kind, edge_kind, nv, ne, src, dst, src_ptr,
                                                              dst_ptr, dst_eid, du, u, p, scratch, s)
                          : launch_static_dtype<float, true>(vertex_kind, edge_kind, nv, ne, src, dst, src_ptr,
                                                             dst_ptr, dst_eid, du, u, p, scratch, s);
    if (err != cudaSuccess) return cuda_fail(err, "nd_rhs_static_scratch kernel launch");
    unsigned long long st[2] = {0, 0};
    err = cudaMemcpyAsync(st, status, sizeof st, cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) return cuda_fail(err, "nd_rhs_static_scratch: reading the device check status");
    if (st[0] == 0) return ND_OK;
    static const char* const what[] = {"",
                                       "src[e] outside [0, nv)",
                                       "dst[e] outside [0, nv)",
                                       "src_ptr[v] > src_ptr[v+1] or src_ptr[v+1] > ne",
                                       "dst_ptr[v] > dst_ptr[v+1] or dst_ptr[v+1] > ne",
                                       "dst_eid[k] outside [0, ne)",
                                       "edge list not canonical (src[e] >= dst[e] or src[e-1] > src[e])",
                                       "src[e] != v inside vertex v's source block",
                                       "dst[dst_eid[k]] != v inside vertex v's destination list",
                                       "dst_eid not ascending inside a vertex's destination list"};
    const unsigned kind = (unsigned)(st[0] >> 48);
    const long long pos = (long long)(st[0] & 0xffffffffffffull);
    const char* at = kind == kChkSrcPtr || kind == kChkDstPtr ? "v" : (kind == kChkDstEid || kind == kChkDstBlock ||
                                                                     kind == kChkDstEidOrder) ? "k" : "e";
    return fail(ND_ERR_DEVICE_CHECK, std::string("nd_rhs_static_scratch: device check: ") +
                                         (kind < sizeof what / sizeof what[0] ? what[kind] : "unknown finding") +
                                         " at " + at + " = " + std::to_string(pos) + " (value " +
                                         std::to_string((long long)st[1]) + ")");
}

extern "C" int nd_set_device_checks(int on) {
    clear_error();
    if (on != 0 && on != 1) return fail(ND_ERR_ARG, "nd_set_device_checks: on must be 0 or 1");
    g_device_checks.store(on == 1);
    return ND_OK;
}
