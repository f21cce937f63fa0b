// C ABI of libnd_b200.so: handle life cycle, argument checks and the RHS entry point.
//
// Argument checks mirror the reference's: sizes of du/u/p (src/coreloop.jl:2-7), the
// precision the caches were adapted to (src/network_structure.jl:145-151), and the
// component library (anything else raises instead of falling back to the CPU).

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "nd_internal.h"
#include "nd_gb300_selftest.h"

namespace nd {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }
int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
int cuda_fail(cudaError_t err, const char* what) {
    std::string msg = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(err);
    g_last_error = msg;
    return err == cudaErrorMemoryAllocation ? ND_ERR_NOMEM : ND_ERR_CUDA;
}

void free_topology(Topology* t) {
    cudaFree(t->slot_ptr);
    cudaFree(t->slot_vertex);
    cudaFree(t->incid);
    cudaFree(t->win_ptr);
    EdgeLayout& el = t->edge;
    cudaFree(el.esrc);
    cudaFree(el.edst);
    cudaFree(el.lslot);
    cudaFree(el.run_start);
    cudaFree(el.run_base);
    cudaFree(el.rmeta);
    cudaFree(el.locp);
    cudaFree(el.y);
    cudaFree(el.ybkt);
    *t = Topology{};
}

// Canonical edge list: sorted by source, src < dst for every edge.
static bool is_canonical(int64_t ne, const int64_t* src, const int64_t* dst) {
    for (int64_t e = 0; e < ne; ++e) {
        if (src[e] >= dst[e]) return false;
        if (e > 0 && src[e] < src[e - 1]) return false;
    }
    return true;
}

// Host side of the edge-centric layout (see EdgeLayout in nd_internal.h).
struct EdgeLayoutHost {
    std::vector<int32_t> esrc, edst, loc, run_base;
    std::vector<uint16_t> lslot, run_start;
    std::vector<uint32_t> dptr, sptr;
    int64_t n_chunks = 0;
};

static void build_edge_layout(int64_t nv, int64_t ne, const int64_t* src, const int64_t* dst, EdgeLayoutHost& h) {
    h.esrc.resize(ne);
    h.edst.resize(ne);
    h.dptr.assign(nv + 1, 0);
    h.sptr.assign(nv + 1, 0);
    for (int64_t e = 0; e < ne; ++e) {
        h.esrc[e] = (int32_t)src[e];
        h.edst[e] = (int32_t)dst[e];
        h.dptr[dst[e] + 1]++;
        h.sptr[src[e] + 1]++;
    }
    for (int64_t v = 0; v < nv; ++v) {
        h.dptr[v + 1] += h.dptr[v];
        h.sptr[v + 1] += h.sptr[v];
    }
    // destination-CSR position of each edge (ascending edge id inside a destination)
    std::vector<uint32_t> tpos(ne);
    {
        std::vector<uint32_t> fill(h.dptr.begin(), h.dptr.end() - 1);
        for (int64_t e = 0; e < ne; ++e) tpos[e] = fill[dst[e]]++;
    }
    // buckets of destination-CSR positions; ybkt is bucket-major, chunk-major inside a
    // bucket, edge order inside a (bucket, chunk) run
    const int64_t bsize = std::max<int64_t>(1, (ne + kBuckets - 1) / kBuckets);
    const int64_t nch = (ne + kEdgeChunk - 1) / kEdgeChunk;
    h.n_chunks = nch;
    std::vector<int64_t> cnt((size_t)kBuckets * std::max<int64_t>(nch, 1), 0);  // [bucket][chunk]
    for (int64_t e = 0; e < ne; ++e) cnt[(tpos[e] / bsize) * nch + e / kEdgeChunk]++;
    // staging order inside a chunk: bucket-major, edge order inside a bucket
    h.run_start.assign((size_t)nch * (kBuckets + 1), 0);
    for (int64_t c = 0; c < nch; ++c)
        for (int b = 0; b < kBuckets; ++b)
            h.run_start[c * (kBuckets + 1) + b + 1] =
                (uint16_t)(h.run_start[c * (kBuckets + 1) + b] + cnt[(size_t)b * nch + c]);
    std::vector<int64_t> next_slot((size_t)kBuckets * std::max<int64_t>(nch, 1));  // [bucket][chunk]
    for (int64_t c = 0; c < nch; ++c)
        for (int b = 0; b < kBuckets; ++b) next_slot[(size_t)b * nch + c] = h.run_start[c * (kBuckets + 1) + b];
    int64_t run = 0;
    for (size_t i = 0; i < cnt.size(); ++i) {
        const int64_t c = cnt[i];
        cnt[i] = run;
        run += c;
    }
    h.run_base.resize((size_t)nch * kBuckets);
    for (int64_t c = 0; c < nch; ++c)
        for (int b = 0; b < kBuckets; ++b) h.run_base[c * kBuckets + b] = (int32_t)cnt[(size_t)b * nch + c];
    h.lslot.resize(ne);
    h.loc.resize(ne);
    for (int64_t e = 0; e < ne; ++e) {
        const size_t key = (size_t)(tpos[e] / bsize) * nch + e / kEdgeChunk;
        const int64_t qe = cnt[key]++;
        h.lslot[e] = (uint16_t)next_slot[key]++;
        h.loc[tpos[e]] = (int32_t)qe;
    }
}

// Destination-sorted CSR.  Row v lists every edge incident to v in ascending edge id;
// an edge that is a self loop appears twice, source side first.  This is the order in
// which SequentialAggregator visits the output buffer (src/aggregators.jl:140-151 over
// the map of src/aggregators.jl:58-79: out ranges are laid out per edge as src then dst,
// src/network_structure.jl:240-250), so a sequential per-row sum reproduces it bitwise.
int build_topology(int64_t nv, int64_t ne, const int64_t* src, const int64_t* dst, int edge_elem,
                   Topology* topo) {
    if (nv <= 0) return fail(ND_ERR_ARG, "network has no vertices");
    if (ne < 0) return fail(ND_ERR_ARG, "negative edge count");
    if (nv > INT32_MAX - 1) return fail(ND_ERR_UNSUPPORTED, "more than 2^31-2 vertices");
    if (ne > (int64_t)(INT32_MAX)) return fail(ND_ERR_UNSUPPORTED, "more than 2^31-1 edges");
    if (2 * ne > (int64_t)UINT32_MAX) return fail(ND_ERR_UNSUPPORTED, "more than 2^32-1 incidences");
    if (ne > 0 && (!src || !dst)) return fail(ND_ERR_ARG, "src/dst pointers are NULL");

    std::vector<uint32_t> deg(nv + 1, 0);
    for (int64_t e = 0; e < ne; ++e) {
        int64_t s = src[e], d = dst[e];
        if (s < 0 || s >= nv || d < 0 || d >= nv) {
            char buf[160];
            snprintf(buf, sizeof buf, "edge %lld has endpoint out of range (%lld => %lld, nv=%lld)",
                     (long long)e, (long long)s, (long long)d, (long long)nv);
            return fail(ND_ERR_ARG, buf);
        }
        deg[s]++;
        deg[d]++;
    }
    std::vector<uint32_t> row_ptr(nv + 1);
    row_ptr[0] = 0;
    uint32_t maxdeg = 0;
    for (int64_t v = 0; v < nv; ++v) {
        row_ptr[v + 1] = row_ptr[v] + deg[v];
        maxdeg = std::max(maxdeg, deg[v]);
    }
    std::vector<Incidence> incid((size_t)2 * ne);
    std::vector<uint32_t> fill(row_ptr.begin(), row_ptr.end() - 1);
    for (int64_t e = 0; e < ne; ++e) {
        int32_t s = (int32_t)src[e], d = (int32_t)dst[e];
        incid[fill[s]++] = Incidence{d, (int32_t)e | kSrcSideBit};  // s receives y_src
        incid[fill[d]++] = Incidence{s, (int32_t)e};                // d receives y_dst
    }
    // Degree buckets (see nd_internal.h).  The windowed rows, medium rows by degree then
    // light rows in runs of consecutive vertices, are cut into windows of at most kWindow
    // rows and kWindowIncidences incidences and sorted by degree (descending, stable)
    // inside each window.
    std::vector<int32_t> light, medium, heavy;
    light.reserve(nv);
    for (int64_t v = 0; v < nv; ++v) {
        if (deg[v] <= (uint32_t)kLightMaxDeg) light.push_back((int32_t)v);
        else if (deg[v] <= (uint32_t)kMediumMaxDeg) medium.push_back((int32_t)v);
        else heavy.push_back((int32_t)v);
    }
    auto by_degree = [&](int32_t a, int32_t b) { return deg[a] > deg[b]; };
    std::stable_sort(medium.begin(), medium.end(), by_degree);
    std::stable_sort(heavy.begin(), heavy.end(), by_degree);
    // Light rows by degree inside runs of kLightRun consecutive vertices: the rows of a warp
    // then have (nearly) equal length, so their per-thread sums keep all lanes busy, while
    // du and u accesses stay within the run.
    for (size_t r0 = 0; r0 < light.size(); r0 += (size_t)kLightRun)
        std::stable_sort(light.begin() + r0, light.begin() + std::min(light.size(), r0 + (size_t)kLightRun), by_degree);
    std::vector<int32_t> windowed;
    windowed.reserve(medium.size() + light.size());
    windowed.insert(windowed.end(), medium.begin(), medium.end());
    windowed.insert(windowed.end(), light.begin(), light.end());
    std::vector<int32_t> win_ptr;  // slot offsets within the windowed part
    win_ptr.push_back(0);
    {
        size_t w0 = 0;
        uint32_t inc = 0;
        for (size_t i = 0; i < windowed.size(); ++i) {
            const uint32_t d = deg[windowed[i]];
            // windows never mix medium and light rows
            if (i - w0 == (size_t)kWindow || inc + d > (uint32_t)kWindowIncidences || (i == medium.size() && i > w0)) {
                std::stable_sort(windowed.begin() + w0, windowed.begin() + i, by_degree);
                win_ptr.push_back((int32_t)i);
                w0 = i;
                inc = 0;
            }
            inc += d;
        }
        if (w0 < windowed.size()) {
            std::stable_sort(windowed.begin() + w0, windowed.end(), by_degree);
            win_ptr.push_back((int32_t)windowed.size());
        }
    }
    // Slot order: heavy rows, then the windows.
    std::vector<int32_t> slot_vertex;
    slot_vertex.reserve(nv);
    slot_vertex.insert(slot_vertex.end(), heavy.begin(), heavy.end());
    slot_vertex.insert(slot_vertex.end(), windowed.begin(), windowed.end());
    std::vector<uint32_t> slot_ptr(nv + 1);
    std::vector<Incidence> sincid((size_t)2 * ne);
    slot_ptr[0] = 0;
    for (int64_t s = 0; s < nv; ++s) {
        const int32_t v = slot_vertex[s];
        const uint32_t b = row_ptr[v], n = deg[v];
        std::copy(incid.begin() + b, incid.begin() + b + n, sincid.begin() + slot_ptr[s]);
        slot_ptr[s + 1] = slot_ptr[s] + n;
    }

    Topology t;
    t.nv = nv;
    t.ne = ne;
    t.max_degree = (int32_t)maxdeg;
    t.n_light = (int32_t)light.size();
    t.n_medium = (int32_t)medium.size();
    t.n_heavy = (int32_t)heavy.size();
    t.n_windows = (int32_t)win_ptr.size() - 1;
    auto upload = [&](void** dptr, const void* hptr, size_t bytes) -> cudaError_t {
        cudaError_t err = cudaMalloc(dptr, std::max<size_t>(bytes, 16));
        if (err != cudaSuccess) return err;
        if (bytes) err = cudaMemcpy(*dptr, hptr, bytes, cudaMemcpyHostToDevice);
        return err;
    };
    cudaError_t err;
    if ((err = upload((void**)&t.slot_ptr, slot_ptr.data(), slot_ptr.size() * sizeof(uint32_t))) != cudaSuccess ||
        (err = upload((void**)&t.slot_vertex, slot_vertex.data(), slot_vertex.size() * sizeof(int32_t))) !=
            cudaSuccess ||
        (err = upload((void**)&t.incid, sincid.data(), sincid.size() * sizeof(Incidence))) != cudaSuccess ||
        (err = upload((void**)&t.win_ptr, win_ptr.data(), win_ptr.size() * sizeof(int32_t))) != cudaSuccess) {
        free_topology(&t);
        return cuda_fail(err, "upload of the network topology");
    }
    if (edge_elem > 0 && ne > 0 && is_canonical(ne, src, dst)) {
        EdgeLayoutHost h;
        build_edge_layout(nv, ne, src, dst, h);
        // the row records and the padded loc array, in slot order of the rows
        std::vector<int64_t> lstart(nv + 1, 0);
        for (int64_t v = 0; v < nv; ++v) lstart[v + 1] = lstart[v] + ((h.dptr[v + 1] - h.dptr[v] + 3) & ~3u);
        if (lstart[nv] > (int64_t)INT32_MAX) {
            free_topology(&t);
            return fail(ND_ERR_UNSUPPORTED, "padded destination-side index array above 2^31-1 entries");
        }
        std::vector<int32_t> locp((size_t)std::max<int64_t>(lstart[nv], 4), 0);
        for (int64_t v = 0; v < nv; ++v)
            for (uint32_t k = h.dptr[v]; k < h.dptr[v + 1]; ++k) locp[lstart[v] + (k - h.dptr[v])] = h.loc[k];
        std::vector<int4> rmeta(nv, int4{0, 0, 0, 0});
        for (int64_t sl = t.n_heavy; sl < nv; ++sl) {
            const int32_t v = slot_vertex[sl];
            const uint32_t nd = h.dptr[v + 1] - h.dptr[v], ns = h.sptr[v + 1] - h.sptr[v];
            rmeta[sl] = int4{v, (int32_t)lstart[v], (int32_t)h.sptr[v], (int32_t)(nd | (ns << 16))};
        }
        EdgeLayout& el = t.edge;
        el.n_chunks = h.n_chunks;
        if ((err = upload((void**)&el.esrc, h.esrc.data(), h.esrc.size() * sizeof(int32_t))) != cudaSuccess ||
            (err = upload((void**)&el.edst, h.edst.data(), h.edst.size() * sizeof(int32_t))) != cudaSuccess ||
            (err = upload((void**)&el.lslot, h.lslot.data(), h.lslot.size() * sizeof(uint16_t))) != cudaSuccess ||
            (err = upload((void**)&el.run_start, h.run_start.data(), h.run_start.size() * sizeof(uint16_t))) !=
                cudaSuccess ||
            (err = upload((void**)&el.run_base, h.run_base.data(), h.run_base.size() * sizeof(int32_t))) !=
                cudaSuccess ||
            (err = upload((void**)&el.rmeta, rmeta.data(), rmeta.size() * sizeof(int4))) != cudaSuccess ||
            (err = upload((void**)&el.locp, locp.data(), locp.size() * sizeof(int32_t))) != cudaSuccess ||
            (err = cudaMalloc(&el.y, (size_t)(ne + 2) * edge_elem)) != cudaSuccess ||
            (err = cudaMemset(el.y, 0, (size_t)(ne + 2) * edge_elem)) != cudaSuccess ||
            (err = cudaMalloc(&el.ybkt, (size_t)ne * edge_elem)) != cudaSuccess) {
            free_topology(&t);
            return cuda_fail(err, "upload of the edge-centric layout");
        }
        int64_t inc_medium = 0, inc_light = 0;
        for (int32_t v : medium) inc_medium += deg[v];
        for (int32_t v : light) inc_light += deg[v];
        el.dense_rows = inc_medium > inc_light;
        int32_t nw32 = 0;  // medium rows are sorted by degree, longest first
        while (nw32 < (int32_t)medium.size() && deg[medium[nw32]] >= (uint32_t)kWarpRowMinF32) ++nw32;
        el.n_warp_f32 = nw32;
        el.enabled = true;
    }
    *topo = t;
    return ND_OK;
}

cudaEvent_t Tracer::event() {
    if (next == pool.size()) {
        cudaEvent_t ev = nullptr;
        if (cudaEventCreate(&ev) != cudaSuccess) return nullptr;
        pool.push_back(ev);
    }
    return pool[next++];
}

void Tracer::release() {
    for (cudaEvent_t ev : pool) cudaEventDestroy(ev);
    pool.clear();
    marks.clear();
    next = 0;
}

// Count one launch of kind `kind` and, with timing on, bracket it with two events on `s`.
template <typename F>
static cudaError_t traced(nd_handle* h, int kind, cudaStream_t s, F&& launch) {
    Tracer& tr = h->tracer;
    ++tr.launches[kind];
    if (!tr.timing) return launch();
    cudaEvent_t start = tr.event(), stop = tr.event();
    if (!start || !stop) return cudaErrorMemoryAllocation;
    cudaError_t err = cudaEventRecord(start, s);
    if (err == cudaSuccess) err = launch();
    if (err == cudaSuccess) err = cudaEventRecord(stop, s);
    if (err == cudaSuccess) tr.marks.push_back({kind, start, stop});
    return err;
}

}  // namespace nd

using namespace nd;

extern "C" {

int nd_version(void) { return ND_VERSION; }

const char* nd_last_error(void) { return g_last_error.c_str(); }

}  // extern "C"

namespace nd {

// A handle with its side stream and fork / join events (no network yet).
static int new_handle(int dtype, nd_handle** out) {
    nd_handle* h = new nd_handle();
    h->dtype = dtype;
    h->sum_order = ND_ORDER_SEQUENTIAL;
    h->rhs_mode = kModeExact;
    h->edge_path = 1;
    // FP64 heavy rows run on a high-priority side stream, so that their blocks take the first
    // SM slots that edge-phase blocks free (see launch_heavy_solo in nd_rhs.cu)
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (cudaStreamCreateWithPriority(&h->side, cudaStreamNonBlocking, dtype == ND_F64 ? prio_hi : prio_lo) !=
            cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        cudaError_t err = cudaGetLastError();
        if (h->side) cudaStreamDestroy(h->side);
        if (h->ev_fork) cudaEventDestroy(h->ev_fork);
        delete h;
        return cuda_fail(err, "nd_create: stream / event creation");
    }
    cudaGetDevice(&h->device);
    *out = h;
    return ND_OK;
}

static void delete_handle(nd_handle* h) {
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->side) cudaStreamDestroy(h->side);
    delete h;
}

// The homogeneous kernels (nd_rhs_edge.cu, nd_rhs.cu) cover one vertex batch of kinds 1-3
// with one static edge batch whose source output is -y_dst: AntiSymmetric, or the
// two-sided diffusionedge_fid!, which computes the same values.
static bool homogeneous_kinds(int vk, int ek, int coupling) {
    return vk >= ND_V_DIFFUSION && vk <= ND_V_SWING && ek >= ND_E_DIFFUSION && ek <= ND_E_KURAMOTO &&
           (coupling == ND_ANTISYMMETRIC || (coupling == ND_FIDUCIAL && ek == ND_E_DIFFUSION));
}

static int create_batched(const nd_batched_network_desc* d, int dtype, nd_handle** out) {
    int rc = validate_batched(d);  // before any device resource
    if (rc != ND_OK) return rc;
    nd_handle* h = nullptr;
    rc = new_handle(dtype, &h);
    if (rc != ND_OK) return rc;
    rc = build_batched(d, dtype == ND_F64 ? 8 : 4, &h->batched);
    if (rc != ND_OK) {
        delete_handle(h);
        return rc;
    }
    const BatchedNet& b = h->batched;
    h->vertex_kind = b.vb.n == 1 ? b.vb.kind[0] : 0;
    h->edge_kind = b.eb.n == 1 ? b.eb.kind[0] : 0;
    h->coupling = b.eb.n == 1 ? b.eb.coupling[0] : 0;
    h->dim = b.dim;
    h->pdim = b.pdim;
    h->topo.nv = b.nv;
    h->topo.ne = b.ne;
    h->topo.max_degree = b.max_degree;
    *out = h;
    return ND_OK;
}

}  // namespace nd

extern "C" {

int nd_create(const nd_network_desc* desc, int dtype, nd_handle** out) {
    clear_error();
    ND_NVTX("nd_create");
    if (!desc || !out) return fail(ND_ERR_ARG, "nd_create: NULL descriptor or output pointer");
    *out = nullptr;
    if (dtype != ND_F32 && dtype != ND_F64)
        return fail(ND_ERR_DTYPE, "nd_create: dtype must be ND_F32 or ND_F64 "
                                  "(adapt the network with CuArray{Float32} or CuArray{Float64})");
    if (desc->vertex_kind < ND_V_DIFFUSION || desc->vertex_kind > ND_V_GENERATOR)
        return fail(ND_ERR_UNSUPPORTED_COMPONENT,
                    "vertex model is not in the GB300 component library "
                    "(diffusion, kuramoto first order, swing); no CPU fallback exists");
    int rc = check_edge_component(desc->edge_kind, desc->coupling);
    if (rc != ND_OK) return rc;
    if (desc->flags != 0) return fail(ND_ERR_ARG, "nd_network_desc.flags must be 0");
    if (!homogeneous_kinds(desc->vertex_kind, desc->edge_kind, desc->coupling)) {
        // one vertex batch and one edge batch on the batched path
        if (desc->nv <= 0) return fail(ND_ERR_ARG, "network has no vertices");
        if (desc->ne < 0) return fail(ND_ERR_ARG, "negative edge count");
        std::vector<int32_t> vb((size_t)desc->nv, 0), eb((size_t)std::max<int64_t>(desc->ne, 0), 0);
        nd_batch vbatch{desc->vertex_kind, 0}, ebatch{desc->edge_kind, desc->coupling};
        nd_batched_network_desc d{};
        d.nv = desc->nv;
        d.ne = desc->ne;
        d.src = desc->src;
        d.dst = desc->dst;
        d.n_vertex_batches = 1;
        d.n_edge_batches = 1;
        d.vertex_batches = &vbatch;
        d.edge_batches = &ebatch;
        d.vertex_batch = vb.data();
        d.edge_batch = eb.data();
        return create_batched(&d, dtype, out);
    }

    nd_handle* h = nullptr;
    rc = new_handle(dtype, &h);
    if (rc != ND_OK) return rc;
    h->vertex_kind = desc->vertex_kind;
    h->edge_kind = desc->edge_kind;
    h->coupling = desc->coupling;
    h->dim = desc->nv * vertex_dim(desc->vertex_kind);
    h->pdim = desc->nv * vertex_pdim(desc->vertex_kind) + desc->ne * edge_pdim(desc->edge_kind);
    rc = build_topology(desc->nv, desc->ne, desc->src, desc->dst, dtype == ND_F64 ? 8 : 4, &h->topo);
    if (rc != ND_OK) {
        delete_handle(h);
        return rc;
    }
    *out = h;
    return ND_OK;
}

int nd_create_batched(const nd_batched_network_desc* desc, int dtype, nd_handle** out) {
    clear_error();
    ND_NVTX("nd_create_batched");
    if (!desc || !out) return fail(ND_ERR_ARG, "nd_create_batched: NULL descriptor or output pointer");
    *out = nullptr;
    if (dtype != ND_F32 && dtype != ND_F64)
        return fail(ND_ERR_DTYPE, "nd_create_batched: dtype must be ND_F32 or ND_F64 "
                                  "(adapt the network with CuArray{Float32} or CuArray{Float64})");
    // one batch of each kind on the homogeneous kernels: the same layout, faster kernels
    if (desc->n_vertex_batches == 1 && desc->n_edge_batches <= 1 && desc->vertex_batches && desc->flags == 0 &&
        (desc->n_edge_batches == 0 ? desc->ne == 0 : desc->edge_batches != nullptr)) {
        const nd_batch vb = desc->vertex_batches[0];
        const nd_batch eb = desc->n_edge_batches ? desc->edge_batches[0] : nd_batch{ND_E_DIFFUSION_UNIT, ND_ANTISYMMETRIC};
        bool ids_ok = desc->vertex_batch != nullptr && (desc->ne == 0 || desc->edge_batch != nullptr);
        for (int64_t v = 0; ids_ok && v < desc->nv; ++v) ids_ok = desc->vertex_batch[v] == 0;
        for (int64_t e = 0; ids_ok && e < desc->ne; ++e) ids_ok = desc->edge_batch[e] == 0;
        if (ids_ok && vb.coupling == 0 && homogeneous_kinds(vb.kind, eb.kind, eb.coupling)) {
            nd_network_desc d{desc->nv, desc->ne, desc->src, desc->dst, vb.kind, eb.kind, eb.coupling, 0};
            return nd_create(&d, dtype, out);
        }
    }
    return create_batched(desc, dtype, out);
}

int nd_destroy(nd_handle* h) {
    clear_error();
    if (!h) return ND_OK;
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != h->device) cudaSetDevice(h->device);
    if (h->side) cudaStreamSynchronize(h->side);
    if (h->batched.enabled) free_batched(&h->batched);
    else free_topology(&h->topo);
    free_jacobian(&h->jac);
    h->tracer.release();
    const int dev = h->device;
    delete_handle(h);
    if (prev >= 0 && prev != dev) cudaSetDevice(prev);
    return ND_OK;
}

int nd_get_info(const nd_handle* h, nd_info* out) {
    clear_error();
    if (!h || !out) return fail(ND_ERR_ARG, "nd_get_info: NULL argument");
    out->dim = h->dim;
    out->pdim = h->pdim;
    out->nv = h->topo.nv;
    out->ne = h->topo.ne;
    out->n_incidences = 2 * h->topo.ne;
    out->dtype = h->dtype;
    out->vertex_kind = h->vertex_kind;
    out->edge_kind = h->edge_kind;
    out->max_degree = h->topo.max_degree;
    out->n_hubs = h->batched.enabled ? (int32_t)h->batched.n_warp_rows : h->topo.n_medium + h->topo.n_heavy;
    out->sum_order = h->sum_order;
    out->n_vertex_batches = h->batched.enabled ? h->batched.vb.n : 1;
    out->n_edge_batches = h->batched.enabled ? h->batched.eb.n : 1;
    return ND_OK;
}

int nd_set_sum_order(nd_handle* h, int order) {
    clear_error();
    if (!h) return fail(ND_ERR_ARG, "nd_set_sum_order: NULL handle");
    if (order != ND_ORDER_SEQUENTIAL && order != ND_ORDER_TREE && order != ND_ORDER_SEQUENTIAL_HW)
        return fail(ND_ERR_ARG, "nd_set_sum_order: unknown order");
    h->sum_order = order;
    h->rhs_mode = order == ND_ORDER_TREE ? kModeTree : (order == ND_ORDER_SEQUENTIAL_HW ? kModeNative : kModeExact);
    return ND_OK;
}

int nd_set_layout(nd_handle* h, int layout) {
    clear_error();
    if (!h) return fail(ND_ERR_ARG, "nd_set_layout: NULL handle");
    if (layout != ND_LAYOUT_AUTO && layout != ND_LAYOUT_FUSED) return fail(ND_ERR_ARG, "nd_set_layout: unknown layout");
    h->edge_path = layout == ND_LAYOUT_AUTO;
    return ND_OK;
}

int nd_rhs(nd_handle* h, int dtype, void* du, int64_t n_du, const void* u, int64_t n_u, const void* p,
           int64_t n_p, double t, void* stream) {
    ND_NVTX("nd_rhs");
    (void)t;
    clear_error();
    if (!h) return fail(ND_ERR_ARG, "nd_rhs: NULL handle");
    if (dtype != h->dtype) {
        const char* have = h->dtype == ND_F64 ? "Float64" : "Float32";
        const char* got = dtype == ND_F64 ? "Float64" : (dtype == ND_F32 ? "Float32" : "an unknown type");
        return fail(ND_ERR_DTYPE, std::string("Network caches are initialized with ") + have +
                                      " but is used for " + got + " data");
    }
    if (n_du != h->dim || n_u != h->dim) {
        return fail(ND_ERR_ARG, "du or u does not have expected size " + std::to_string(h->dim));
    }
    if (h->pdim > 0 && n_p != h->pdim) {
        return fail(ND_ERR_ARG, "p does not has expected size " + std::to_string(h->pdim));
    }
    if (!du || !u || (h->pdim > 0 && !p)) return fail(ND_ERR_ARG, "nd_rhs: NULL buffer");
    cudaStream_t s = (cudaStream_t)stream;
    if (h->batched.enabled) {
        const BatchedNet& b = h->batched;
        cudaError_t err = cudaSuccess;
        if (b.ne > 0)
            err = traced(h, kKernelBatchedEdges, s,
                         [&] { return launch_batched(h->dtype, b, du, u, p, h->rhs_mode, s, kPhaseEdge); });
        if (err == cudaSuccess)
            err = traced(h, kKernelBatchedRows, s,
                         [&] { return launch_batched(h->dtype, b, du, u, p, h->rhs_mode, s, kPhaseRow); });
        return err == cudaSuccess ? ND_OK : cuda_fail(err, "nd_rhs kernel launch");
    }
    RhsArgs a;
    a.du = du;
    a.u = u;
    a.p = p;
    a.nv = h->topo.nv;
    a.slot_ptr = h->topo.slot_ptr;
    a.slot_vertex = h->topo.slot_vertex;
    a.incid = h->topo.incid;
    a.win_ptr = h->topo.win_ptr;
    a.n_light = h->topo.n_light;
    a.n_medium = h->topo.n_medium;
    a.n_heavy = h->topo.n_heavy;
    a.n_windows = h->topo.n_windows;
    a.vertex_kind = h->vertex_kind;
    a.edge_kind = h->edge_kind;
    a.mode = h->rhs_mode;
    const EdgeLayout& el = h->topo.edge;
    a.ne = h->topo.ne;
    a.n_chunks = el.n_chunks;
    a.esrc = el.esrc;
    a.edst = el.edst;
    a.lslot = el.lslot;
    a.run_start = el.run_start;
    a.run_base = el.run_base;
    a.rmeta = el.rmeta;
    a.locp = el.locp;
    a.y = el.y;
    a.ybkt = el.ybkt;
    a.heavy_only = 0;
    a.heavy_separate = 0;
    a.dense_rows = el.dense_rows ? 1 : 0;
    a.n_warp_f32 = el.n_warp_f32;
    const bool edge = el.enabled && h->edge_path;
    const bool split = h->topo.n_heavy > 0;  // heavy rows: their own kernel, on the side stream
    a.heavy_separate = split ? 1 : 0;
    const int64_t main_rows = (split ? 0 : h->topo.n_heavy) + h->topo.n_windows;
    cudaError_t err = cudaSuccess;
    if (split) {
        // Heavy rows run concurrently on the handle's side stream, one per SM, computed
        // from u and p directly (they need nothing from the other kernels); fork / join
        // with events so the call stays ordered on the caller's stream (and capturable).
        RhsArgs hv = a;
        hv.heavy_only = 1;
        if ((err = cudaEventRecord(h->ev_fork, s)) != cudaSuccess ||
            (err = cudaStreamWaitEvent(h->side, h->ev_fork, 0)) != cudaSuccess ||
            (err = traced(h, kKernelHeavyRows, h->side, [&] { return launch_rhs(h->dtype, hv, h->side); })) !=
                cudaSuccess)
            return cuda_fail(err, "nd_rhs kernel launch");
    }
    if (edge) {
        if (el.n_chunks > 0)
            err = traced(h, kKernelEdgePhase, s, [&] { return launch_rhs_edge(h->dtype, a, s, kPhaseEdge); });
        if (err == cudaSuccess && main_rows > 0)
            err = traced(h, kKernelRowPhase, s, [&] { return launch_rhs_edge(h->dtype, a, s, kPhaseRow); });
    } else if (main_rows > 0) {
        err = traced(h, kKernelFused, s, [&] { return launch_rhs(h->dtype, a, s); });
    }
    if (err == cudaSuccess && split) {
        if ((err = cudaEventRecord(h->ev_join, h->side)) == cudaSuccess) err = cudaStreamWaitEvent(s, h->ev_join, 0);
    }
    if (err != cudaSuccess) return cuda_fail(err, "nd_rhs kernel launch");
    return ND_OK;
}

int nd_set_kernel_timing(nd_handle* h, int on) {
    clear_error();
    if (!h) return fail(ND_ERR_ARG, "nd_set_kernel_timing: NULL handle");
    h->tracer.timing = on != 0;
    return ND_OK;
}

int nd_kernel_times(nd_handle* h, int64_t* launches, double* ms, int n) {
    clear_error();
    if (!h || n < 0 || (n > 0 && (!launches || !ms))) return fail(ND_ERR_ARG, "nd_kernel_times: bad arguments");
    double total[kKernelKinds] = {};
    for (const Tracer::Mark& m : h->tracer.marks) {
        float t = 0.f;
        cudaError_t err = cudaEventSynchronize(m.stop);
        if (err == cudaSuccess) err = cudaEventElapsedTime(&t, m.start, m.stop);
        if (err != cudaSuccess) return cuda_fail(err, "nd_kernel_times");
        total[m.kind] += t;
    }
    for (int k = 0; k < n; ++k) {
        launches[k] = k < kKernelKinds ? h->tracer.launches[k] : 0;
        ms[k] = k < kKernelKinds ? total[k] : 0.0;
    }
    for (int k = 0; k < kKernelKinds; ++k) h->tracer.launches[k] = 0;
    h->tracer.marks.clear();
    h->tracer.next = 0;
    return ND_OK;
}

}  // extern "C"

// ----------------------------------------------------------------------------------------
// Diagnostic entry points (include/nd_gb300_selftest.h).
extern "C" {

int nd_selftest_exact_add(const double* a, const double* b, double* out, int64_t n, void* stream) {
    clear_error();
    if (n < 0 || (n > 0 && (!a || !b || !out))) return fail(ND_ERR_ARG, "nd_selftest_exact_add: bad arguments");
    cudaError_t err = launch_exact_selftest(a, b, out, n, (cudaStream_t)stream);
    return err == cudaSuccess ? ND_OK : cuda_fail(err, "nd_selftest_exact_add");
}

int nd_selftest_exact_scan(const double* terms, const int64_t* seg, const double* s0, double* out, int64_t nseg,
                           void* stream) {
    clear_error();
    if (nseg < 0 || (nseg > 0 && (!terms || !seg || !s0 || !out)))
        return fail(ND_ERR_ARG, "nd_selftest_exact_scan: bad arguments");
    cudaError_t err = launch_scan_selftest(terms, seg, s0, out, nseg, (cudaStream_t)stream);
    return err == cudaSuccess ? ND_OK : cuda_fail(err, "nd_selftest_exact_scan");
}

}  // extern "C"
