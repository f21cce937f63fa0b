// Internal declarations shared by the translation units of libnd_b200.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "nd_gb300.h"

namespace nd {

// NVTX range around a C-ABI call: the call shows up by name on a profiler's timeline
// (Nsight Systems / Compute); without a tool attached a push / pop is a branch on a null
// function pointer.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};
#define ND_NVTX(name) ::nd::NvtxRange nd_nvtx_range_(name)

// Thread-local error message behind nd_last_error().
void set_error(const std::string& msg);
void clear_error();
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t err, const char* what);

#define ND_CUDA_TRY(expr)                                  \
    do {                                                   \
        cudaError_t _e = (expr);                           \
        if (_e != cudaSuccess) return nd::cuda_fail(_e, #expr); \
    } while (0)

// Incidence of the destination-sorted CSR: the neighbour and the edge id, with bit 31 of
// `eid` set when the row's vertex is the *source* of the edge (it then receives y_src).
struct __align__(8) Incidence {
    int32_t nbr;
    int32_t eid;
};
constexpr int32_t kSrcSideBit = int32_t(0x80000000u);

// Dimensions of the library components.
inline int vertex_dim(int vk) {
    return vk == ND_V_GENERATOR ? 4
                                : (vk == ND_V_SWING || vk == ND_V_SWING_UNIT || vk == ND_V_PQ || vk == ND_V_PQ_CONST ? 2 : 1);
}
inline int vertex_pdim(int vk) {
    switch (vk) {
        case ND_V_DIFFUSION: case ND_V_PQ_CONST: return 0;
        case ND_V_KURAMOTO: case ND_V_SWING_UNIT: return 1;
        case ND_V_SWING: return 3;
        case ND_V_PQ: return 2;
        default: return 11;  // ND_V_GENERATOR
    }
}
inline int edge_dim(int ek) { return ek == ND_E_DIFFUSION_ODE || ek == ND_E_DIFFUSION_ODE_FIXED ? 2 : 0; }
inline int edge_pdim(int ek) {
    return ek == ND_E_DIFFUSION_UNIT || ek == ND_E_DIFFUSION_ODE_FIXED ? 0 : (ek == ND_E_PILINE ? 4 : 1);
}
// output dimension (vdepth / edepth)
inline int vertex_outdim(int vk) { return vk == ND_V_PQ || vk == ND_V_GENERATOR || vk == ND_V_PQ_CONST ? 2 : 1; }
inline int edge_outdim(int ek) { return ek == ND_E_PILINE ? 2 : 1; }

// Degree buckets.  Rows with degree <= kMediumMaxDeg are processed in windows: a block
// evaluates all edge terms of up to kWindow rows / kWindowIncidences incidences in
// parallel, then sums one row per thread; rows are sorted by degree inside a window so
// the lanes of a warp walk rows of nearly equal length.  Medium rows (degree above
// kLightMaxDeg) come first, globally sorted by degree; light rows follow in runs of
// kLightRun consecutive vertices, sorted by degree inside each run.
// Longer rows (power-law hubs) get a block each and are summed by an exact parallel scan:
// a per-thread chain that long would wait on the shared FP64 pipe at every step.
constexpr int kLightMaxDeg = 32;
constexpr int kMediumMaxDeg = 2048;
constexpr int kWindow = 256;
constexpr int kWarpRowMinF32 = 128;  // FP32 rows at least this long take a warp in the row phase
constexpr int kLightRun = 128;

// Device-resident topology of one network.
// Rows are stored in processing order ("slots"): heavy rows (by degree, descending), then
// medium rows (by degree, descending), then the light windows, each window's rows sorted
// by degree.  slot_ptr indexes the incidences of a slot, slot_vertex names its vertex.
constexpr int kWindowIncidences = 2048;  // light window: at most this many incidences

// Edge-centric layout, used when the edge list is canonical: sorted by source with
// src < dst for every edge, the order Graphs.jl's edges(g) gives for a SimpleGraph.
// Then every row is [its dst-side edges, ascending] followed by [its own source block,
// a contiguous edge range], so the RHS can run in two phases:
//   E: each edge's value y_e = g(u_src, u_dst, p_e) once, in edge order, written to y
//      (edge order) and to ybkt, the same values grouped into kBuckets buckets of
//      destination-CSR positions: a block stages its chunk's values in shared memory in
//      (bucket, edge) order and writes each bucket's run of them as one contiguous piece;
//   R: each row sums its dst-side values (gathered from one bucket, which stays in L2
//      while the rows of that range run) and then -y over its source block; its position
//      in locp, its source block and both lengths come in one 16-byte record per slot.
// Each edge's function is evaluated once instead of twice, and the edge parameters and
// the incidence stream are read in order instead of gathered.
constexpr int kEdgeChunk = 2048;  // edges per phase-E block
constexpr int kBuckets = 64;

struct EdgeLayout {
    bool enabled = false;
    int64_t n_chunks = 0;
    int32_t* esrc = nullptr;   // [ne]
    int32_t* edst = nullptr;   // [ne]
    uint16_t* lslot = nullptr;     // [ne] slot of edge e in its chunk's (bucket, edge)-ordered staging
    uint16_t* run_start = nullptr;  // [n_chunks][kBuckets+1] first staging slot of each bucket's run
    int32_t* run_base = nullptr;    // [n_chunks][kBuckets] ybkt position of each bucket's run
    // per row slot (rows of degree <= kMediumMaxDeg; zero for the heavy slots): the vertex,
    // the row's first entry in locp, its source block's first edge, nd | ns << 16
    int4* rmeta = nullptr;
    // ybkt positions of every row's destination-side values, each row's run starting on a
    // multiple of 4 entries (padding entries hold 0), so they load as 16-byte vectors
    int32_t* locp = nullptr;
    void* y = nullptr;         // [ne + 2] scratch, element type of the handle (+2: pair loads)
    // rows of degree 33..kMediumMaxDeg carry most of the incidences (a dense graph): the
    // row phase takes its dense-network kernel
    bool dense_rows = false;
    int32_t n_warp_f32 = 0;  // medium rows of at least kWarpRowMinF32 terms (the first medium slots)
    void* ybkt = nullptr;      // [ne] scratch
};

struct Topology {
    int64_t nv = 0, ne = 0;
    int32_t max_degree = 0;
    uint32_t* slot_ptr = nullptr;    // [nv+1] offsets into incid, by slot
    int32_t* slot_vertex = nullptr;  // [nv] vertex of each slot
    Incidence* incid = nullptr;      // [2ne] incidences in slot order, each row by edge id (fused path)
    int32_t* win_ptr = nullptr;      // [n_windows+1] first slot of each light window
    int32_t n_light = 0, n_medium = 0, n_heavy = 0, n_windows = 0;
    EdgeLayout edge;
};

// Build the CSR on the host and upload it.  src/dst are 0-based host arrays.  The
// edge-centric layout is built too when the edge list is canonical and edge_elem > 0
// (the scratch element size, 4 or 8 bytes).
int build_topology(int64_t nv, int64_t ne, const int64_t* src, const int64_t* dst, int edge_elem,
                   Topology* topo);
void free_topology(Topology* topo);

// Accumulation modes of the FP64 RHS.
enum RhsMode : int32_t {
    kModeExact = 0,   // sequential order; integer-exact adds; hubs by exact scan (default)
    kModeNative = 1,  // sequential order; hardware DADD chains (reference timing mode)
    kModeTree = 2     // sequential order for short rows, warp tree at hubs (not bitwise)
};

struct RhsArgs {
    void* du;
    const void* u;
    const void* p;
    int64_t nv;
    const uint32_t* slot_ptr;
    const int32_t* slot_vertex;
    const Incidence* incid;
    const int32_t* win_ptr;
    int32_t n_light, n_medium, n_heavy, n_windows;
    int32_t vertex_kind, edge_kind;
    int32_t mode;
    int32_t heavy_only;      // launch_rhs: only the heavy rows, one per SM
    int32_t heavy_separate;  // heavy rows are launched separately (heavy_only), not by this launch
    // edge-centric layout (see EdgeLayout)
    int64_t ne, n_chunks;
    const int32_t* esrc;
    const int32_t* edst;
    const uint16_t* lslot;
    const uint16_t* run_start;
    const int32_t* run_base;
    const int4* rmeta;
    const int32_t* locp;
    void* y;
    void* ybkt;
    int32_t dense_rows;  // the row phase runs dense_row_kernel (see EdgeLayout::dense_rows)
    int32_t n_warp_f32;  // FP32: the first medium slots with >= kWarpRowMinF32 terms, a warp each
};

// Launch the fused RHS for the given element type.
cudaError_t launch_rhs(int dtype, const RhsArgs& a, cudaStream_t stream);
// Launch the two-phase (edge-centric) RHS: phase E, phase R or both (kPhase* bits).
enum : int { kPhaseEdge = 1, kPhaseRow = 2, kPhaseBoth = 3 };
cudaError_t launch_rhs_edge(int dtype, const RhsArgs& a, cudaStream_t stream, int phases = kPhaseBoth);

// Kernel kinds that nd_rhs launches, for launch counting and optional per-kernel timing.
enum KernelKind : int {
    kKernelEdgePhase = 0,
    kKernelRowPhase = 1,
    kKernelHeavyRows = 2,
    kKernelFused = 3,
    kKernelBatchedEdges = 4,
    kKernelBatchedRows = 5,
    kKernelKinds = 6
};

// ---- batched (heterogeneous) networks -------------------------------------------------------
// Batch table of one component class (vertices or edges).  Components are numbered by
// "position": their rank in the reference's batch-major order; batch b holds positions
// [pos0[b], pos0[b+1]), its states start at s0[b] with stride dim(kind), its parameters at
// p0[b] with stride pdim(kind) (the BatchStride of src/utils.jl:1-35).  consts holds
// kBatchConstants numbers per batch for components that close over values of their own
// (the PQ bus of pqnode_inhomogeneous).  Tables can hold many batches (one per component
// when every component is distinct), so the kernels read them from device memory.
constexpr int64_t kMaxBatches = ND_MAX_BATCHES;
constexpr int kBatchConstants = ND_BATCH_CONSTANTS;
struct BatchTable {
    int32_t n = 0;
    std::vector<int32_t> kind, coupling;
    std::vector<int64_t> pos0;  // n + 1 entries
    std::vector<int64_t> s0, p0;
    std::vector<double> consts;  // kBatchConstants per batch
};
// The device copy, passed to the kernels by value.
struct BatchTableDev {
    int32_t n = 0;
    const int32_t* kind = nullptr;
    const int32_t* coupling = nullptr;
    const int64_t* pos0 = nullptr;
    const int64_t* s0 = nullptr;
    const int64_t* p0 = nullptr;
    const double* consts = nullptr;
};

// Device data of a batched network.  Edge values go to y2, two per edge position k:
// y2[2k] = y_src, y2[2k+1] = y_dst -- the reference's output buffer for edges, which lays
// out src then dst per edge (src/network_structure.jl:240-250).  Every row lists the y2
// indices of its terms in ascending order, which is SequentialAggregator's order of
// additions (src/aggregators.jl:140-151).
struct BatchedNet {
    bool enabled = false;
    BatchTable vb, eb;                // host copies
    BatchTableDev dvb, deb;           // device copies, read by the kernels
    void* table_mem = nullptr;        // the device memory behind dvb and deb
    int64_t nv = 0, ne = 0, dim = 0, pdim = 0;
    int32_t max_degree = 0;
    int32_t depth = 1;           // output dimension of vertices and edge sides (2: complex)
    int64_t n_warp_rows = 0;     // slots [0, n_warp_rows): the long rows, a warp per row
    bool dense_rows = false;
    int32_t n_warp_f32 = 0;  // medium rows of at least kWarpRowMinF32 terms (the first medium slots)     // FP64 thread rows in deep batches (a dense network)
    int2* eu = nullptr;          // [ne] by edge position: u indices of the src / dst vertex outputs
    uint32_t* tptr = nullptr;    // [nv+1] by slot: range of the slot's terms in tidx
    int32_t* tidx = nullptr;     // [2ne] y2 indices of every row's terms, ascending
    int32_t* slot_vpos = nullptr;  // [nv] vertex position of each slot
    void* y2 = nullptr;          // [2ne·depth] scratch, element type of the handle
};

#ifdef __CUDACC__
// Batch of position `pos`: the last batch whose first position is <= pos, by binary search
// (an empty batch starts where the next one does, so it is never the answer).
__device__ __forceinline__ int find_batch(const BatchTableDev& t, int64_t pos) {
    int lo = 0, hi = t.n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(t.pos0 + mid) <= pos) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}
#endif
// The same on the host table.
inline int host_find_batch(const BatchTable& t, int64_t pos) {
    int lo = 0, hi = t.n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (t.pos0[mid] <= pos) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

int check_edge_component(int edge_kind, int coupling);  // ND_OK or ND_ERR_UNSUPPORTED_COMPONENT
// elem: scratch element size (4 / 8); 0 builds the structure without the y2 scratch (a
// view of a network for the Jacobian).  validate_batched runs every check on the host.
int validate_batched(const nd_batched_network_desc* d);
int build_batched(const nd_batched_network_desc* d, int elem, BatchedNet* out);
void free_batched(BatchedNet* b);
cudaError_t launch_batched(int dtype, const BatchedNet& b, void* du, const void* u, const void* p, int mode,
                           cudaStream_t s, int phases);

// Launch counter and CUDA-event timer for the kernels of one handle.  Timing is off by
// default; when on, each launch is bracketed by two events on its stream, and
// nd_kernel_times sums the bracketed durations.
struct Tracer {
    bool timing = false;
    int64_t launches[kKernelKinds] = {};
    struct Mark {
        int kind;
        cudaEvent_t start, stop;
    };
    std::vector<cudaEvent_t> pool;
    size_t next = 0;
    std::vector<Mark> marks;
    cudaEvent_t event();  // an event from the pool (created on demand), nullptr on failure
    void release();       // destroy every pooled event
};

// Restarted GMRES on a CSR matrix (nd_newton.cu), shared by the Newton fixpoint and the
// Rosenbrock solver.  attach() lays its workspace out in `buf` (doubles(n, m) doubles).
struct GmresSolver {
    int64_t n = 0;
    int m = 0;
    cudaStream_t s = nullptr;
    double *w = nullptr, *dinv = nullptr, *z = nullptr, *V = nullptr, *partial = nullptr, *dscal = nullptr;
    static size_t doubles(int64_t n, int m);
    void attach(double* buf, int64_t n, int m, cudaStream_t s);
    void jacobi(const int32_t* rowptr, const int32_t* col, const double* vals);  // D^-1 from the diagonal
    int solve(const int32_t* rowptr, const int32_t* col, const double* vals, const double* b, double* x, double rtol,
              int restarts, double* rel_res);
    int multidot(const double* V, int nv, const double* x, double* dots);
    int sync(const char* what);
};
void vec_axpby(int64_t n, double a, const double* x, double b, double* y, cudaStream_t s);  // y = a x + b y

cudaError_t launch_exact_selftest(const double* a, const double* b, double* out, int64_t n, cudaStream_t s);
cudaError_t launch_scan_selftest(const double* terms, const int64_t* seg, const double* s0, double* out,
                                 int64_t nseg, cudaStream_t s);

}  // namespace nd

namespace nd {
// Sparse Jacobian of a handle (nd_jacobian.cu): the CSR pattern of ∂f/∂u, built on first
// use, and for homogeneous handles the batched view of their network it is built from.
struct JacPlan {
    bool ready = false;
    BatchedNet view;  // homogeneous handles only (batched handles use their own)
    int64_t nnz = 0;
    std::vector<int32_t> rowptr_h, colidx_h;
    int32_t* rowptr = nullptr;  // device copies
    int32_t* colidx = nullptr;
    int32_t* long_slots = nullptr;  // slots of the rows that take a warp each
    int64_t n_long = 0;
    void* values = nullptr;         // Jacobian values kept for nd_jvp of batched handles
};
void free_jacobian(JacPlan* j);

}  // namespace nd

struct nd_handle {
    int dtype;
    int vertex_kind, edge_kind, coupling;
    int sum_order;
    int rhs_mode;
    int edge_path;  // use the two-phase layout when it exists (default on)
    int device;
    cudaStream_t side = nullptr;  // heavy rows run here, forked from / joined to the caller's stream
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int64_t dim, pdim;
    nd::Topology topo;
    nd::BatchedNet batched;  // enabled: the handle is a batched network (topo unused)
    nd::JacPlan jac;
    nd::Tracer tracer;
};
