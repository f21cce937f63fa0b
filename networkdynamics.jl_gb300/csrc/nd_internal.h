// Internal declarations shared by the translation units of libnd_b200.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "nd_gb300.h"

namespace nd {

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
inline int vertex_dim(int vk) { return vk == ND_V_SWING ? 2 : 1; }
inline int vertex_pdim(int vk) { return vk == ND_V_DIFFUSION ? 0 : (vk == ND_V_KURAMOTO ? 1 : 3); }
inline int edge_pdim(int ek) { return ek == ND_E_DIFFUSION_UNIT ? 0 : 1; }

// Degree-bucket thresholds.  Rows with degree <= kThreadMaxDeg run thread-per-vertex,
// rows above it run on the cooperative hub path (a warp per row).
constexpr int kThreadMaxDeg = 32;

// Device-resident topology of one network.
struct Topology {
    int64_t nv = 0, ne = 0;
    int32_t max_degree = 0;
    uint32_t* row_ptr = nullptr;     // [nv+1] offsets into incid
    Incidence* incid = nullptr;      // [2ne]
    int32_t* light = nullptr;        // [n_light] vertices on the thread-per-vertex path, ascending
    int32_t* hubs = nullptr;         // [n_hubs] vertices on the cooperative path, by degree desc
    int32_t n_light = 0, n_hubs = 0;
};

// Build the CSR on the host and upload it.  src/dst are 0-based host arrays.
int build_topology(int64_t nv, int64_t ne, const int64_t* src, const int64_t* dst, Topology* topo);
void free_topology(Topology* topo);

struct RhsArgs {
    void* du;
    const void* u;
    const void* p;
    int64_t nv;
    const uint32_t* row_ptr;
    const Incidence* incid;
    const int32_t* light;
    const int32_t* hubs;
    int32_t n_light, n_hubs;
    int32_t vertex_kind, edge_kind;
    int32_t sum_order;
    int32_t kahan_min_degree;  // F32: compensated sums on rows at least this long
};

// Launch the fused RHS for the given element type.
cudaError_t launch_rhs(int dtype, const RhsArgs& a, cudaStream_t stream);

}  // namespace nd

struct nd_handle {
    int dtype;
    int vertex_kind, edge_kind, coupling;
    int sum_order;
    int kahan_min_degree;
    int device;
    int64_t dim, pdim;
    nd::Topology topo;
};
