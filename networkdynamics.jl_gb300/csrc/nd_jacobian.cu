// Sparse Jacobian ∂f/∂u of the network RHS: its CSR pattern and its analytic values.
//
// The reference gets the pattern by tracing the RHS with SparseConnectivityTracer
// (get_jac_prototype, ext/NetworkDynamicsSparsityExt.jl:57-127) and leaves the values to
// the solver's colored ForwardDiff passes.  For the component library both follow from the
// structure of the network:
//   vertex row  (the state that receives the aggregated input: u for diffusion / Kuramoto,
//               ω for the swing vertices): a column for the output of each endpoint of an
//               incident static edge whose output to this vertex is not identically zero,
//               and one for the state that an incident ODE edge outputs to it; the swing
//               rows add their own ω (dθ = ω, and -D/M or -1 in dω);
//   ODE edge    the two state rows of an ODE edge: the outputs of both endpoints and the
//               state itself.
// Columns are sorted and unique per row; a structural entry can be numerically zero (a
// self loop, whose two derivatives cancel), as in a traced pattern.
//
// Power grids (complex outputs): a vertex's rows have its own states (generators) and the
// voltage states of both endpoints of every incident line; the values come from dual
// numbers carried through the component functions (jac_powergrid_kernel).
//
// Values: one thread per vertex row of up to 32 terms adds its terms' derivatives into its
// row (found by binary search in the sorted columns), in the order of its terms; longer
// rows take a warp each; one thread per ODE edge writes that edge's two rows.  For simple
// graphs the result is deterministic.  Homogeneous handles
// get a batched view of their network (no scratch) built from their device topology.
#include <algorithm>
#include <string>
#include <vector>

#include "nd_components.cuh"
#include "nd_dual.cuh"
#include "nd_internal.h"

namespace nd {

namespace {

constexpr int kJacBlock = 128;

bool is_ode(int ek) { return ek == ND_E_DIFFUSION_ODE || ek == ND_E_DIFFUSION_ODE_FIXED; }
bool is_swing(int vk) { return vk == ND_V_SWING || vk == ND_V_SWING_UNIT; }


template <typename T>
struct JacArgs {
    T* values;
    const T* u;
    const T* p;
    const int32_t* rowptr;
    const int32_t* colidx;
    int64_t nv, ne;
    BatchTableDev vb, eb;
    const int2* eu;
    const uint32_t* tptr;
    const int32_t* tidx;
    const int32_t* slot_vpos;
};

// Add v at column c of the row whose columns are cols[0..n): binary search.  The pattern
// holds every column the kernels add to; a column that is not found is skipped.
template <typename T>
__device__ __forceinline__ void jadd(T* __restrict__ vals, const int32_t* __restrict__ cols, int n, int32_t c, T v) {
    if (n <= 0) return;
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(cols + mid) < c) lo = mid + 1;
        else hi = mid;
    }
    if (__ldg(cols + lo) == c) vals[lo] += v;
}

template <typename T>
__device__ __forceinline__ void jadd_atomic(T* __restrict__ vals, const int32_t* __restrict__ cols, int n, int32_t c,
                                            T v) {
    if (n <= 0) return;
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(cols + mid) < c) lo = mid + 1;
        else hi = mid;
    }
    if (__ldg(cols + lo) == c) atomicAdd(vals + lo, v);
}

// ∂g/∂vs and ∂g/∂vd of a static edge.
template <typename T>
__device__ __forceinline__ void static_edge_dg(int kind, T vs, T vd, T w, T& gs, T& gd) {
    using A = Arith<T>;
    if (kind == ND_E_DIFFUSION) {
        gs = w;
        gd = -w;
    } else if (kind == ND_E_DIFFUSION_UNIT) {
        gs = T(1);
        gd = T(-1);
    } else {
        const T c = A::mul(w, A::cos_phase(A::sub(vs, vd)));  // K cos(θs - θd)
        gs = c;
        gd = -c;
    }
}

// Rows with more terms than this take a warp each (jac_long_row_kernel).
constexpr uint32_t kJacLongRow = 32;

template <typename T>
__global__ void __launch_bounds__(kJacBlock) jac_vertex_kernel(JacArgs<T> a) {
    using A = Arith<T>;
    const int64_t slot = (int64_t)blockIdx.x * kJacBlock + threadIdx.x;
    if (slot >= a.nv) return;
    if (__ldg(a.tptr + slot + 1) - __ldg(a.tptr + slot) > kJacLongRow) return;
    const int64_t pos = __ldg(a.slot_vpos + slot);
    const int b = find_batch(a.vb, pos);
    const int vk = __ldg(a.vb.kind + b);
    const int64_t r = pos - __ldg(a.vb.pos0 + b);
    const int dim = vk == ND_V_SWING || vk == ND_V_SWING_UNIT ? 2 : 1;
    const int pd = vk == ND_V_DIFFUSION ? 0 : (vk == ND_V_SWING ? 3 : 1);
    const int64_t s = __ldg(a.vb.s0 + b) + dim * r, q = __ldg(a.vb.p0 + b) + pd * r;
    T scale = T(1);
    if (dim == 2) {
        // dθ = ω
        const int32_t r0 = __ldg(a.rowptr + s);
        jadd<T>(a.values + r0, a.colidx + r0, __ldg(a.rowptr + s + 1) - r0, (int32_t)(s + 1), T(1));
        if (vk == ND_V_SWING) {
            const T M = __ldg(a.p + q), D = __ldg(a.p + q + 1);
            scale = A::div(T(1), M);
            const int32_t r1 = __ldg(a.rowptr + s + 1);
            jadd<T>(a.values + r1, a.colidx + r1, __ldg(a.rowptr + s + 2) - r1, (int32_t)(s + 1), -A::mul(scale, D));
        } else {
            const int32_t r1 = __ldg(a.rowptr + s + 1);
            jadd<T>(a.values + r1, a.colidx + r1, __ldg(a.rowptr + s + 2) - r1, (int32_t)(s + 1), T(-1));
        }
    }
    const int64_t row = s + dim - 1;  // the row that receives the aggregated input
    const int32_t r0 = __ldg(a.rowptr + row);
    const int n = __ldg(a.rowptr + row + 1) - r0;
    T* vals = a.values + r0;
    const int32_t* cols = a.colidx + r0;
    const uint32_t t0 = __ldg(a.tptr + slot), t1 = __ldg(a.tptr + slot + 1);
    for (uint32_t j = t0; j < t1; ++j) {
        const int32_t t = __ldg(a.tidx + j);
        const int64_t k = t >> 1;
        const bool dst_side = t & 1;
        const int eb = find_batch(a.eb, k);
        const int ek = __ldg(a.eb.kind + eb);
        const int64_t re = k - __ldg(a.eb.pos0 + eb);
        if (ek == ND_E_DIFFUSION_ODE || ek == ND_E_DIFFUSION_ODE_FIXED) {
            // Fiducial(dst=1:1, src=2:2): this vertex receives e1 (destination) or e2 (source)
            const int64_t es = __ldg(a.eb.s0 + eb) + 2 * re + (dst_side ? 0 : 1);
            jadd<T>(vals, cols, n, (int32_t)es, scale);
            continue;
        }
        const int c = __ldg(a.eb.coupling + eb);
        if (!dst_side && c == ND_DIRECTED) continue;  // y_src = 0
        const int2 o = __ldg(a.eu + k);
        const T w = ek == ND_E_DIFFUSION_UNIT ? T(0) : __ldg(a.p + __ldg(a.eb.p0 + eb) + re);
        T gs, gd;
        static_edge_dg<T>(ek, __ldg(a.u + o.x), __ldg(a.u + o.y), w, gs, gd);
        // source side: y_src = -y_dst (AntiSymmetric, two-sided fiducial) or y_dst (Symmetric)
        const T f = dst_side || c == ND_SYMMETRIC ? scale : -scale;
        jadd<T>(vals, cols, n, o.x, A::mul(f, gs));
        jadd<T>(vals, cols, n, o.y, A::mul(f, gd));
    }
}

// The same for the rows of more than kJacLongRow terms, a warp each: the lanes take the
// terms in turn.  The derivatives with respect to the vertex's own output (one per term)
// are summed per lane and then across the warp; the neighbour columns are distinct in a
// simple graph, and are added atomically for the repeated ones of a multigraph.
template <typename T>
__global__ void __launch_bounds__(kJacBlock) jac_long_row_kernel(JacArgs<T> a, const int32_t* __restrict__ slots,
                                                                 int64_t n_long) {
    using A = Arith<T>;
    const int lane = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * kJacBlock + threadIdx.x) >> 5;
    if (w >= n_long) return;  // warp-uniform
    const int64_t slot = __ldg(slots + w);
    const int64_t pos = __ldg(a.slot_vpos + slot);
    const int b = find_batch(a.vb, pos);
    const int vk = __ldg(a.vb.kind + b);
    const int64_t r = pos - __ldg(a.vb.pos0 + b);
    const int dim = vk == ND_V_SWING || vk == ND_V_SWING_UNIT ? 2 : 1;
    const int pd = vk == ND_V_DIFFUSION ? 0 : (vk == ND_V_SWING ? 3 : 1);
    const int64_t s = __ldg(a.vb.s0 + b) + dim * r, q = __ldg(a.vb.p0 + b) + pd * r;
    T scale = T(1);
    if (dim == 2) {
        T dw = T(-1);
        if (vk == ND_V_SWING) {
            scale = A::div(T(1), __ldg(a.p + q));
            dw = -A::mul(scale, __ldg(a.p + q + 1));
        }
        if (lane == 0) {
            const int32_t r0 = __ldg(a.rowptr + s), r1 = __ldg(a.rowptr + s + 1), r2 = __ldg(a.rowptr + s + 2);
            jadd<T>(a.values + r0, a.colidx + r0, r1 - r0, (int32_t)(s + 1), T(1));
            jadd<T>(a.values + r1, a.colidx + r1, r2 - r1, (int32_t)(s + 1), dw);
        }
    }
    const int64_t row = s + dim - 1;
    const int32_t r0 = __ldg(a.rowptr + row);
    const int n = __ldg(a.rowptr + row + 1) - r0;
    T* vals = a.values + r0;
    const int32_t* cols = a.colidx + r0;
    const int32_t own = (int32_t)s;
    T own_sum = T(0);
    const uint32_t t0 = __ldg(a.tptr + slot), t1 = __ldg(a.tptr + slot + 1);
    for (uint32_t j = t0 + lane; j < t1; j += 32) {
        const int32_t t = __ldg(a.tidx + j);
        const int64_t k = t >> 1;
        const bool dst_side = t & 1;
        const int eb = find_batch(a.eb, k);
        const int ek = __ldg(a.eb.kind + eb);
        const int64_t re = k - __ldg(a.eb.pos0 + eb);
        if (ek == ND_E_DIFFUSION_ODE || ek == ND_E_DIFFUSION_ODE_FIXED) {
            jadd_atomic<T>(vals, cols, n, (int32_t)(__ldg(a.eb.s0 + eb) + 2 * re + (dst_side ? 0 : 1)), scale);
            continue;
        }
        const int c = __ldg(a.eb.coupling + eb);
        if (!dst_side && c == ND_DIRECTED) continue;
        const int2 o = __ldg(a.eu + k);
        const T wgt = ek == ND_E_DIFFUSION_UNIT ? T(0) : __ldg(a.p + __ldg(a.eb.p0 + eb) + re);
        T gs, gd;
        static_edge_dg<T>(ek, __ldg(a.u + o.x), __ldg(a.u + o.y), wgt, gs, gd);
        const T f = dst_side || c == ND_SYMMETRIC ? scale : -scale;
        const T ds = A::mul(f, gs), dd = A::mul(f, gd);
        if (o.x == own) own_sum = A::add(own_sum, ds);
        else jadd_atomic<T>(vals, cols, n, o.x, ds);
        if (o.y == own) own_sum = A::add(own_sum, dd);
        else jadd_atomic<T>(vals, cols, n, o.y, dd);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) own_sum = A::add(own_sum, __shfl_xor_sync(0xffffffffu, own_sum, off));
    if (lane == 0) jadd<T>(vals, cols, n, own, own_sum);
}

template <typename T>
__global__ void __launch_bounds__(kJacBlock) jac_ode_edge_kernel(JacArgs<T> a) {
    using A = Arith<T>;
    const int64_t k = (int64_t)blockIdx.x * kJacBlock + threadIdx.x;
    if (k >= a.ne) return;
    const int eb = find_batch(a.eb, k);
    const int ek = __ldg(a.eb.kind + eb);
    if (ek != ND_E_DIFFUSION_ODE && ek != ND_E_DIFFUSION_ODE_FIXED) return;
    const int64_t re = k - __ldg(a.eb.pos0 + eb);
    const int64_t es = __ldg(a.eb.s0 + eb) + 2 * re;
    const int2 o = __ldg(a.eu + k);
    const T rate = ek == ND_E_DIFFUSION_ODE ? A::div(T(1), __ldg(a.p + __ldg(a.eb.p0 + eb) + re)) : T(100);
    const T c = A::mul(rate, A::cos_phase(A::sub(__ldg(a.u + o.x), __ldg(a.u + o.y))));
    // de1 = rate (sin(vs - vd) - e1), de2 = rate (sin(vd - vs) - e2)
    for (int i = 0; i < 2; ++i) {
        const int32_t r0 = __ldg(a.rowptr + es + i);
        const int n = __ldg(a.rowptr + es + i + 1) - r0;
        const T sgn = i == 0 ? T(1) : T(-1);
        jadd<T>(a.values + r0, a.colidx + r0, n, o.x, A::mul(sgn, c));
        jadd<T>(a.values + r0, a.colidx + r0, n, o.y, -A::mul(sgn, c));
        jadd<T>(a.values + r0, a.colidx + r0, n, (int32_t)(es + i), -rate);
    }
}

// ---- networks with complex outputs (power grids: PQ buses, generators, π-lines) ----------
// A vertex thread differentiates its component with dual numbers: the generator with
// respect to its four states and the two components of the aggregated current, the PQ bus
// with respect to the current (its output does not depend on its own states).  Each
// incident π-line side is differentiated with respect to the two endpoint voltages (four
// partials); the chain rule ∂f/∂i · ∂i/∂V gives the voltage columns.
template <typename T, int N>
__device__ __forceinline__ Cx<Dual<T, N>> cx_seed(T re, T im, int k) {
    return {Dual<T, N>::seed(re, k), Dual<T, N>::seed(im, k + 1)};
}

template <typename T>
__global__ void __launch_bounds__(kJacBlock) jac_powergrid_kernel(JacArgs<T> a) {
    using A = Arith<T>;
    using D4 = Dual<T, 4>;
    using D6 = Dual<T, 6>;
    const int64_t slot = (int64_t)blockIdx.x * kJacBlock + threadIdx.x;
    if (slot >= a.nv) return;
    const int64_t pos = __ldg(a.slot_vpos + slot);
    const int b = find_batch(a.vb, pos);
    const int vk = __ldg(a.vb.kind + b);
    const int64_t r = pos - __ldg(a.vb.pos0 + b);
    const int dim = vk == ND_V_GENERATOR ? 4 : 2;
    const int pd = vk == ND_V_GENERATOR ? 11 : (vk == ND_V_PQ ? 2 : 0);
    const int64_t s = __ldg(a.vb.s0 + b) + dim * r, q = __ldg(a.vb.p0 + b) + pd * r;
    const uint32_t t0 = __ldg(a.tptr + slot), t1 = __ldg(a.tptr + slot + 1);
    // the output of line side j at this vertex and its derivatives by (Vs_r, Vs_i, Vd_r, Vd_i)
    auto side = [&](uint32_t j, int2& o, Cx<D4>& y) {
        const int32_t t = __ldg(a.tidx + j);
        const int64_t k = t >> 1;
        const int eb = find_batch(a.eb, k);
        const int64_t pe = __ldg(a.eb.p0 + eb) + 4 * (k - __ldg(a.eb.pos0 + eb));
        o = __ldg(a.eu + k);
        const Cx<D4> vs = cx_seed<T, 4>(__ldg(a.u + o.x), __ldg(a.u + o.x + 1), 0);
        const Cx<D4> vd = cx_seed<T, 4>(__ldg(a.u + o.y), __ldg(a.u + o.y + 1), 2);
        Cx<D4> ys, yd;
        piline_g<D4>(vs, vd, D4(__ldg(a.p + pe)), D4(__ldg(a.p + pe + 1)), D4(__ldg(a.p + pe + 2)),
                     D4(__ldg(a.p + pe + 3)), ys, yd);
        y = (t & 1) ? yd : ys;
    };
    // the aggregated current (any order: only its value enters the derivatives)
    T ir = T(0), ii = T(0);
    for (uint32_t j = t0; j < t1; ++j) {
        int2 o;
        Cx<D4> y;
        side(j, o, y);
        ir = A::add(ir, y.r.v);
        ii = A::add(ii, y.i.v);
    }
    // ∂f/∂(states) and ∂f/∂(current) for the rows f = 0..dim-1
    T dfs[4][4] = {}, dfi[4][2] = {};
    if (vk == ND_V_GENERATOR) {
        D6 uu[4], pp[11], out[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) uu[c] = D6::seed(__ldg(a.u + s + c), c);
#pragma unroll
        for (int c = 0; c < 11; ++c) pp[c] = D6(__ldg(a.p + q + c));
        vertex_f2_at<D6, ND_V_GENERATOR>(out, uu, pp, 0, 0, cx_seed<T, 6>(ir, ii, 4));
#pragma unroll
        for (int f = 0; f < 4; ++f) {
#pragma unroll
            for (int c = 0; c < 4; ++c) dfs[f][c] = out[f].d[c];
            dfi[f][0] = out[f].d[4];
            dfi[f][1] = out[f].d[5];
        }
    } else {
        using D2 = Dual<T, 2>;
        const Cx<D2> in = cx_seed<T, 2>(ir, ii, 0);
        Cx<D2> uc;
        if (vk == ND_V_PQ) {
            uc = cdiv<D2>({D2(__ldg(a.p + q)), D2(__ldg(a.p + q + 1))}, {in.r, -in.i});
        } else {  // ND_V_PQ_CONST: P, Q are the batch's constants
            uc = cdiv<D2>({D2((T)__ldg(a.vb.consts + kBatchConstants * b)),
                           D2((T)__ldg(a.vb.consts + kBatchConstants * b + 1))},
                          {in.r, -in.i});
        }
        dfi[0][0] = uc.r.d[0];
        dfi[0][1] = uc.r.d[1];
        dfi[1][0] = uc.i.d[0];
        dfi[1][1] = uc.i.d[1];
    }
    for (int f = 0; f < dim; ++f) {
        const int32_t r0 = __ldg(a.rowptr + s + f);
        const int n = __ldg(a.rowptr + s + f + 1) - r0;
        T* vals = a.values + r0;
        const int32_t* cols = a.colidx + r0;
        if (vk == ND_V_GENERATOR)
            for (int c = 0; c < 4; ++c) jadd<T>(vals, cols, n, (int32_t)(s + c), dfs[f][c]);
        for (uint32_t j = t0; j < t1; ++j) {
            int2 o;
            Cx<D4> y;
            side(j, o, y);
#pragma unroll
            for (int x = 0; x < 4; ++x) {
                const T v = A::add(A::mul(dfi[f][0], y.r.d[x]), A::mul(dfi[f][1], y.i.d[x]));
                jadd<T>(vals, cols, n, (x < 2 ? o.x : o.y) + (x & 1), v);
            }
        }
    }
}

// The batched view of a homogeneous handle: its edge list recovered from the device CSR
// (every edge appears once on its source side), one vertex and one edge batch.
int build_view(nd_handle* h, BatchedNet* view) {
    const Topology& t = h->topo;
    const int64_t nv = t.nv, ne = t.ne;
    std::vector<uint32_t> slot_ptr(nv + 1);
    std::vector<int32_t> slot_vertex(nv);
    std::vector<Incidence> incid((size_t)2 * ne);
    cudaError_t err;
    if ((err = cudaMemcpy(slot_ptr.data(), t.slot_ptr, slot_ptr.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost)) !=
            cudaSuccess ||
        (err = cudaMemcpy(slot_vertex.data(), t.slot_vertex, slot_vertex.size() * sizeof(int32_t),
                          cudaMemcpyDeviceToHost)) != cudaSuccess ||
        (ne > 0 && (err = cudaMemcpy(incid.data(), t.incid, incid.size() * sizeof(Incidence), cudaMemcpyDeviceToHost)) !=
                       cudaSuccess))
        return cuda_fail(err, "nd_jacobian: topology download");
    std::vector<int64_t> src(ne), dst(ne);
    for (int64_t s = 0; s < nv; ++s)
        for (uint32_t i = slot_ptr[s]; i < slot_ptr[s + 1]; ++i)
            if (incid[i].eid < 0) {
                const int32_t e = incid[i].eid & 0x7fffffff;
                src[e] = slot_vertex[s];
                dst[e] = incid[i].nbr;
            }
    std::vector<int32_t> vb(nv, 0), ebi(ne, 0);
    nd_batch vbatch{h->vertex_kind, 0}, ebatch{h->edge_kind, h->coupling};
    nd_batched_network_desc d{};
    d.nv = nv;
    d.ne = ne;
    d.src = src.data();
    d.dst = dst.data();
    d.n_vertex_batches = 1;
    d.n_edge_batches = 1;
    d.vertex_batches = &vbatch;
    d.edge_batches = &ebatch;
    d.vertex_batch = vb.data();
    d.edge_batch = ebi.data();
    return build_batched(&d, 0, view);
}

// Pattern of the Jacobian (see the file comment), built on the host from the batched
// structure.
int build_plan(nd_handle* h) {
    JacPlan& J = h->jac;
    if (!h->batched.enabled && !J.view.enabled) {
        const int rc = build_view(h, &J.view);
        if (rc != ND_OK) return rc;
    }
    const BatchedNet& b = h->batched.enabled ? h->batched : J.view;
    const int64_t nv = b.nv, ne = b.ne, dim = b.dim;
    std::vector<uint32_t> tptr(nv + 1);
    std::vector<int32_t> tidx((size_t)2 * ne), slot_vpos(nv);
    std::vector<int2> eu(ne);
    cudaError_t err;
    if ((err = cudaMemcpy(tptr.data(), b.tptr, tptr.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost)) != cudaSuccess ||
        (err = cudaMemcpy(slot_vpos.data(), b.slot_vpos, slot_vpos.size() * sizeof(int32_t), cudaMemcpyDeviceToHost)) !=
            cudaSuccess ||
        (ne > 0 && ((err = cudaMemcpy(tidx.data(), b.tidx, tidx.size() * sizeof(int32_t), cudaMemcpyDeviceToHost)) !=
                        cudaSuccess ||
                    (err = cudaMemcpy(eu.data(), b.eu, eu.size() * sizeof(int2), cudaMemcpyDeviceToHost)) != cudaSuccess)))
        return cuda_fail(err, "nd_jacobian: structure download");
    std::vector<std::vector<int32_t>> rows(dim);
    // power grids: every state row of a vertex has its own states (generators) and both
    // voltage states of both endpoints of each incident line side
    for (int64_t slot = 0; b.depth == 2 && slot < nv; ++slot) {
        const int64_t pos = slot_vpos[slot];
        const int vbi = host_find_batch(b.vb, pos);
        const int vk = b.vb.kind[vbi];
        const int vdim = vertex_dim(vk);
        const int64_t s = b.vb.s0[vbi] + vdim * (pos - b.vb.pos0[vbi]);
        std::vector<int32_t> cols;
        if (vk == ND_V_GENERATOR)
            for (int c = 0; c < 4; ++c) cols.push_back((int32_t)(s + c));
        for (uint32_t j = tptr[slot]; j < tptr[slot + 1]; ++j) {
            const int2 o = eu[tidx[j] >> 1];
            for (int c = 0; c < 2; ++c) {
                cols.push_back(o.x + c);
                cols.push_back(o.y + c);
            }
        }
        for (int f = 0; f < vdim; ++f) rows[s + f] = cols;
    }
    for (int64_t slot = 0; b.depth == 1 && slot < nv; ++slot) {
        const int64_t pos = slot_vpos[slot];
        const int vbi = host_find_batch(b.vb, pos);
        const int vk = b.vb.kind[vbi];
        const int vdim = vertex_dim(vk);
        const int64_t s = b.vb.s0[vbi] + vdim * (pos - b.vb.pos0[vbi]);
        if (is_swing(vk)) {
            rows[s].push_back((int32_t)(s + 1));
            rows[s + 1].push_back((int32_t)(s + 1));
        }
        std::vector<int32_t>& row = rows[s + vdim - 1];
        for (uint32_t j = tptr[slot]; j < tptr[slot + 1]; ++j) {
            const int64_t k = tidx[j] >> 1;
            const bool dst_side = tidx[j] & 1;
            const int ebi = host_find_batch(b.eb, k);
            const int ek = b.eb.kind[ebi];
            if (is_ode(ek)) {
                row.push_back((int32_t)(b.eb.s0[ebi] + 2 * (k - b.eb.pos0[ebi]) + (dst_side ? 0 : 1)));
            } else if (dst_side || b.eb.coupling[ebi] != ND_DIRECTED) {
                row.push_back(eu[k].x);
                row.push_back(eu[k].y);
            }
        }
    }
    for (int64_t k = 0; b.depth == 1 && k < ne; ++k) {
        const int ebi = host_find_batch(b.eb, k);
        if (!is_ode(b.eb.kind[ebi])) continue;
        const int64_t es = b.eb.s0[ebi] + 2 * (k - b.eb.pos0[ebi]);
        for (int i = 0; i < 2; ++i) {
            rows[es + i].push_back(eu[k].x);
            rows[es + i].push_back(eu[k].y);
            rows[es + i].push_back((int32_t)(es + i));
        }
    }
    J.rowptr_h.assign(dim + 1, 0);
    int64_t nnz = 0;
    for (int64_t i = 0; i < dim; ++i) {
        std::vector<int32_t>& r = rows[i];
        std::sort(r.begin(), r.end());
        r.erase(std::unique(r.begin(), r.end()), r.end());
        nnz += (int64_t)r.size();
        if (nnz > (int64_t)INT32_MAX) return fail(ND_ERR_UNSUPPORTED, "nd_jacobian: more than 2^31-1 nonzeros");
        J.rowptr_h[i + 1] = (int32_t)nnz;
    }
    std::vector<int32_t> long_slots;
    for (int64_t slot = 0; b.depth == 1 && slot < nv; ++slot)
        if (tptr[slot + 1] - tptr[slot] > kJacLongRow) long_slots.push_back((int32_t)slot);
    J.n_long = (int64_t)long_slots.size();
    J.colidx_h.resize(nnz);
    for (int64_t i = 0; i < dim; ++i) std::copy(rows[i].begin(), rows[i].end(), J.colidx_h.begin() + J.rowptr_h[i]);
    J.nnz = nnz;
    if ((err = cudaMalloc(&J.rowptr, (dim + 1) * sizeof(int32_t))) != cudaSuccess ||
        (err = cudaMalloc(&J.colidx, std::max<int64_t>(nnz, 1) * sizeof(int32_t))) != cudaSuccess ||
        (err = cudaMemcpy(J.rowptr, J.rowptr_h.data(), (dim + 1) * sizeof(int32_t), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (nnz > 0 &&
         (err = cudaMemcpy(J.colidx, J.colidx_h.data(), nnz * sizeof(int32_t), cudaMemcpyHostToDevice)) != cudaSuccess) ||
        (err = cudaMalloc(&J.long_slots, std::max<int64_t>(J.n_long, 1) * sizeof(int32_t))) != cudaSuccess ||
        (J.n_long > 0 && (err = cudaMemcpy(J.long_slots, long_slots.data(), J.n_long * sizeof(int32_t),
                                           cudaMemcpyHostToDevice)) != cudaSuccess))
        return cuda_fail(err, "nd_jacobian: pattern upload");
    J.ready = true;
    return ND_OK;
}

template <typename T>
cudaError_t launch_values(nd_handle* h, void* values, const void* u, const void* p, cudaStream_t s) {
    const JacPlan& J = h->jac;
    const BatchedNet& b = h->batched.enabled ? h->batched : J.view;
    JacArgs<T> a;
    a.values = static_cast<T*>(values);
    a.u = static_cast<const T*>(u);
    a.p = static_cast<const T*>(p);
    a.rowptr = J.rowptr;
    a.colidx = J.colidx;
    a.nv = b.nv;
    a.ne = b.ne;
    a.vb = b.dvb;
    a.eb = b.deb;
    a.eu = b.eu;
    a.tptr = b.tptr;
    a.tidx = b.tidx;
    a.slot_vpos = b.slot_vpos;
    cudaError_t err = cudaMemsetAsync(values, 0, std::max<int64_t>(J.nnz, 1) * sizeof(T), s);
    if (err != cudaSuccess) return err;
    if (b.depth == 2) {
        jac_powergrid_kernel<T><<<(unsigned)((b.nv + kJacBlock - 1) / kJacBlock), kJacBlock, 0, s>>>(a);
        return cudaGetLastError();
    }
    jac_vertex_kernel<T><<<(unsigned)((b.nv + kJacBlock - 1) / kJacBlock), kJacBlock, 0, s>>>(a);
    if (J.n_long > 0)
        jac_long_row_kernel<T><<<(unsigned)((J.n_long * 32 + kJacBlock - 1) / kJacBlock), kJacBlock, 0, s>>>(
            a, J.long_slots, J.n_long);
    if (b.ne > 0) jac_ode_edge_kernel<T><<<(unsigned)((b.ne + kJacBlock - 1) / kJacBlock), kJacBlock, 0, s>>>(a);
    return cudaGetLastError();
}

template <typename T>
__global__ void __launch_bounds__(kJacBlock) csr_times_kernel(int64_t n, const int32_t* __restrict__ rowptr,
                                                              const int32_t* __restrict__ col,
                                                              const T* __restrict__ val, const T* __restrict__ x,
                                                              T* __restrict__ y) {
    using A = Arith<T>;
    const int64_t i = (int64_t)blockIdx.x * kJacBlock + threadIdx.x;
    if (i >= n) return;
    T s = T(0);
    for (int32_t k = __ldg(rowptr + i); k < __ldg(rowptr + i + 1); ++k)
        s = A::add(s, A::mul(__ldg(val + k), __ldg(x + __ldg(col + k))));
    y[i] = s;
}

}  // namespace

// jv = J(u, p) v for handles without a direct JVP kernel (batched networks): the Jacobian
// assembled into a buffer the handle keeps, then one CSR product.
int jacobian_times(nd_handle* h, void* jv, const void* u, const void* p, const void* v, cudaStream_t s) {
    if (!h->jac.ready) {
        const int rc = build_plan(h);
        if (rc != ND_OK) return rc;
    }
    JacPlan& J = h->jac;
    const size_t elem = h->dtype == ND_F64 ? 8 : 4;
    if (!J.values) {
        const cudaError_t e = cudaMalloc(&J.values, std::max<int64_t>(J.nnz, 1) * elem);
        if (e != cudaSuccess) return cuda_fail(e, "nd_jvp: Jacobian buffer");
    }
    cudaError_t err = h->dtype == ND_F64 ? launch_values<double>(h, J.values, u, p, s)
                                         : launch_values<float>(h, J.values, u, p, s);
    const int64_t n = h->dim;
    const unsigned grid = (unsigned)((n + kJacBlock - 1) / kJacBlock);
    if (err == cudaSuccess && n > 0) {
        if (h->dtype == ND_F64)
            csr_times_kernel<double><<<grid, kJacBlock, 0, s>>>(n, J.rowptr, J.colidx, static_cast<double*>(J.values),
                                                                static_cast<const double*>(v), static_cast<double*>(jv));
        else
            csr_times_kernel<float><<<grid, kJacBlock, 0, s>>>(n, J.rowptr, J.colidx, static_cast<float*>(J.values),
                                                               static_cast<const float*>(v), static_cast<float*>(jv));
        err = cudaGetLastError();
    }
    return err == cudaSuccess ? ND_OK : cuda_fail(err, "nd_jvp");
}

void free_jacobian(JacPlan* j) {
    if (j->view.enabled) free_batched(&j->view);
    cudaFree(j->rowptr);
    cudaFree(j->colidx);
    cudaFree(j->long_slots);
    cudaFree(j->values);
    *j = JacPlan{};
}

}  // namespace nd

using namespace nd;

extern "C" int nd_jacobian_pattern(nd_handle* h, int64_t* nnz, int32_t* rowptr, int32_t* colidx) {
    clear_error();
    if (!h || !nnz) return fail(ND_ERR_ARG, "nd_jacobian_pattern: NULL argument");
    if (!h->jac.ready) {
        const int rc = build_plan(h);
        if (rc != ND_OK) return rc;
    }
    *nnz = h->jac.nnz;
    if (rowptr) std::copy(h->jac.rowptr_h.begin(), h->jac.rowptr_h.end(), rowptr);
    if (colidx) std::copy(h->jac.colidx_h.begin(), h->jac.colidx_h.end(), colidx);
    return ND_OK;
}

extern "C" int nd_jacobian(nd_handle* h, int dtype, void* values, const void* u, const void* p, double t,
                           void* stream) {
    ND_NVTX("nd_jacobian");
    (void)t;
    clear_error();
    if (!h || !values || !u) return fail(ND_ERR_ARG, "nd_jacobian: NULL argument");
    if (dtype != h->dtype) return fail(ND_ERR_DTYPE, "nd_jacobian: element type differs from the handle's");
    if (h->pdim > 0 && !p) return fail(ND_ERR_ARG, "nd_jacobian: p is NULL");
    if (!h->jac.ready) {
        const int rc = build_plan(h);
        if (rc != ND_OK) return rc;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const cudaError_t err = h->dtype == ND_F64 ? launch_values<double>(h, values, u, p, s)
                                               : launch_values<float>(h, values, u, p, s);
    return err == cudaSuccess ? ND_OK : cuda_fail(err, "nd_jacobian");
}
