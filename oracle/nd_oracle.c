/*
 * ORACLE — test infrastructure, not product code.
 *
 * CPU restatement of NetworkDynamics.jl's network right-hand side for the component
 * library of the GB300 path, written to follow the reference operation by operation:
 *
 *   nd_oracle_rhs_*        (nw::Network)(du,u,p,t) with SequentialExecution +
 *                          SequentialAggregator(+)     src/coreloop.jl:1-102
 *   nd_oracle_rhs_poly_*   the same with PolyesterExecution + PolyesterAggregator(+):
 *                          component loops and the inverse aggregation map run on
 *                          OpenMP threads              src/coreloop.jl:131-139,
 *                                                      src/aggregators.jl:159-177,203-235
 *   nd_oracle_tsit5        Tsit5 (Tsitouras 2011, the published tableau) with a PI step
 *                          controller, driving the sequential RHS
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline load this library,
 * to check the GPU results against.  Compile with -ffp-contract=off: the reference performs no fused
 * multiply-adds in these functions, so neither may the restatement.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Component kinds and output wrappers: same numbering as the C ABI of the GB300 library. */
enum { V_DIFFUSION = 1, V_KURAMOTO = 2, V_SWING = 3, V_SWING_UNIT = 4, V_PQ = 5, V_GENERATOR = 6, V_PQ_CONST = 7 };
enum { E_DIFFUSION = 1, E_DIFFUSION_UNIT = 2, E_KURAMOTO = 3, E_DIFFUSION_ODE = 4, E_DIFFUSION_ODE_FIXED = 5,
       E_PILINE = 6 };
enum { C_ANTISYMMETRIC = 1, C_SYMMETRIC = 2, C_DIRECTED = 3, C_FIDUCIAL = 4 };

static int vdim(int vk) {
    return vk == V_GENERATOR ? 4 : (vk == V_SWING || vk == V_SWING_UNIT || vk == V_PQ || vk == V_PQ_CONST ? 2 : 1);
}
static int vpdim(int vk) {
    switch (vk) {
        case V_DIFFUSION: case V_PQ_CONST: return 0;
        case V_KURAMOTO: case V_SWING_UNIT: return 1;
        case V_SWING: return 3;
        case V_PQ: return 2;
        default: return 11; /* generator */
    }
}
static int is_ode_edge(int ek) { return ek == E_DIFFUSION_ODE || ek == E_DIFFUSION_ODE_FIXED; }
static int edim(int ek) { return is_ode_edge(ek) ? 2 : 0; }
static int epdim(int ek) {
    return ek == E_DIFFUSION_UNIT || ek == E_DIFFUSION_ODE_FIXED ? 0 : (ek == E_PILINE ? 4 : 1);
}
/* output dimension (vdepth / edepth): the power-grid components carry complex values */
static int voutdim(int vk) { return vk == V_PQ || vk == V_GENERATOR || vk == V_PQ_CONST ? 2 : 1; }
static int eoutdim(int ek) { return ek == E_PILINE ? 2 : 1; }

/*
 * Index layout of src/network_structure.jl:224-289, built as src/construction.jl:155-195
 * does: components are batched by identity in order of first appearance
 * (find_identical, src/utils.jl:197-216), all vertex batches are registered before the
 * edge batches, and every edge owns an output range for src followed by one for dst.
 * vdepth = edepth = 1 (StateMask(1) vertex outputs, scalar edge outputs).
 */
typedef struct {
    int64_t nv, ne;
    int depth; /* output dimension of every vertex and edge side (vdepth = edepth) */
    const int64_t* src;
    const int64_t* dst;
    int32_t* vkind; /* [nv] kind of every vertex */
    double* vconst; /* [2 nv] the constants of every vertex's batch (pqnode_inhomogeneous's P, Q) */
    int32_t* ekind; /* [ne] kind of every edge */
    int32_t* ecoup; /* [ne] output wrapper of every edge */
    /* layout, 0-based offsets */
    int64_t* v_data; /* first state index of vertex */
    int64_t* e_data; /* first state index of edge (ODE edges) */
    int64_t* v_out;  /* output index */
    int64_t* v_para; /* first parameter index */
    int64_t* v_aggr; /* aggregation index */
    int64_t* e_out_src;
    int64_t* e_out_dst;
    int64_t* e_para;
    int64_t* vbatch_order; /* vertices in batch (processing) order */
    int64_t* ebatch_order; /* edges in batch (processing) order */
    int64_t lastidx_dynamic, lastidx_out, lastidx_p, lastidx_aggr;
    int64_t agg_first, agg_len; /* tightened aggregation range of the output buffer */
    int64_t* agg_map;           /* [agg_len] output index -> aggregation index + 1, 0 = skip */
    /* inverse map for the Polyester aggregator: per aggregation index, its output indices */
    int64_t* inv_ptr;
    int64_t* inv_idx;
} layout_t;

/* Batch order: batches in index order, components ascending inside a batch (a stable
 * counting sort by batch). */
static void batch_order(int64_t n, const int32_t* batch, int nb, int64_t* order) {
    int64_t* start = (int64_t*)calloc((size_t)nb + 1, sizeof(int64_t));
    for (int64_t i = 0; i < n; ++i) start[batch[i] + 1]++;
    for (int b = 0; b < nb; ++b) start[b + 1] += start[b];
    for (int64_t i = 0; i < n; ++i) order[start[batch[i]]++] = i;
    free(start);
}

void nd_oracle_layout_free(layout_t* L);

/* Layout of a network whose batches are given explicitly: vertex v belongs to vertex batch
 * vbatch[v] of kind vb_kind[.], edge e to edge batch ebatch[e] of kind eb_kind[.] and
 * wrapper eb_coup[.].  The batches are laid out in index order, which is the reference's
 * order of first appearance when the caller numbers them that way. */
layout_t* nd_oracle_layout_new_batched(int64_t nv, int64_t ne, const int64_t* src, const int64_t* dst,
                                       int nvb, const int32_t* vb_kind, const int32_t* vbatch, int neb,
                                       const int32_t* eb_kind, const int32_t* eb_coup, const int32_t* ebatch,
                                       const double* vb_const) {
    layout_t* L = (layout_t*)calloc(1, sizeof(layout_t));
    L->nv = nv;
    L->ne = ne;
    L->src = src;
    L->dst = dst;
    L->vkind = (int32_t*)malloc(sizeof(int32_t) * (nv + 1));
    L->ekind = (int32_t*)malloc(sizeof(int32_t) * (ne + 1));
    L->ecoup = (int32_t*)malloc(sizeof(int32_t) * (ne + 1));
    L->vconst = (double*)calloc((size_t)(2 * nv + 2), sizeof(double));
    for (int64_t v = 0; v < nv; ++v) {
        L->vkind[v] = vb_kind[vbatch[v]];
        if (vb_const) {
            L->vconst[2 * v] = vb_const[2 * vbatch[v]];
            L->vconst[2 * v + 1] = vb_const[2 * vbatch[v] + 1];
        }
    }
    for (int64_t e = 0; e < ne; ++e) {
        L->ekind[e] = eb_kind[ebatch[e]];
        L->ecoup[e] = eb_coup[ebatch[e]];
    }
    L->v_data = (int64_t*)malloc(sizeof(int64_t) * (nv + 1));
    L->v_out = (int64_t*)malloc(sizeof(int64_t) * (nv + 1));
    L->v_para = (int64_t*)malloc(sizeof(int64_t) * (nv + 1));
    L->v_aggr = (int64_t*)malloc(sizeof(int64_t) * (nv + 1));
    L->e_data = (int64_t*)malloc(sizeof(int64_t) * (ne + 1));
    L->e_out_src = (int64_t*)malloc(sizeof(int64_t) * (ne + 1));
    L->e_out_dst = (int64_t*)malloc(sizeof(int64_t) * (ne + 1));
    L->e_para = (int64_t*)malloc(sizeof(int64_t) * (ne + 1));
    L->vbatch_order = (int64_t*)malloc(sizeof(int64_t) * (nv + 1));
    L->ebatch_order = (int64_t*)malloc(sizeof(int64_t) * (ne + 1));
    batch_order(nv, vbatch, nvb, L->vbatch_order);
    batch_order(ne, ebatch, neb, L->ebatch_order);
    const int32_t* vkind = L->vkind;
    const int32_t* ekind = L->ekind;
    /* all vertex models and all edge models share one output dimension
       (src/construction.jl:98-106); the library's depths agree across the two */
    const int depth = nv > 0 ? voutdim(vkind[0]) : 1;
    int bad = 0;
    for (int64_t v = 0; v < nv; ++v) bad |= voutdim(vkind[v]) != depth;
    for (int64_t e = 0; e < ne; ++e) bad |= eoutdim(ekind[e]) != depth;
    L->depth = depth;
    if (bad) {
        nd_oracle_layout_free(L);
        return NULL;
    }
    int64_t dyn = 0, out = 0, par = 0, agg = 0;
    for (int64_t k = 0; k < nv; ++k) { /* register_vertices! */
        int64_t v = L->vbatch_order[k];
        L->v_data[v] = dyn;
        dyn += vdim(vkind[v]);
        L->v_out[v] = out;
        out += depth;
        L->v_para[v] = par;
        par += vpdim(vkind[v]);
        L->v_aggr[v] = agg;
        agg += depth;
    }
    for (int64_t k = 0; k < ne; ++k) { /* register_edges!: states after every vertex state */
        int64_t e = L->ebatch_order[k];
        L->e_data[e] = dyn;
        dyn += edim(ekind[e]);
        L->e_out_src[e] = out;
        out += depth;
        L->e_out_dst[e] = out;
        out += depth;
        L->e_para[e] = par;
        par += epdim(ekind[e]);
    }
    L->lastidx_dynamic = dyn;
    L->lastidx_out = out;
    L->lastidx_p = par;
    L->lastidx_aggr = agg;
    /* AggregationMap (src/aggregators.jl:58-86): map[out index] = aggr index, tightened. */
    int64_t* full = (int64_t*)calloc((size_t)out + 1, sizeof(int64_t));
    for (int64_t k = 0; k < ne; ++k) {
        int64_t e = L->ebatch_order[k];
        for (int j = 0; j < depth; ++j) {
            full[L->e_out_dst[e] + j] = L->v_aggr[dst[e]] + j + 1;
            full[L->e_out_src[e] + j] = L->v_aggr[src[e]] + j + 1;
        }
    }
    int64_t first = -1, last = -1;
    for (int64_t i = 0; i < out; ++i)
        if (full[i]) {
            if (first < 0) first = i;
            last = i;
        }
    if (first < 0) {
        L->agg_first = 0;
        L->agg_len = 0;
        L->agg_map = (int64_t*)malloc(sizeof(int64_t));
    } else {
        L->agg_first = first;
        L->agg_len = last - first + 1;
        L->agg_map = (int64_t*)malloc(sizeof(int64_t) * (size_t)L->agg_len);
        memcpy(L->agg_map, full + first, sizeof(int64_t) * (size_t)L->agg_len);
    }
    free(full);
    /* _inv_aggregation_map (src/aggregators.jl:203-235): per vertex, its incident output
     * indices in edge-batch order, dst mapping before src mapping within an edge. */
    L->inv_ptr = (int64_t*)calloc((size_t)agg + 1, sizeof(int64_t));
    L->inv_idx = (int64_t*)malloc(sizeof(int64_t) * (size_t)(2 * depth * ne + 1));
    for (int64_t e = 0; e < ne; ++e)
        for (int j = 0; j < depth; ++j) {
            L->inv_ptr[L->v_aggr[dst[e]] + j + 1]++;
            L->inv_ptr[L->v_aggr[src[e]] + j + 1]++;
        }
    for (int64_t a = 0; a < agg; ++a) L->inv_ptr[a + 1] += L->inv_ptr[a];
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * ((size_t)agg + 1));
    memcpy(fill, L->inv_ptr, sizeof(int64_t) * ((size_t)agg + 1));
    for (int64_t k = 0; k < ne; ++k) {
        int64_t e = L->ebatch_order[k];
        for (int j = 0; j < depth; ++j) {
            L->inv_idx[fill[L->v_aggr[dst[e]] + j]++] = L->e_out_dst[e] + j;
            L->inv_idx[fill[L->v_aggr[src[e]] + j]++] = L->e_out_src[e] + j;
        }
    }
    free(fill);
    return L;
}

/* Layout from per-component kinds: one batch per kind in order of first appearance
 * (find_identical over identical components), every edge AntiSymmetric. */
layout_t* nd_oracle_layout_new(int64_t nv, int64_t ne, const int64_t* src, const int64_t* dst,
                               const int32_t* vkind, const int32_t* ekind) {
    int32_t vk[16], ek[16], ec[16];
    int nvb = 0, neb = 0;
    int32_t* vb = (int32_t*)malloc(sizeof(int32_t) * (nv + 1));
    int32_t* eb = (int32_t*)malloc(sizeof(int32_t) * (ne + 1));
    for (int64_t v = 0; v < nv; ++v) {
        int b = 0;
        while (b < nvb && vk[b] != vkind[v]) ++b;
        if (b == nvb && nvb < 16) vk[nvb++] = vkind[v];
        vb[v] = b;
    }
    for (int64_t e = 0; e < ne; ++e) {
        int b = 0;
        while (b < neb && ek[b] != ekind[e]) ++b;
        if (b == neb && neb < 16) {
            ek[neb] = ekind[e];
            ec[neb++] = ekind[e] == E_PILINE ? C_FIDUCIAL : C_ANTISYMMETRIC;
        }
        eb[e] = b;
    }
    layout_t* L = nd_oracle_layout_new_batched(nv, ne, src, dst, nvb, vk, vb, neb, ek, ec, eb, NULL);
    free(vb);
    free(eb);
    return L;
}

void nd_oracle_layout_free(layout_t* L) {
    if (!L) return;
    free(L->vkind);
    free(L->vconst);
    free(L->ekind);
    free(L->ecoup);
    free(L->e_data);
    free(L->v_data);
    free(L->v_out);
    free(L->v_para);
    free(L->v_aggr);
    free(L->e_out_src);
    free(L->e_out_dst);
    free(L->e_para);
    free(L->vbatch_order);
    free(L->ebatch_order);
    free(L->agg_map);
    free(L->inv_ptr);
    free(L->inv_idx);
    free(L);
}

int64_t nd_oracle_dim(const layout_t* L) { return L->lastidx_dynamic; }
int64_t nd_oracle_pdim(const layout_t* L) { return L->lastidx_p; }
int64_t nd_oracle_v_data(const layout_t* L, int64_t v) { return L->v_data[v]; }
int64_t nd_oracle_v_para(const layout_t* L, int64_t v) { return L->v_para[v]; }
int64_t nd_oracle_e_para(const layout_t* L, int64_t e) { return L->e_para[e]; }
int64_t nd_oracle_e_data(const layout_t* L, int64_t e) { return L->e_data[e]; }
int nd_oracle_depth(const layout_t* L) { return L->depth; }
int64_t nd_oracle_n_out(const layout_t* L) { return L->lastidx_out; }
int64_t nd_oracle_n_aggr(const layout_t* L) { return L->lastidx_aggr; }

/*
 * The RHS, once per precision.  Steps and line references follow src/coreloop.jl.
 * Workspace o (lastidx_out) and aggbuf (lastidx_aggr) are caller-provided.
 *
 * Component functions (test/ComponentLibrary.jl, benchmark/benchmark_models.jl):
 *   diffusionedge!   e = p * (v_s - v_d)                 :8-13
 *   diffusion_edge!  e = v_s - v_d                       test/diffusion_test.jl:57-60
 *   kuramoto_edge!   e = K * sin(θ_s - θ_d)              :51-57
 *   diffusion_dedge! de1 = 1/τ * (sin(v_s - v_d) - e1), de2 = 1/τ * (sin(v_d - v_s) - e2)
 *                    with outputs Fiducial(dst=1:1, src=2:2)   :30-40; the benchmark
 *                    variant has 100.0 in place of 1/τ (benchmark_models.jl:11-16)
 *   AntiSymmetric    y_src = -y_dst                      src/component_functions.jl:117-126
 *   Symmetric        y_src = y_dst                       :142-151
 *   Directed         y_src = 0                           :167-175
 *   diffusionedge_fid! (two-sided)  e_d = p * (v_s - v_d), e_s = -e_d   :22-28
 *   diffusionvertex! dv = acc                            :42-46
 *   kuramoto_vertex! dθ = ω + esum                       :69-72
 *   kuramoto_inertia! dv1 = v2; dv2 = 1/M*(Pm - D*v2 + acc)  :59-67
 *   kuramoto_inertia! (benchmarks) dv1 = v2; dv2 = P - 1.0*v2; dv2 += esum
 *                    benchmark_models.jl:37-42 (the literal 1.0 is a Float64, so for
 *                    Float32 data P - 1.0*v2 is computed in double and rounded on store)
 * Power-grid components (outputs and inputs of dimension 2, a complex number):
 *   piline!          two-sided π-line currents                   benchmark_models.jl:46-63
 *   pq!              algebraic PQ bus: du = S / conj(i)          :65-73
 *   gen!             4-state generator                           :76-109
 * Complex arithmetic follows Julia's definitions operation by operation: the product
 * (ac - bd, ad + bc), and division by the robust method of Baudin & Smith ("A Robust
 * Complex Division in Scilab", 2012, with their improved r = 0 / br = 0 branches) that
 * Julia's Base uses; its range scaling only acts near the overflow / underflow thresholds,
 * which these models never reach, and is left out.
 */
#define DEFINE_COMPLEX(T, SFX)                                                                      \
    static inline void cdiv2_##SFX(T a, T b, T c, T d, T r, T t, T* out) {                         \
        if (r != 0) {                                                                               \
            T br = b * r;                                                                           \
            *out = br != 0 ? (a + br) * t : a * t + (b * t) * r;                                    \
        } else {                                                                                    \
            *out = (a + d * (b / c)) * t;                                                           \
        }                                                                                           \
    }                                                                                               \
    static inline void cdiv1_##SFX(T a, T b, T c, T d, T* p, T* q) {                               \
        T r = d / c;                                                                                \
        T t = (T)1 / (c + d * r);                                                                   \
        cdiv2_##SFX(a, b, c, d, r, t, p);                                                           \
        cdiv2_##SFX(b, -a, c, d, r, t, q);                                                          \
    }                                                                                               \
    /* (a + bi) / (c + di) */                                                                       \
    static inline void cdiv_##SFX(T a, T b, T c, T d, T* re, T* im) {                              \
        T p, q;                                                                                     \
        if (fabs((double)d) <= fabs((double)c)) {                                                   \
            cdiv1_##SFX(a, b, c, d, &p, &q);                                                        \
        } else {                                                                                    \
            cdiv1_##SFX(b, a, d, c, &p, &q);                                                        \
            q = -q;                                                                                 \
        }                                                                                           \
        *re = p;                                                                                    \
        *im = q;                                                                                    \
    }                                                                                               \
    static inline void cmul_##SFX(T a, T b, T c, T d, T* re, T* im) {                              \
        *re = a * c - b * d;                                                                        \
        *im = a * d + b * c;                                                                        \
    }
DEFINE_COMPLEX(double, f64)
DEFINE_COMPLEX(float, f32)

/* 2π·50 as Julia evaluates 2π*50 in Float64 */
#define PILINE_OMEGA 314.1592653589793

#define DEFINE_ORACLE_RHS(T, SFX, SIN, COS)                                                              \
    static inline T edge_g_##SFX(int ek, T vs, T vd, const T* pe) {                                \
        if (ek == E_DIFFUSION) return pe[0] * (vs - vd);                                            \
        if (ek == E_DIFFUSION_UNIT) return vs - vd;                                                 \
        return pe[0] * SIN(vs - vd);                                                                \
    }                                                                                               \
    static inline void vertex_f_##SFX(int vk, T* du, const T* u, const T* pv, const T* in,         \
                                      const double* cst) {                                          \
        T acc = in[0];                                                                              \
        if (vk == V_DIFFUSION) {                                                                    \
            du[0] = acc;                                                                            \
        } else if (vk == V_KURAMOTO) {                                                              \
            du[0] = pv[0] + acc;                                                                    \
        } else if (vk == V_SWING) {                                                                 \
            T M = pv[0], D = pv[1], Pm = pv[2];                                                     \
            du[0] = u[1];                                                                           \
            du[1] = (T)1 / M * (Pm - D * u[1] + acc);                                               \
        } else if (vk == V_SWING_UNIT) {                                                            \
            du[0] = u[1];                                                                           \
            du[1] = (T)((double)pv[0] - 1.0 * (double)u[1]);                                       \
            du[1] = du[1] + acc;                                                                    \
        } else if (vk == V_PQ) { /* uc = S / conj(ic) */                                            \
            cdiv_##SFX(pv[0], pv[1], in[0], -in[1], &du[0], &du[1]);                                \
        } else if (vk == V_PQ_CONST) { /* the same with the P, Q the closure captured */            \
            cdiv_##SFX((T)cst[0], (T)cst[1], in[0], -in[1], &du[0], &du[1]);                        \
        } else { /* gen! */                                                                         \
            T H = pv[0], P = pv[1], D = pv[2], Om = pv[3], E_f = pv[4], T_d_dash = pv[5];           \
            T T_q_dash = pv[6], X_q_dash = pv[7], X_d_dash = pv[8], X_d = pv[9], X_q = pv[10];      \
            T Om_H = Om / ((T)2 * H);                                                               \
            T ir = in[0], ii = in[1], ur = u[0], ui = u[1], th = u[2], w = u[3];                    \
            T c = COS(-th), sn = SIN(-th); /* exp(-im*θ): exp(±0) = 1 times cis(-θ) */               \
            T ic_r, ic_i, ec_r, ec_i, pr, pim;                                                      \
            cmul_##SFX(-ii, ir, c, sn, &ic_r, &ic_i);    /* (im*i)*exp(-im*θ), im*i = (-ii, ir) */  \
            cmul_##SFX(-ui, ur, c, sn, &ec_r, &ec_i);    /* (im*u)*exp(-im*θ) */                    \
            cmul_##SFX(ur, ui, ir, -ii, &pr, &pim);      /* u*conj(i) */                            \
            T de_d = (T)1 / T_q_dash * (-ec_r + (X_q - X_q_dash) * ic_i);                           \
            T de_q = (T)1 / T_d_dash * (-ec_i - (X_d - X_d_dash) * ic_r + E_f);                     \
            T t_r, t_i;                                                                             \
            cmul_##SFX(de_q, -de_d, COS(th), SIN(th), &t_r, &t_i); /* (-im*de_c)*exp(im*θ) */       \
            du[0] = t_r + (-ui) * w;                     /* + (u*im)*ω, u*im = (-ui, ur) */         \
            du[1] = t_i + ur * w;                                                                   \
            du[2] = w;                                                                              \
            du[3] = (P - D * w - pr - (X_q_dash - X_d_dash) * ic_r * ic_i) * Om_H;                  \
        }                                                                                           \
    }                                                                                               \
    /* edge g: ODE edges map their states (PureStateMap, :41), static edges evaluate g */         \
    /* on the vertex outputs (PureFeedForward, :76-78) and apply their wrapper */                   \
    static void edges_g_##SFX(const layout_t* L, T* o, const T* u, const T* p, int64_t k) {        \
        int64_t e = L->ebatch_order[k];                                                             \
        int ek = L->ekind[e];                                                                       \
        if (is_ode_edge(ek)) {                                                                      \
            o[L->e_out_dst[e]] = u[L->e_data[e]];                                                   \
            o[L->e_out_src[e]] = u[L->e_data[e] + 1];                                               \
            return;                                                                                 \
        }                                                                                           \
        if (ek == E_PILINE) { /* piline!: two-sided, complex currents */                            \
            const T* pe = p + L->e_para[e];                                                         \
            T Lh = pe[0], R = pe[1], C1 = pe[2], C2 = pe[3], w = (T)PILINE_OMEGA;                   \
            const T* vs = o + L->v_out[L->src[e]];                                                  \
            const T* vd = o + L->v_out[L->dst[e]];                                                  \
            T im_r, im_i;                                                                           \
            cdiv_##SFX(vs[0] - vd[0], vs[1] - vd[1], R, w * Lh, &im_r, &im_i); /* R + im*ω*L */     \
            T c1_r = (-vs[1]) * w * C1, c1_i = vs[0] * w * C1; /* Vsrc*im*ω*C1 */                   \
            T c2_r = (-vd[1]) * w * C2, c2_i = vd[0] * w * C2;                                      \
            T is_r = -(im_r + c1_r), is_i = -(im_i + c1_i);                                         \
            T id_r = im_r - c2_r, id_i = im_i - c2_i;                                               \
            o[L->e_out_dst[e]] = -id_r;                                                             \
            o[L->e_out_dst[e] + 1] = -id_i;                                                         \
            o[L->e_out_src[e]] = -is_r;                                                             \
            o[L->e_out_src[e] + 1] = -is_i;                                                         \
            return;                                                                                 \
        }                                                                                           \
        T vs = o[L->v_out[L->src[e]]], vd = o[L->v_out[L->dst[e]]];                                 \
        T y = edge_g_##SFX(ek, vs, vd, p + L->e_para[e]);                                           \
        o[L->e_out_dst[e]] = y;                                                                     \
        int c = L->ecoup[e];                                                                        \
        o[L->e_out_src[e]] = c == C_SYMMETRIC ? y : (c == C_DIRECTED ? (T)0 : -y);                  \
    }                                                                                               \
    /* edge f of the ODE edges (:71) */                                                             \
    static void edges_f_##SFX(const layout_t* L, T* du, const T* u, const T* o, const T* p,         \
                              int64_t k) {                                                          \
        int64_t e = L->ebatch_order[k];                                                             \
        int ek = L->ekind[e];                                                                       \
        if (!is_ode_edge(ek)) return;                                                               \
        T vs = o[L->v_out[L->src[e]]], vd = o[L->v_out[L->dst[e]]];                                 \
        const T* x = u + L->e_data[e];                                                              \
        T* dx = du + L->e_data[e];                                                                  \
        if (ek == E_DIFFUSION_ODE) {                                                                \
            T tau = p[L->e_para[e]];                                                                \
            dx[0] = (T)1 / tau * (SIN(vs - vd) - x[0]);                                             \
            dx[1] = (T)1 / tau * (SIN(vd - vs) - x[1]);                                             \
        } else {                                                                                    \
            dx[0] = (T)100.0 * (SIN(vs - vd) - x[0]);                                               \
            dx[1] = (T)100.0 * (SIN(vd - vs) - x[1]);                                               \
        }                                                                                           \
    }                                                                                               \
    void nd_oracle_rhs_##SFX(const layout_t* L, T* du, const T* u, const T* p, T* o, T* aggbuf) {   \
        int64_t i;                                                                                  \
        for (i = 0; i < L->lastidx_dynamic; ++i) du[i] = 0;       /* fill!(du, 0)      :24 */       \
        for (i = 0; i < L->lastidx_out; ++i) o[i] = (T)NAN;       /* fill!(o, NaN)  ns:153 */       \
        for (i = 0; i < L->lastidx_aggr; ++i) aggbuf[i] = 0;      /* fill!(aggbuf, 0)  :30 */       \
        for (int64_t k = 0; k < L->nv; ++k) {                     /* vertex g, StateMask :39 */     \
            int64_t v = L->vbatch_order[k];                                                         \
            for (int j = 0; j < L->depth; ++j) o[L->v_out[v] + j] = u[L->v_data[v] + j];            \
        }                                                                                           \
        for (int64_t k = 0; k < L->ne; ++k) edges_g_##SFX(L, o, u, p, k);                           \
        for (int64_t k = 0; k < L->ne; ++k) edges_f_##SFX(L, du, u, o, p, k);                       \
        /* SequentialAggregator: walk the tightened output range in index order :90 */              \
        for (int64_t j = 0; j < L->agg_len; ++j) {                                                  \
            int64_t m = L->agg_map[j];                                                              \
            if (m != 0) aggbuf[m - 1] = aggbuf[m - 1] + o[L->agg_first + j];                        \
        }                                                                                           \
        for (int64_t k = 0; k < L->nv; ++k) {                     /* vertex f :97 */                \
            int64_t v = L->vbatch_order[k];                                                         \
            vertex_f_##SFX(L->vkind[v], du + L->v_data[v], u + L->v_data[v], p + L->v_para[v],      \
                           aggbuf + L->v_aggr[v], L->vconst + 2 * v);                               \
        }                                                                                           \
    }                                                                                               \
    void nd_oracle_rhs_poly_##SFX(const layout_t* L, T* du, const T* u, const T* p, T* o,           \
                                  T* aggbuf) {                                                      \
        int64_t i;                                                                                  \
        _Pragma("omp parallel for schedule(static)") for (i = 0; i < L->lastidx_dynamic; ++i) du[i] = 0; \
        _Pragma("omp parallel for schedule(static)") for (i = 0; i < L->lastidx_aggr; ++i) aggbuf[i] = 0; \
        _Pragma("omp parallel for schedule(static)") for (i = 0; i < L->nv; ++i) {                 \
            int64_t v = L->vbatch_order[i];                                                         \
            for (int j = 0; j < L->depth; ++j) o[L->v_out[v] + j] = u[L->v_data[v] + j];            \
        }                                                                                           \
        _Pragma("omp parallel for schedule(static)") for (i = 0; i < L->ne; ++i)                   \
            edges_g_##SFX(L, o, u, p, i);                                                           \
        _Pragma("omp parallel for schedule(static)") for (i = 0; i < L->ne; ++i)                   \
            edges_f_##SFX(L, du, u, o, p, i);                                                       \
        _Pragma("omp parallel for schedule(static)") for (i = 0; i < L->lastidx_aggr; ++i) {       \
            T acc = aggbuf[i];                                                                      \
            for (int64_t q = L->inv_ptr[i]; q < L->inv_ptr[i + 1]; ++q) acc = acc + o[L->inv_idx[q]]; \
            aggbuf[i] = acc;                                                                        \
        }                                                                                           \
        _Pragma("omp parallel for schedule(static)") for (i = 0; i < L->nv; ++i) {                 \
            int64_t v = L->vbatch_order[i];                                                         \
            vertex_f_##SFX(L->vkind[v], du + L->v_data[v], u + L->v_data[v], p + L->v_para[v],      \
                           aggbuf + L->v_aggr[v], L->vconst + 2 * v);                               \
        }                                                                                           \
    }

DEFINE_ORACLE_RHS(double, f64, sin, cos)
DEFINE_ORACLE_RHS(float, f32, sinf, cosf)

int nd_oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void nd_oracle_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/*
 * Tsit5 — Tsitouras, "Runge–Kutta pairs of order 5(4) satisfying only the first column
 * simplifying assumption", Comput. Math. Appl. 62 (2011) 770-775: the published 7-stage
 * FSAL tableau (b equals the last row of a) and the embedded error weights btilde.
 * Step control: RMS norm of err_i / (abstol + reltol * max(|u_i|, |u_new_i|)), a PI
 * controller with beta1 = 7/50, beta2 = 2/25, safety 9/10, step ratio clamped to
 * [1/10, 5] (as q in [1/5, 10]), and the Hairer–Wanner initial step.  The reference
 * delegates all of this to OrdinaryDiffEqTsit5 (solve(prob, Tsit5()),
 * test/diffusion_test.jl:119-120); the controller constants restate that solver's
 * documented defaults.
 */
static const double TS_C[7] = {0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0};
static const double TS_A[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {0.161, 0, 0, 0, 0, 0},
    {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0},
    {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0},
    {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0},
    {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0},
    {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774}};
static const double TS_BTILDE[7] = {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
                                    -0.1447110071732629,     0.5823571654525552,     -0.45808210592918697,
                                    0.015151515151515152};

void nd_oracle_tsit5_tableau(double* c, double* a, double* btilde) {
    for (int i = 0; i < 7; ++i) {
        c[i] = TS_C[i];
        btilde[i] = TS_BTILDE[i];
        for (int j = 0; j < 6; ++j) a[i * 6 + j] = TS_A[i][j];
    }
}

typedef struct {
    int64_t naccept, nreject, nf;
    double t_final, dt_last;
    int status; /* 0 ok, -5 max steps, -8 dt underflow */
} tsit5_stats_t;

static double rms_scaled(int64_t n, const double* e, const double* u0, const double* u1, double abstol,
                         double reltol) {
    double s = 0;
    for (int64_t i = 0; i < n; ++i) {
        double sc = abstol + reltol * fmax(fabs(u0[i]), fabs(u1[i]));
        double r = e[i] / sc;
        s += r * r;
    }
    return sqrt(s / (double)(n > 0 ? n : 1));
}

/* threaded != 0: the RHS is the PolyesterExecution restatement and the stage updates run on
 * all threads.  Both give the same bits as the sequential code (the RHS per vertex sums in
 * the same order; the stage updates are elementwise); the error norm stays sequential. */
static int tsit5_impl(const layout_t* L, double* u, const double* p, double t0, double t1, double reltol,
                      double abstol, int64_t maxsteps, tsit5_stats_t* st, int threaded) {
#define TS_RHS(out, in) \
    (threaded ? nd_oracle_rhs_poly_f64(L, out, in, p, o, ab) : nd_oracle_rhs_f64(L, out, in, p, o, ab))
    int64_t n = L->lastidx_dynamic;
    double* k[7];
    for (int i = 0; i < 7; ++i) k[i] = (double*)malloc(sizeof(double) * (size_t)(n + 1));
    double* y = (double*)malloc(sizeof(double) * (size_t)(n + 1));
    double* un = (double*)malloc(sizeof(double) * (size_t)(n + 1));
    double* err = (double*)malloc(sizeof(double) * (size_t)(n + 1));
    double* o = (double*)malloc(sizeof(double) * (size_t)(L->lastidx_out + 1));
    double* ab = (double*)malloc(sizeof(double) * (size_t)(L->lastidx_aggr + 1));
    memset(st, 0, sizeof(*st));
    double t = t0, tdir = t1 >= t0 ? 1.0 : -1.0;
    TS_RHS(k[0], u);
    st->nf++;
    /* Hairer–Wanner initial step (order 5). */
    double d0 = 0, d1 = 0;
    for (int64_t i = 0; i < n; ++i) {
        double sc = abstol + fabs(u[i]) * reltol;
        d0 += (u[i] / sc) * (u[i] / sc);
        d1 += (k[0][i] / sc) * (k[0][i] / sc);
    }
    d0 = sqrt(d0 / (double)(n ? n : 1));
    d1 = sqrt(d1 / (double)(n ? n : 1));
    double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
    h0 = fmin(h0, fabs(t1 - t0));
    for (int64_t i = 0; i < n; ++i) y[i] = u[i] + tdir * h0 * k[0][i];
    TS_RHS(k[1], y);
    st->nf++;
    double d2 = 0;
    for (int64_t i = 0; i < n; ++i) {
        double sc = abstol + fabs(u[i]) * reltol;
        double r = (k[1][i] - k[0][i]) / sc;
        d2 += r * r;
    }
    d2 = sqrt(d2 / (double)(n ? n : 1)) / h0;
    double h1 = (fmax(d1, d2) <= 1e-15) ? fmax(1e-6, h0 * 1e-3) : pow(0.01 / fmax(d1, d2), 1.0 / 5.0);
    double dt = fmin(fmin(100 * h0, h1), fabs(t1 - t0));
    const double beta1 = 7.0 / 50.0, beta2 = 2.0 / 25.0, gamma = 0.9, qmin = 0.2, qmax = 10.0;
    double qold = 1e-4;
    int64_t steps = 0;
    int status = 0;
    while (tdir * (t1 - t) > 0) {
        if (steps++ >= maxsteps) {
            status = -5;
            break;
        }
        if (fabs(t1 - t) < dt * (1 + 1e-12)) dt = fabs(t1 - t);
        double h = tdir * dt;
        for (int s = 1; s < 7; ++s) {
            int64_t i;
            _Pragma("omp parallel for schedule(static) if (threaded)") for (i = 0; i < n; ++i) {
                double acc = 0;
                for (int j = 0; j < s; ++j) acc += TS_A[s][j] * k[j][i];
                y[i] = u[i] + h * acc;
            }
            TS_RHS(k[s], y);
            st->nf++;
            if (s == 6) memcpy(un, y, sizeof(double) * (size_t)n);
        }
        int64_t i;
        _Pragma("omp parallel for schedule(static) if (threaded)") for (i = 0; i < n; ++i) {
            double acc = 0;
            for (int j = 0; j < 7; ++j) acc += TS_BTILDE[j] * k[j][i];
            err[i] = h * acc;
        }
        double EEst = rms_scaled(n, err, u, un, abstol, reltol);
        if (!(EEst == EEst)) EEst = 1e10; /* NaN: reject */
        double q11 = pow(EEst, beta1);
        if (EEst <= 1.0) {
            double q = q11 / pow(qold, beta2);
            q = fmax(1.0 / qmax, fmin(1.0 / qmin, q / gamma));
            t = (fabs(t1 - t - h) <= 1e-14 * fmax(1.0, fabs(t1))) ? t1 : t + h;
            memcpy(u, un, sizeof(double) * (size_t)n);
            memcpy(k[0], k[6], sizeof(double) * (size_t)n); /* FSAL */
            qold = fmax(EEst, 1e-4);
            st->naccept++;
            dt = dt / q;
        } else {
            st->nreject++;
            dt = dt / fmin(1.0 / qmin, q11 / gamma);
        }
        if (dt < 1e-14 * fmax(1.0, fabs(t))) {
            status = -8;
            break;
        }
    }
    st->t_final = t;
    st->dt_last = dt;
    st->status = status;
    for (int i = 0; i < 7; ++i) free(k[i]);
    free(y);
    free(un);
    free(err);
    free(o);
    free(ab);
    return status;
#undef TS_RHS
}

int nd_oracle_tsit5(const layout_t* L, double* u, const double* p, double t0, double t1, double reltol,
                    double abstol, int64_t maxsteps, tsit5_stats_t* st) {
    return tsit5_impl(L, u, p, t0, t1, reltol, abstol, maxsteps, st, 0);
}

int nd_oracle_tsit5_threaded(const layout_t* L, double* u, const double* p, double t0, double t1, double reltol,
                             double abstol, int64_t maxsteps, tsit5_stats_t* st) {
    return tsit5_impl(L, u, p, t0, t1, reltol, abstol, maxsteps, st, 1);
}

/* ------------------------------------------------------------------------------------------
 * Barabási–Albert graph for the CPU reference arm of the benchmark, so that the arm loads
 * nothing outside this directory.  It restates the package's seeded generator (splitmix64-
 * seeded xoshiro256**, unbiased bounded draws, m initial isolated vertices, every later
 * vertex attaching m edges to distinct earlier vertices drawn from the endpoint list) and
 * returns the edges(g) order: (src < dst), sorted lexicographically.  A CPU test checks
 * that both generators give the same edge lists.
 * ------------------------------------------------------------------------------------------ */
typedef struct {
    uint64_t s[4];
} gen_rng_t;

static uint64_t gen_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static void gen_seed(gen_rng_t* r, uint64_t seed) {
    uint64_t x = seed;
    for (int i = 0; i < 4; ++i) {
        x += 0x9E3779B97F4A7C15ull;
        uint64_t z = x;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        r->s[i] = z ^ (z >> 31);
    }
}

static uint64_t gen_next(gen_rng_t* r) {
    const uint64_t out = gen_rotl(r->s[1] * 5, 7) * 9;
    const uint64_t t = r->s[1] << 17;
    r->s[2] ^= r->s[0];
    r->s[3] ^= r->s[1];
    r->s[1] ^= r->s[2];
    r->s[0] ^= r->s[3];
    r->s[2] ^= t;
    r->s[3] = gen_rotl(r->s[3], 45);
    return out;
}

static uint64_t gen_below(gen_rng_t* r, uint64_t n) {
    const uint64_t lim = UINT64_MAX - UINT64_MAX % n;
    uint64_t x;
    do x = gen_next(r);
    while (x >= lim);
    return x % n;
}

static int cmp_i64(const void* a, const void* b) {
    const int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
    return (x > y) - (x < y);
}

/* Returns the number of edges (written up to cap), -1 on bad arguments, -2 out of memory. */
int64_t nd_oracle_gen_barabasi_albert(int64_t n, int64_t m, uint64_t seed, int64_t* src, int64_t* dst, int64_t cap) {
    if (m < 1 || n <= m) return -1;
    const int64_t np = m * (n - m);
    int64_t* ends = (int64_t*)malloc(sizeof(int64_t) * (size_t)(2 * np));
    int64_t* ps = (int64_t*)malloc(sizeof(int64_t) * (size_t)np);
    int64_t* pd = (int64_t*)malloc(sizeof(int64_t) * (size_t)np);
    int64_t* chosen = (int64_t*)malloc(sizeof(int64_t) * (size_t)m);
    int64_t* cnt = (int64_t*)calloc((size_t)(n + 1), sizeof(int64_t));
    int64_t* col = (int64_t*)malloc(sizeof(int64_t) * (size_t)np);
    if (!ends || !ps || !pd || !chosen || !cnt || !col) {
        free(ends), free(ps), free(pd), free(chosen), free(cnt), free(col);
        return -2;
    }
    gen_rng_t rng;
    gen_seed(&rng, seed);
    int64_t ne_ends = 0, npairs = 0;
    for (int64_t v = m; v < n; ++v) {
        int64_t nc = 0;
        if (v == m) {
            for (int64_t t = 0; t < m; ++t) chosen[nc++] = t;
        } else {
            while (nc < m) {
                const int64_t t = ends[gen_below(&rng, (uint64_t)ne_ends)];
                int dup = 0;
                for (int64_t q = 0; q < nc; ++q) dup |= chosen[q] == t;
                if (!dup) chosen[nc++] = t;
            }
        }
        for (int64_t q = 0; q < m; ++q) {
            ps[npairs] = chosen[q];
            pd[npairs] = v;
            ++npairs;
            ends[ne_ends++] = chosen[q];
            ends[ne_ends++] = v;
        }
    }
    /* counting sort by source (chosen < v always), then each source's targets sorted */
    for (int64_t i = 0; i < npairs; ++i) cnt[ps[i] + 1]++;
    for (int64_t i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    int64_t* fill = ends; /* reused: n entries are enough (2 np >= n since m >= 1, n > m) */
    for (int64_t i = 0; i < n; ++i) fill[i] = cnt[i];
    for (int64_t i = 0; i < npairs; ++i) col[fill[ps[i]]++] = pd[i];
    int64_t ne = 0;
    for (int64_t s = 0; s < n; ++s) {
        qsort(col + cnt[s], (size_t)(cnt[s + 1] - cnt[s]), sizeof(int64_t), cmp_i64);
        int64_t last = -1;
        for (int64_t k = cnt[s]; k < cnt[s + 1]; ++k) {
            if (col[k] == last || col[k] == s) continue;
            last = col[k];
            if (ne < cap) {
                src[ne] = s;
                dst[ne] = col[k];
            }
            ++ne;
        }
    }
    free(ends), free(ps), free(pd), free(chosen), free(cnt), free(col);
    return ne;
}
