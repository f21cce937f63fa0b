/*
 * nd_gb300.h — C ABI of libnd_b200.so, the GB300 (sm_103a) network right-hand side
 * of NetworkDynamics.jl and the solvers built on it.
 *
 * Everything here is plain C: pointers, sizes and status codes, no CUDA or torch
 * types in the signatures.  Device pointers are CUDA device addresses; `stream` is a
 * cudaStream_t passed as void* (NULL = legacy default stream).  All calls that take a
 * stream are stream-ordered: they enqueue work and return without synchronising,
 * unless stated otherwise.
 *
 * Reference paths cited below are relative to the NetworkDynamics.jl source tree.
 */
#ifndef ND_GB300_H
#define ND_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ND_VERSION 10000 /* 1.0.0 */

/* ---------------------------------------------------------------------------------
 * Status codes.  The reference raises Julia exceptions; the C ABI returns a code and
 * keeps a thread-local message (nd_last_error).  The Julia shim maps ND_ERR_ARG and
 * ND_ERR_DTYPE to ArgumentError (src/coreloop.jl:2-7, src/network_structure.jl:146-150),
 * ND_ERR_UNSUPPORTED_COMPONENT to ArgumentError at construction, and
 * ND_ERR_NOT_CONVERGED to NetworkInitError (src/initialization.jl:86-142).
 * ------------------------------------------------------------------------------- */
enum nd_status {
    ND_OK = 0,
    ND_ERR_ARG = -1,                   /* bad size, pointer or descriptor field            */
    ND_ERR_UNSUPPORTED_COMPONENT = -2, /* component outside the hand-written library       */
    ND_ERR_DTYPE = -3,                 /* buffer eltype differs from the handle precision  */
    ND_ERR_CUDA = -4,                  /* a CUDA runtime call failed                       */
    ND_ERR_MAXITERS = -5,              /* a solver hit its step / iteration budget         */
    ND_ERR_UNSUPPORTED = -6,           /* feature outside the GB300 path (perturb, RET...) */
    ND_ERR_NOMEM = -7,                 /* device allocation failed                         */
    ND_ERR_NOT_CONVERGED = -8,         /* Newton / fixpoint did not reach the tolerance    */
    ND_ERR_DEVICE_CHECK = -9           /* a device-side check found a bad index (checks on) */
};

/* Element type of caller buffers.  A handle is built for one of them, like
 * adapt(CuArray{Float32}/CuArray{Float64}, nw) (ext/NetworkDynamicsCUDAExt.jl:16-45).
 * ND_F32X2 (ensembles only; no counterpart in the reference): FP64 buffers, RHS arithmetic
 * in double-float (pairs of floats, ~48-bit significands) on the FP32 pipe. */
enum nd_dtype { ND_F32 = 1, ND_F64 = 2, ND_F32X2 = 3 };

/* Hand-written component library.  Anything else is rejected with
 * ND_ERR_UNSUPPORTED_COMPONENT: there is no CPU fallback. */
enum nd_vertex_kind {
    ND_V_DIFFUSION = 1, /* diffusionvertex!  dv = Σe                 test/ComponentLibrary.jl:42-46   dim 1, pdim 0          */
    ND_V_KURAMOTO = 2,  /* kuramoto_vertex!  dθ = ω + Σe             test/ComponentLibrary.jl:69-72   dim 1, pdim 1 (ω)      */
    ND_V_SWING = 3,     /* kuramoto_inertia! dθ = ω, dω = (Pm-Dω+Σe)/M test/ComponentLibrary.jl:59-67 dim 2, pdim 3 (M,D,Pm) */
    ND_V_SWING_UNIT = 4, /* kuramoto_inertia! of the benchmarks: dθ = ω, dω = (P - 1.0ω) + Σe
                           benchmark/benchmark_models.jl:37-42                                 dim 2, pdim 1 (P)      */
    /* Power-grid vertices: complex voltage output (StateMask(1:2)), complex current input. */
    ND_V_PQ = 5,        /* pq!  algebraic PQ bus (mass matrix 0): du = S / conj(i), S = P + iQ
                           benchmark/benchmark_models.jl:65-74                                 dim 2, pdim 2 (P,Q)    */
    ND_V_GENERATOR = 6, /* gen!  generator with states (u_r, u_i, θ, ω)
                           benchmark/benchmark_models.jl:76-111                                dim 4, pdim 11         */
    ND_V_PQ_CONST = 7   /* pq! of pqnode_inhomogeneous: the PQ bus closing over its own P, Q,
                           taken from its batch's constants (P, Q)   benchmark_models.jl:113-123  dim 2, pdim 0 */
};
enum nd_edge_kind {
    ND_E_DIFFUSION = 1,      /* diffusionedge!   e = w·(vs-vd)   test/ComponentLibrary.jl:8-13   pdim 1 (w) */
    ND_E_DIFFUSION_UNIT = 2, /* diffusion_edge!  e = vs-vd       test/diffusion_test.jl:57-60    pdim 0     */
    ND_E_KURAMOTO = 3,       /* kuramoto_edge! / static power line  e = K·sin(vs-vd)
                                test/ComponentLibrary.jl:51-57, :96-115                          pdim 1 (K) */
    /* Edges with states (ODE edges).  States (e1, e2); outputs Fiducial(dst=1, src=2):
     * y_dst = e1, y_src = e2. */
    ND_E_DIFFUSION_ODE = 4,      /* diffusion_dedge!  de1 = 1/τ·(sin(vs-vd) - e1), de2 = 1/τ·(sin(vd-vs) - e2)
                                    test/ComponentLibrary.jl:30-40                  dim 2, pdim 1 (τ)  */
    ND_E_DIFFUSION_ODE_FIXED = 5, /* the same with the rate fixed: de = 100.0·(sin(..) - e)
                                    benchmark/benchmark_models.jl:11-16             dim 2, pdim 0      */
    ND_E_PILINE = 6               /* piline!  two-sided π-line currents (complex outputs), coupling
                                    ND_FIDUCIAL   benchmark/benchmark_models.jl:46-63  pdim 4 (L,R,C1,C2) */
};
/* All vertex models of a network share one output dimension, and all edge models one
 * (src/construction.jl:98-106): 1 for kinds 1-5 / 1-3, 2 (a complex value) for
 * ND_V_PQ, ND_V_GENERATOR and ND_E_PILINE.  A mix is ND_ERR_ARG. */
/* Output wrapper of the edge (src/component_functions.jl:101-203):
 *   ND_ANTISYMMETRIC  y_dst = g(...), y_src = -y_dst          (:117-126)
 *   ND_SYMMETRIC      y_dst = g(...), y_src = y_dst           (:142-151)
 *   ND_DIRECTED       y_dst = g(...), y_src = 0               (:167-175)
 *   ND_FIDUCIAL       separate src / dst outputs: Fiducial(src, dst) of StateMasks
 *                     (:190-203), the outputs of the ODE kinds, and the two-sided
 *                     diffusionedge_fid! (test/ComponentLibrary.jl:22-28: y_dst = w·(vs-vd),
 *                     y_src = -y_dst), the only static kind that takes ND_FIDUCIAL.
 * Static kinds take the first three; ND_FIDUCIAL is the only coupling of the ODE kinds. */
enum nd_coupling { ND_ANTISYMMETRIC = 1, ND_SYMMETRIC = 2, ND_DIRECTED = 3, ND_FIDUCIAL = 4 };

/* Summation order of the per-vertex edge aggregation. */
enum nd_sum_order {
    ND_ORDER_SEQUENTIAL = 0,   /* ascending out-buffer index, = SequentialAggregator (bitwise);
                                  FP64 adds run as exact integer arithmetic, hubs as an exact scan */
    ND_ORDER_TREE = 1,         /* deterministic tree inside a warp at hubs (not bitwise)          */
    ND_ORDER_SEQUENTIAL_HW = 2 /* the sequential order with hardware FP64 adds (bitwise, slower on
                                  GB300, whose FP64 pipe is 1/64 of FP32)                         */
};

/* Network description, the information Network(g, vertexm, edgem) holds
 * (src/construction.jl:31-236).  Edges are given in Graphs.jl `edges(g)` order with
 * 0-based endpoints; edge k owns parameter slot k of the edge parameter block (and, for
 * ODE edges, states 2k, 2k+1 of the edge state block after the vertex states).  One
 * homogeneous vertex batch and one homogeneous edge batch; nd_create_batched takes
 * several. */
typedef struct nd_network_desc {
    int64_t nv;          /* number of vertices                           */
    int64_t ne;          /* number of edges                              */
    const int64_t* src;  /* [ne] host pointer, 0-based source vertex      */
    const int64_t* dst;  /* [ne] host pointer, 0-based destination vertex */
    int32_t vertex_kind; /* enum nd_vertex_kind                          */
    int32_t edge_kind;   /* enum nd_edge_kind                            */
    int32_t coupling;    /* enum nd_coupling                             */
    int32_t flags;       /* reserved, must be 0                          */
} nd_network_desc;

/* Sizes of the flat reference layout (src/network_structure.jl:224-289). */
typedef struct nd_info {
    int64_t dim;          /* lastidx_dynamic: length of u and du            */
    int64_t pdim;         /* lastidx_p: length of p                         */
    int64_t nv;           /* vertices                                       */
    int64_t ne;           /* edges                                          */
    int64_t n_incidences; /* 2·ne entries of the destination-sorted CSR     */
    int32_t dtype;        /* enum nd_dtype of the handle                    */
    int32_t vertex_kind;
    int32_t edge_kind;
    int32_t max_degree;
    int32_t n_hubs;       /* vertices on the cooperative (warp / CTA) path   */
    int32_t sum_order;    /* enum nd_sum_order in use                       */
    int32_t n_vertex_batches; /* batches of the layout (1 for nd_create)    */
    int32_t n_edge_batches;
} nd_info;

typedef struct nd_handle nd_handle;

/* Library version (ND_VERSION). */
int nd_version(void);

/* Message of the last failing call on this host thread ("" if none). */
const char* nd_last_error(void);

/* Build a handle: validate the description, build the destination-sorted CSR with
 * degree buckets and upload it.  Replaces the aggregator constructor call
 * `aggregator(im, edgebatches)` (src/construction.jl:198) together with
 * Adapt.adapt_structure(CuArray{T}, nw) (ext/NetworkDynamicsCUDAExt.jl:16-45).
 * Uses the current CUDA device.  A description outside the static AntiSymmetric kinds
 * 1-3 (an ODE edge, another coupling, ND_V_SWING_UNIT) is built as a batched network of
 * one vertex and one edge batch (nd_create_batched). */
int nd_create(const nd_network_desc* desc, int dtype, nd_handle** out);

/* Heterogeneous networks: several vertex and edge batches, Network(g, vertexms, edgems)
 * with vectors of components (src/construction.jl:155-195).  The reference groups
 * identical components into batches in order of first appearance (find_identical,
 * src/utils.jl:197-216) and lays the flat vectors out batch by batch
 * (src/network_structure.jl:224-258): all vertex batches first (states, outputs,
 * parameters), then the edge batches (states after every vertex state, parameters after
 * every vertex parameter); inside a batch, components in ascending index order.  The
 * caller passes the batches in the reference's order and the batch of every component;
 * the handle then uses exactly that layout for u, du and p.
 *   batch kinds      vertex batches: enum nd_vertex_kind, coupling 0; edge batches:
 *                    enum nd_edge_kind with its enum nd_coupling (ND_ERR_UNSUPPORTED_COMPONENT
 *                    for a pair outside the library)
 *   n_*_batches      1..ND_MAX_BATCHES vertex batches; 0..ND_MAX_BATCHES edge batches (0
 *                    only without edges).  A batch may be empty.  Components that close
 *                    over values of their own (pqnode_inhomogeneous) are one batch per
 *                    distinct value, their values in vertex_constants.
 * The RHS follows the reference's order of operations and SequentialAggregator's order
 * of additions (ascending output index).  Networks of one static AntiSymmetric edge
 * batch and one vertex batch of kinds 1-3 take the same kernels as nd_create; all others
 * a batched two-kernel RHS (edge kernel with per-batch dispatch, then row sums and
 * vertex functions).  nd_jvp of a batched handle assembles the sparse Jacobian
 * (nd_jacobian) and multiplies; the ensemble calls do not take batched handles. */
#define ND_MAX_BATCHES (1 << 20)
#define ND_BATCH_CONSTANTS 2 /* numbers per vertex batch in vertex_constants */
typedef struct nd_batch {
    int32_t kind;     /* enum nd_vertex_kind / enum nd_edge_kind */
    int32_t coupling; /* edge batches: enum nd_coupling; vertex batches: 0 */
} nd_batch;
typedef struct nd_batched_network_desc {
    int64_t nv;                     /* number of vertices                              */
    int64_t ne;                     /* number of edges                                 */
    const int64_t* src;             /* [ne] host, 0-based, edges(g) order              */
    const int64_t* dst;             /* [ne] host                                       */
    int32_t n_vertex_batches;
    int32_t n_edge_batches;
    const nd_batch* vertex_batches; /* [n_vertex_batches] host                         */
    const nd_batch* edge_batches;   /* [n_edge_batches] host                           */
    const int32_t* vertex_batch;    /* [nv] host: batch index of every vertex          */
    const int32_t* edge_batch;      /* [ne] host: batch index of every edge            */
    int32_t flags;                  /* reserved, must be 0                             */
    int32_t reserved;
    const double* vertex_constants; /* [n_vertex_batches * ND_BATCH_CONSTANTS] host, or
                                       NULL: values a component closes over (the P, Q of
                                       ND_V_PQ_CONST); required when that kind is used  */
} nd_batched_network_desc;
int nd_create_batched(const nd_batched_network_desc* desc, int dtype, nd_handle** out);

/* Free the handle and its device buffers (the Julia finalizer calls this). */
int nd_destroy(nd_handle* h);

int nd_get_info(const nd_handle* h, nd_info* out);

/* Select the aggregation order (enum nd_sum_order).  Default ND_ORDER_SEQUENTIAL. */
int nd_set_sum_order(nd_handle* h, int order);

/* Kernel layout of the RHS.  ND_LAYOUT_AUTO (default) evaluates each edge once in edge
 * order and then sums the rows (two phases; needs the canonical edge list of an
 * undirected Graphs.jl graph: sorted by source, src < dst); other edge lists, or
 * ND_LAYOUT_FUSED, use one fused kernel over the destination-sorted CSR.  Both give the
 * same bits. */
enum nd_layout { ND_LAYOUT_AUTO = 0, ND_LAYOUT_FUSED = 1 };
int nd_set_layout(nd_handle* h, int layout);

/* Kernel accounting (no reference counterpart; a tracing aid like the reference's
 * benchmark timers, benchmark/benchmark_utils.jl).  Every nd_rhs call counts the kernels
 * it launches by kind.  With nd_set_kernel_timing(h, 1) it also brackets each launch with
 * two CUDA events on the launching stream (heavy rows: the handle's side stream); the
 * events make a captured graph record them too, so leave timing off while capturing.
 * nd_kernel_times synchronizes the recorded events and writes, for kinds 0..n-1, the
 * launches since the last call and their summed device time in ms (0 when timing was
 * off), then resets both.  Recorded events stay in the handle's pool until that call. */
enum nd_kernel_kind {
    ND_KERNEL_EDGE_PHASE = 0, /* one thread per edge: edge outputs y, bucketed by destination */
    ND_KERNEL_ROW_PHASE = 1,  /* row sums over y + vertex functions (rows of degree <= 2048) */
    ND_KERNEL_HEAVY_ROWS = 2, /* rows of degree > 2048, a block per row on the side stream */
    ND_KERNEL_FUSED = 3,      /* single-kernel RHS (ND_LAYOUT_FUSED or non-canonical edges) */
    ND_KERNEL_BATCHED_EDGES = 4, /* batched networks: edge functions of every edge batch */
    ND_KERNEL_BATCHED_ROWS = 5,  /* batched networks: row sums + vertex functions */
    ND_KERNEL_KINDS = 6
};
int nd_set_kernel_timing(nd_handle* h, int on);
int nd_kernel_times(nd_handle* h, int64_t* launches, double* ms, int n);

/* One network right-hand side du = f(u, p, t), the method
 * `(nw::Network)(du, u, p, t)` (src/coreloop.jl:1-102) for RET=:du and no perturbation,
 * with SequentialAggregator(+) semantics (src/aggregators.jl:133-151).
 *   dtype       element type of du/u/p; ND_ERR_DTYPE if it differs from the handle's
 *               (src/network_structure.jl:146-150)
 *   n_du, n_u   must equal info.dim, else ND_ERR_ARG (src/coreloop.jl:2-4)
 *   n_p         must equal info.pdim when pdim > 0, else ND_ERR_ARG (src/coreloop.jl:5-7);
 *               p may be NULL when pdim == 0
 *   t           unused by the library components, may be NaN
 * du, u, p are device pointers in the reference's flat order (no permutation). */
int nd_rhs(nd_handle* h, int dtype, void* du, int64_t n_du, const void* u, int64_t n_u,
           const void* p, int64_t n_p, double t, void* stream);

/* Analytic Jacobian-vector product jv = (∂f/∂u)(u, p, t) · v of the RHS, replacing the
 * ForwardDiff Dual-number pass through the core loop (src/coreloop.jl:10-21) for the
 * library components.  jv, u, v: device, length dim; p: device, length pdim; element type
 * of the handle.  Stream-ordered. */
int nd_jvp(nd_handle* h, int dtype, void* jv, const void* u, const void* p, const void* v, double t, void* stream);

/* Sparse Jacobian ∂f/∂u of the RHS in CSR form, rows and columns in the flat state order.
 * nd_jacobian_pattern replaces get_jac_prototype(nw) (ext/NetworkDynamicsSparsityExt.jl:
 * 57-127, SparseConnectivityTracer): the structural pattern of the library components
 * (columns sorted and unique per row; an entry may be numerically zero, e.g. for a self
 * loop).  It writes nnz, and, when the pointers are not NULL, rowptr[dim + 1] and
 * colidx[nnz] (host arrays, 0-based).  nd_jacobian replaces the solver's colored
 * ForwardDiff Jacobian on that prototype: the analytic values at (u, p, t) into
 * values[nnz] (device, element type of the handle), in the pattern's order.  Both take
 * homogeneous and batched handles; the pattern is built on first use (host work and a
 * copy of the structure) and kept by the handle.  nd_jacobian is stream-ordered. */
int nd_jacobian_pattern(nd_handle* h, int64_t* nnz, int32_t* rowptr, int32_t* colidx);
int nd_jacobian(nd_handle* h, int dtype, void* values, const void* u, const void* p, double t, void* stream);

/* Steady state of a network whose outputs have dimension 1 (every kind but the power-grid
 * ones), the counterpart of find_fixpoint(nw, x0, p) (src/initialization.jl:44-144), which
 * solves a SteadyStateProblem with NonlinearSolve: Newton's method with restarted GMRES
 * (Krylov dimension krylov_dim <= 64, default 40; max_restarts cycles, default 20) on the
 * sparse Jacobian of nd_jacobian, and a backtracking line search on max|F|.  u (device,
 * FP64, length dim): x0 in, the steady state out.  Stops at max|du| <= tol.  Writes the
 * Newton iterations and the final max|du| to the host pointers iters / resid.  An RHS
 * with NaN at x0 and a solve that does not reach tol give ND_ERR_NOT_CONVERGED (the
 * reference's NetworkInitError).  FP64 handles; synchronous. */
int nd_find_fixpoint(nd_handle* h, double* u, const double* p, double t, double tol, int max_newton, int krylov_dim,
                     int max_restarts, int32_t* iters, double* resid, void* stream);

/* Result of a solve. */
typedef struct nd_solve_stats {
    int64_t naccept; /* accepted steps                               */
    int64_t nreject; /* rejected steps                               */
    int64_t nf;      /* RHS evaluations                              */
    double t_final;  /* time reached                                 */
    double dt_last;  /* last proposed step size                      */
    int32_t status;  /* ND_OK, ND_ERR_MAXITERS or ND_ERR_NOT_CONVERGED */
    int32_t reserved;
} nd_solve_stats;

/* Integrate du/dt = f(u, p, t) from t0 to t1 with Tsit5 (Tsitouras 2011) and adaptive
 * steps on the GPU: `solve(ODEProblem(nw, u0, (t0, t1), p), Tsit5(); reltol, abstol)`
 * (src/post_utils.jl:43-100; the stepper of OrdinaryDiffEqTsit5).  u (device, FP64, length
 * dim) holds u0 on entry and u(t1) on return; the state, stage vectors, error norm and
 * step control are FP64, the RHS runs in the handle's precision.  Error norm: RMS of
 * err_i / (abstol + reltol max(|u_i|, |u_new_i|)); PI step control.  max_steps <= 0: no
 * limit.  Synchronous: returns when the solve has finished (ordered after `stream`). */
int nd_solve_tsit5(nd_handle* h, double* u, const void* p, double t0, double t1, double reltol, double abstol,
                   int64_t max_steps, nd_solve_stats* stats, void* stream);

/* Rosenbrock23 (Shampine & Reichelt 1997) for M u' = f(u) with a diagonal mass matrix:
 * mass[dim] (device, FP64; NULL = identity), zero entries making states algebraic, as
 * construct_mass_matrix builds it (src/construction.jl:409-467) for components with
 * mass_matrix = 0 (the PQ bus, benchmark/benchmark_models.jl:66-74).  Each step uses the
 * analytic sparse Jacobian (nd_jacobian) and solves its three linear systems with
 * W = M - h d J by Jacobi-preconditioned GMRES.  u: FP64 device state, consistent for the
 * algebraic rows (in: u0, out: u(t1)).  max_steps <= 0 means ND_ENSEMBLE_DEFAULT_MAX_STEPS.
 * FP64 handles only.  Synchronous.  Replaces solve(ODEProblem(nw, u0, tspan, p),
 * Rosenbrock23()) of SciML (src/post_utils.jl:43-100 builds that ODEFunction). */
int nd_solve_rosenbrock23(nd_handle* h, double* u, const double* p, const double* mass, double t0, double t1,
                          double reltol, double abstol, int64_t max_steps, nd_solve_stats* stats, void* stream);

/* Rodas4 (Hairer & Wanner, Solving ODEs II, section VI.4: the first method of RODAS; order
 * 4, L-stable, stiffly accurate, embedded order 3) for M u' = f(u) with a diagonal mass
 * matrix, on the same stage machinery as nd_solve_rosenbrock23: six linear systems per step
 * with W = M - h γ J (γ = 1/4, J from nd_jacobian), each solved by Jacobi-preconditioned
 * GMRES.  Step control h <- h min(6, max(0.2, 0.9 err^(-1/4))) on the scaled RMS norm of
 * the embedded estimate.  Arguments, stats and errors as for nd_solve_rosenbrock23.  FP64
 * handles only.  Synchronous.  Replaces solve(prob, Rodas4()) (the reference's tests solve
 * its heterogeneous and ODE-edge networks with Rodas4 / Rodas5,
 * test/inhomogeneous_test.jl:51, test/diffusion_test.jl:121). */
int nd_solve_rodas4(nd_handle* h, double* u, const double* p, const double* mass, double t0, double t1, double reltol,
                    double abstol, int64_t max_steps, nd_solve_stats* stats, void* stream);

/* Allocation-free RHS.  This entry point has no counterpart in the reference.  It is for
 * callers that must not allocate device memory while they evaluate the RHS: a process
 * whose device memory belongs to a caching allocator (CUDA.jl's or PyTorch's pool), where a
 * library's own cudaMalloc can fail or fragment the pool, or a host program that budgets
 * its device memory once up front.  It calls no cudaMalloc / cudaFree: the caller passes
 * the topology as device arrays, and the edge values go to one file-scope device array of
 * 64 MiB (8 Mi FP64 or 16 Mi FP32 edges) that every GPU loading the library holds until the
 * process exits.
 *   edges  canonical list (sorted by source, src < dst): src[ne], dst[ne] (0-based int32)
 *   src_ptr[nv+1]  first edge of each vertex's source block
 *   dst_ptr[nv+1], dst_eid[ne]  each vertex's destination-side edge ids, ascending
 *   du, u, p  as for nd_rhs, element type `dtype`
 * The arrays must describe a canonical list exactly as nd_create would sort it; they are
 * device arrays and are not checked.  Another order still gives the network's RHS, but its
 * sums run in that order, not the reference's.
 * Result: the same du as nd_rhs on the same network: in FP64 bit for bit; in FP32 bit for
 * bit on every row of fewer than 128 terms (rows longer than 32 with Kahan compensation,
 * as in nd_rhs), within the FP32 rounding on longer rows, which nd_rhs sums a warp per row.
 * ne above the scratch size returns
 * ND_ERR_ARG.  The first call on a device looks up the scratch array's device address
 * (cudaGetSymbolAddress, with that device current) and should come before any stream
 * capture; the lookup is repeated only after the device's context was reset.  All calls
 * share the scratch and it keeps the last call's values: calls that overlap on the GPU
 * (other streams, other host threads) race. */
int nd_rhs_static_scratch(int dtype, int vertex_kind, int edge_kind, int64_t nv, int64_t ne, const int32_t* src,
                          const int32_t* dst, const uint32_t* src_ptr, const uint32_t* dst_ptr,
                          const int32_t* dst_eid, void* du, const void* u, const void* p, void* stream);
/* Device-side checks of the topology arrays that nd_rhs_static_scratch reads (the entry
 * point whose device indices no host code validates; nd_create checks its input on the
 * host).  With checks on (process-wide; default off), its kernels test every index they
 * read from src, dst, src_ptr, dst_ptr and dst_eid before using it, and the list's
 * canonical order (src ascending, src < dst, each source block holding its vertex's
 * edges, each destination list ascending and holding its vertex's edges).  An index out of
 * range is not dereferenced (its term counts as zero).  The first finding is kept on the
 * device; the call then synchronises its stream, reads it back and returns
 * ND_ERR_DEVICE_CHECK, with the array, position and value in nd_last_error().  Nothing
 * traps, and the context stays usable.  A checked call synchronises, so it cannot be
 * captured into a graph. */
int nd_set_device_checks(int on);

/* ---------------------------------------------------------------------------------
 * External inputs and loopback edges.  No library component reads external inputs or is
 * an injector with a feed-forward output, so nd_create rejects networks that use them;
 * a host that keeps its own components calls these two gathers between its component
 * passes, where the reference's core loop makes the same copies.  Every pointer is a
 * device pointer; indices are 0-based and must lie inside the buffers (not checked on
 * the device).  n = 0 launches nothing.  dtype ND_F32 or ND_F64 for all value buffers.
 * ------------------------------------------------------------------------------- */
/* extbuf[k] = from_state[k] ? u[idx[k]] : o[idx[k]] for k < n: the ExtMap gather
 * collect_externals! (src/external_inputs.jl:51-80), one entry per StateBufIdx /
 * OutBufIdx of the map with the index shifted to 0-based. */
int nd_collect_externals(int dtype, int64_t n, const int64_t* idx, const uint8_t* from_state, void* extbuf,
                         const void* u, const void* o, void* stream);
/* aggbuf[agg_idx[k]] = obuf[out_idx[k]] for k < n: apply_loopback! (src/post_utils.jl:230-248)
 * on the map of gen_loopback_map (src/post_utils.jl:213-224), the destination vertex's
 * outputs copied into its source vertex's aggregated inputs.  Repeated agg_idx entries
 * race (the reference's GPU kernel has the same rule). */
int nd_apply_loopback(int dtype, int64_t n, const int64_t* out_idx, const int64_t* agg_idx, void* aggbuf,
                      const void* obuf, void* stream);


/* ---------------------------------------------------------------------------------
 * Ensembles: many instances of one vertex / edge model pair on different graphs (the
 * basin-stability and parameter-sweep workloads).  Instance i has vertices
 * [v_offset[i], v_offset[i+1]) and edges [e_offset[i], e_offset[i+1]) of the packed
 * numbering, its edges given with LOCAL 0-based endpoints in edges(g) order.  The packed
 * u / du / p are the instances' reference layouts one after another (p: instance i's
 * vertex parameters, then its edge parameters).  No counterpart in the reference, where
 * an ensemble is a loop of solve() calls (EnsembleProblem in SciML).
 * ------------------------------------------------------------------------------- */
typedef struct nd_ensemble_desc {
    int64_t n_instances;
    const int64_t* v_offset; /* [n+1] host */
    const int64_t* e_offset; /* [n+1] host */
    const int64_t* src;      /* [e_offset[n]] host, local endpoints */
    const int64_t* dst;
    int32_t vertex_kind, edge_kind, coupling, flags;
} nd_ensemble_desc;

typedef struct nd_ensemble nd_ensemble;

int nd_ensemble_create(const nd_ensemble_desc* desc, int dtype, nd_ensemble** out);
int nd_ensemble_destroy(nd_ensemble* e);
int nd_ensemble_get_info(const nd_ensemble* e, int64_t* dim, int64_t* pdim);

/* du of every instance (each equal to nd_rhs on that instance). */
int nd_ensemble_rhs(nd_ensemble* e, int dtype, void* du, const void* u, const void* p, void* stream);

/* Every instance integrated from t0 to t1 by Tsit5 with its own adaptive steps (FP64
 * state, error norm and control; RHS in the ensemble's precision), in one persistent
 * kernel replayed from a CUDA graph.  u: packed FP64 device state (in: u0, out: u(t1)).
 * status[i] (device int32): ND_OK, ND_ERR_MAXITERS (more than max_steps steps, the
 * per-instance budget; max_steps <= 0 means ND_ENSEMBLE_DEFAULT_MAX_STEPS, the 1e5 of
 * SciML's default maxiters, so that no solve can keep the GPU busy without end) or
 * ND_ERR_NOT_CONVERGED; nsteps[i] (device int64): steps taken.  threads per instance:
 * 64/128/256/512, or 0 for the autotuned / default choice.  Stream-ordered. */
#define ND_ENSEMBLE_DEFAULT_MAX_STEPS 100000
int nd_ensemble_solve_tsit5(nd_ensemble* e, double* u, const void* p, double t0, double t1, double reltol,
                            double abstol, int64_t max_steps, int threads, int32_t* status, int64_t* nsteps,
                            void* stream);

/* nd_ensemble_solve_tsit5 with a snapshot of the step control (no reference counterpart:
 * the reference hands the integrator to OrdinaryDiffEq, whose integrator state is
 * serialised with Julia's Serialization, benchmark/benchmarks.jl:162-167).  control: NULL,
 * or a device array of 3 doubles per instance, (t, dt, qold) = the time reached, the next
 * step size the controller proposed and its error history, written when each instance
 * ends.  resume != 0 starts every instance from the control array's dt and qold (dt
 * clipped to t1 - t0) instead of the initial-step heuristic, so that a long solve can be
 * split at a snapshot time t_s: solve to t_s, save u and control, and later solve from
 * t_s with resume = 1.  Stream-ordered like nd_ensemble_solve_tsit5. */
int nd_ensemble_solve_tsit5_ex(nd_ensemble* e, double* u, const void* p, double t0, double t1, double reltol,
                               double abstol, int64_t max_steps, int threads, int32_t* status, int64_t* nsteps,
                               double* control, int resume, void* stream);

/* Autotuner: times a short solve (t0 .. t0 + t_probe) with each block size on a copy of
 * u and keeps the fastest for threads = 0.  Synchronous. */
int nd_ensemble_autotune(nd_ensemble* e, const double* u, const void* p, double t0, double t_probe, double reltol,
                         double abstol, int* chosen, void* stream);
int nd_ensemble_set_threads(nd_ensemble* e, int threads);

/* Steady states of swing ensembles (the batched find_fixpoint,
 * src/initialization.jl:44-144): Newton's method on the power balance at ω = 0, each
 * step's linear system solved by conjugate gradients on the analytic Jacobian (the
 * graph Laplacian weighted by K cos(θ_n - θ_v)), in the subspace orthogonal to the
 * uniform phase shift.  u (packed FP64, device): initial θ in, steady state out (ω set
 * to 0).  Stops at max |du| <= tol (the reference's residual maximum(abs.(resid))).
 * Device outputs per instance: iters, resid, status (ND_OK / ND_ERR_MAXITERS /
 * ND_ERR_NOT_CONVERGED) and, if not NULL, the CG iterations.  max_cg <= 0: 4 x the
 * largest instance.  FP64 ensembles only.  Stream-ordered. */
int nd_ensemble_fixpoint(nd_ensemble* e, double* u, const double* p, double tol, int max_newton, int max_cg,
                         int32_t* iters, double* resid, int32_t* status, int32_t* cg_iters, void* stream);

/* ---------------------------------------------------------------------------------
 * Learned warm start (no reference counterpart: find_fixpoint, src/initialization.jl:44-144,
 * starts Newton from the guess its caller passes; a prediction of this network is such a
 * guess).  A message-passing network on one fixed graph maps per-instance vertex power
 * injections P [batch][nv] and line weights K [batch][ne] (edges in the given order) to
 * steady-state phases θ [batch][nv], centred per instance; the steady-state frequencies
 * of swing vertices are 0.  FP32 throughout, hidden width 64, `layers` residual
 * message-passing layers.  Parameters, gradients and Adam moments live on the device;
 * every pointer below is a device pointer (params copies accept host pointers too).
 * ------------------------------------------------------------------------------- */
typedef struct nd_mpnn nd_mpnn;

/* Seeded Glorot-uniform initialisation.  hidden must be 64, layers 1..16. */
int nd_mpnn_create(int64_t nv, int64_t ne, const int64_t* src, const int64_t* dst, int layers, int hidden,
                   uint64_t seed, nd_mpnn** out);
int nd_mpnn_destroy(nd_mpnn* m);
int nd_mpnn_num_params(const nd_mpnn* m, int64_t* n);
int nd_mpnn_get_params(const nd_mpnn* m, float* dst, void* stream);
int nd_mpnn_set_params(nd_mpnn* m, const float* src, void* stream);
int nd_mpnn_get_grads(const nd_mpnn* m, float* dst, void* stream);
/* θ = network(P, K) for `batch` instances. */
int nd_mpnn_forward(nd_mpnn* m, int64_t batch, const float* P, const float* K, float* theta, void* stream);
/* Mean squared error of the centred prediction against the centred θ*; writes the loss
 * (device float) and the gradient of every parameter (read by nd_mpnn_get_grads). */
int nd_mpnn_loss_grad(nd_mpnn* m, int64_t batch, const float* P, const float* K, const float* theta_star,
                      float* loss, void* stream);
/* One Adam step on the last gradients (bias-corrected moments). */
int nd_mpnn_adam(nd_mpnn* m, double lr, double beta1, double beta2, double eps, void* stream);
int nd_mpnn_reset_optimizer(nd_mpnn* m, void* stream);
/* Weighted-mean steps per message (default 1): each layer's message is M^hops h, so the
 * receptive field is layers x hops vertices deep. */
int nd_mpnn_set_hops(nd_mpnn* m, int hops);

#ifdef __cplusplus
}
#endif
#endif /* ND_GB300_H */
