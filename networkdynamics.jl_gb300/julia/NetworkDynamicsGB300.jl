"""
    NetworkDynamicsGB300

Julia side of the GB300 network right-hand side: an `ExecutionStyle` / aggregator pair
that NetworkDynamics.jl's `Network` constructor accepts like its own
(`execution=GB300Execution(), aggregator=GB300Aggregator(+)`), and whose RHS `ccall`s
`libnd_b200.so` (C ABI in `include/nd_gb300.h`).

Plug points used (paths relative to the NetworkDynamics.jl source tree):
- `ExecutionStyle{buffered}` (src/executionstyles.jl:13): `GB300Execution <: ExecutionStyle{false}`;
- the curried aggregator constructor called as `aggregator(im, edgebatches)`
  (src/construction.jl:198) and `get_aggr_constructor` (src/aggregators.jl:287-292);
- `Adapt.adapt_structure(CuArray{T}, nw)` (ext/NetworkDynamicsCUDAExt.jl:16-45), which adapts
  `nw.layer` field by field and so reaches `Adapt.adapt_structure(to, ::GB300Aggregator)`;
- `iscudacompatible` (src/executionstyles.jl:50-52, src/aggregators.jl:294-295).

Only the hand-written component library runs on this path; any other component function
raises an `ArgumentError` when the aggregator is built.  There is no CPU fallback.

Heterogeneous networks (several vertex / edge batches), ODE edges and the Symmetric /
Directed / Fiducial outputs go through `nd_create_batched`: the shim hands over the
reference's own batches (the edge batches the aggregator constructor receives, and the
vertex batches `_find_identical_components` forms, both in order of first appearance),
so the device handle uses exactly the layout of `u` and `p` the `Network` defines.
"""
module NetworkDynamicsGB300

using NetworkDynamics: NetworkDynamics, Network, ExecutionStyle, AntiSymmetric, Symmetric, Directed, Fiducial,
                       executionstyle
using CUDA: CUDA, CuArray, CuPtr
using Adapt: Adapt
using SparseArrays: SparseArrays

export GB300Execution, GB300Aggregator, register_gb300_vertex!, register_gb300_edge!

const libnd = get(ENV, "ND_GB300_LIB", joinpath(@__DIR__, "..", "nd_gb300", "lib", "libnd_b200.so"))

# status codes and enums of include/nd_gb300.h
const ND_OK = Cint(0)
const ND_ERR_ARG = Cint(-1)
const ND_ERR_UNSUPPORTED_COMPONENT = Cint(-2)
const ND_ERR_DTYPE = Cint(-3)
const ND_F32 = Cint(1)
const ND_F64 = Cint(2)
const ND_ANTISYMMETRIC = Cint(1)
const ND_SYMMETRIC = Cint(2)
const ND_DIRECTED = Cint(3)
const ND_FIDUCIAL = Cint(4)

struct nd_batch
    kind::Int32
    coupling::Int32
end

struct nd_batched_network_desc
    nv::Int64
    ne::Int64
    src::Ptr{Int64}
    dst::Ptr{Int64}
    n_vertex_batches::Int32
    n_edge_batches::Int32
    vertex_batches::Ptr{nd_batch}
    edge_batches::Ptr{nd_batch}
    vertex_batch::Ptr{Int32}
    edge_batch::Ptr{Int32}
    flags::Int32
    reserved::Int32
    vertex_constants::Ptr{Cdouble}  # values a component closes over (C_NULL: none)
end

"""
    GB300Execution(; sum_order=:sequential, layout=:auto)

Unbuffered execution style whose RHS is one call into libnd_b200.so.  The options are type
parameters, because a Network rebuilds its style from its type (`executionstyle(nw) = EX()`,
src/network_structure.jl:83-116):

- `sum_order`: `:sequential` (SequentialAggregator's bits), `:sequential_hw` (the same bits,
  hardware adds at hubs) or `:tree` (deterministic warp tree at hubs, not bitwise);
- `layout`: `:auto` (two-phase kernels for canonical edge lists) or `:fused`.

They are applied to the device handle at adapt time.
"""
struct GB300Execution{O,L} <: ExecutionStyle{false} end
function GB300Execution(; sum_order::Symbol=:sequential, layout::Symbol=:auto)
    sum_order in (:sequential, :sequential_hw, :tree) || throw(ArgumentError("unknown sum_order $sum_order"))
    layout in (:auto, :fused) || throw(ArgumentError("unknown layout $layout"))
    GB300Execution{sum_order,layout}()
end
const ND_ORDER_CODES = Dict(:sequential => Cint(0), :tree => Cint(1), :sequential_hw => Cint(2))
const ND_LAYOUT_CODES = Dict(:auto => Cint(0), :fused => Cint(1))

# Known component functions -> library kinds (nd_vertex_kind / nd_edge_kind).  Models
# built from the component library register their functions here: vertex f, the
# single-sided g inside an AntiSymmetric / Symmetric / Directed wrapper, the f of an ODE
# edge, or a two-sided g (diffusionedge_fid!, registered with register_gb300_edge!(g, 1)).
const VERTEX_KINDS = IdDict{Any,Cint}()
const EDGE_KINDS = IdDict{Any,Cint}()
register_gb300_vertex!(f, kind::Integer) = (VERTEX_KINDS[f] = Cint(kind); f)
register_gb300_edge!(g, kind::Integer) = (EDGE_KINDS[g] = Cint(kind); g)

mutable struct GB300Aggregator{F}
    f::F
    nv::Int
    src::Vector{Int64}                # 0-based, edges(g) order
    dst::Vector{Int64}
    vertex_batches::Vector{nd_batch}  # in the reference's batch order
    edge_batches::Vector{nd_batch}
    vertex_batch::Vector{Int32}       # batch of every vertex / edge (0-based)
    edge_batch::Vector{Int32}
    handle::Ptr{Cvoid}                # C_NULL until adapted to the device
    dtype::Cint
end

"""
    GB300Aggregator(+)

Curried like every NetworkDynamics aggregator: returns the `(im, batches)` constructor the
`Network` calls with its index layout.  Only `+` is supported (as for SparseAggregator).
"""
function GB300Aggregator(f)
    f === (+) || throw(ArgumentError("GB300Aggregator only works with + as reducer."))
    (im, batches) -> GB300Aggregator(im, batches, f)
end

unsupported(what) = throw(ArgumentError("$what is not in the GB300 component library; \
                                         GB300Execution has no CPU fallback"))

function edge_batch_kind(batch)
    g = batch.compg
    if g isa Fiducial        # ODE edges: StateMask outputs, the kind is the edge's f
        return nd_batch(get(() -> unsupported("edge function $(batch.compf)"), EDGE_KINDS, batch.compf), ND_FIDUCIAL)
    end
    for (W, c) in ((AntiSymmetric, ND_ANTISYMMETRIC), (Symmetric, ND_SYMMETRIC), (Directed, ND_DIRECTED))
        g isa W && return nd_batch(get(() -> unsupported("edge function $(g.g)"), EDGE_KINDS, g.g), c)
    end
    nd_batch(get(() -> unsupported("edge function $g"), EDGE_KINDS, g), ND_FIDUCIAL)  # two-sided g
end

function GB300Aggregator(im, batches, f)
    # External inputs (the ExtMap gather, src/external_inputs.jl:51-80) and loopback edges
    # (the injector copy, src/post_utils.jl:213-248) are rejected by name, before any
    # component lookup: no library component reads external inputs or is an injector.
    NetworkDynamics.has_external_input(im) &&
        throw(ArgumentError("GB300Execution supports networks without external inputs only"))
    any(NetworkDynamics.is_loopback, im.edgem) &&
        throw(ArgumentError("GB300Execution supports networks without LoopbackConnection edges only"))
    # vertex batches exactly as the Network formed them (src/construction.jl:155-160)
    vidxs = NetworkDynamics._find_identical_components(im.vertexm)
    vbatches = map(vidxs) do idxs
        vf = im.vertexm[first(idxs)].f
        nd_batch(get(() -> unsupported("vertex function $vf"), VERTEX_KINDS, vf), 0)
    end
    vbatch = zeros(Int32, length(im.v_data))
    for (b, idxs) in enumerate(vidxs), i in idxs
        vbatch[i] = b - 1
    end
    ebatches = nd_batch[edge_batch_kind(batch) for batch in batches]
    ebatch = zeros(Int32, length(im.edgevec))
    for (b, batch) in enumerate(batches), i in batch.indices
        ebatch[i] = b - 1
    end
    src = Int64[e.src - 1 for e in im.edgevec]
    dst = Int64[e.dst - 1 for e in im.edgevec]
    GB300Aggregator{typeof(f)}(f, length(im.v_data), src, dst, collect(vbatches), ebatches, vbatch, ebatch,
                               C_NULL, Cint(0))
end

NetworkDynamics.get_aggr_constructor(a::GB300Aggregator) = GB300Aggregator(a.f)
NetworkDynamics.iscudacompatible(::GB300Execution) = true
NetworkDynamics.iscudacompatible(::Type{<:GB300Execution}) = true
NetworkDynamics.iscudacompatible(::GB300Aggregator) = true

last_error() = unsafe_string(ccall((:nd_last_error, libnd), Cstring, ()))

function check(code::Cint)
    code == ND_OK && return nothing
    msg = last_error()
    code in (ND_ERR_ARG, ND_ERR_DTYPE, ND_ERR_UNSUPPORTED_COMPONENT) && throw(ArgumentError(msg))
    error("libnd_b200: [$code] $msg")
end

# adapt(CuArray{T}, nw) reaches the aggregator through @adapt_structure NetworkLayer: build
# the device handle for element type T (the reference's cache typing at adapt time).
function Adapt.adapt_structure(::Type{<:CuArray{T}}, a::GB300Aggregator) where {T<:Union{Float32,Float64}}
    dtype = T === Float64 ? ND_F64 : ND_F32
    out = GB300Aggregator{typeof(a.f)}(a.f, a.nv, a.src, a.dst, a.vertex_batches, a.edge_batches, a.vertex_batch,
                                       a.edge_batch, C_NULL, dtype)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve a begin
        desc = nd_batched_network_desc(a.nv, length(a.src), pointer(a.src), pointer(a.dst),
                                       length(a.vertex_batches), length(a.edge_batches), pointer(a.vertex_batches),
                                       pointer(a.edge_batches), pointer(a.vertex_batch), pointer(a.edge_batch), 0, 0,
                                       C_NULL)
        check(ccall((:nd_create_batched, libnd), Cint, (Ref{nd_batched_network_desc}, Cint, Ref{Ptr{Cvoid}}),
                    desc, dtype, h))
    end
    out.handle = h[]
    finalizer(x -> x.handle == C_NULL || ccall((:nd_destroy, libnd), Cint, (Ptr{Cvoid},), x.handle), out)
    out
end

# The execution style's options on the handle (host-side settings, no device work).
function configure!(a::GB300Aggregator, ::GB300Execution{O,L}) where {O,L}
    check(ccall((:nd_set_sum_order, libnd), Cint, (Ptr{Cvoid}, Cint), a.handle, ND_ORDER_CODES[O]))
    check(ccall((:nd_set_layout, libnd), Cint, (Ptr{Cvoid}, Cint), a.handle, ND_LAYOUT_CODES[L]))
end

# The RHS: one stream-ordered call on CUDA.jl's task-local stream.
function (nw::Network{<:GB300Execution})(du::CuArray{T}, u::CuArray{T}, p, t) where {T}
    a = nw.layer.aggregator
    a.handle == C_NULL && throw(ArgumentError("adapt the network with adapt(CuArray{$T}, nw) first"))
    configure!(a, NetworkDynamics.executionstyle(nw))
    dtype = T === Float64 ? ND_F64 : T === Float32 ? ND_F32 : Cint(0)
    pp, np = p === nothing || isempty(p) ? (CuPtr{T}(0), 0) : (pointer(p), length(p))
    check(ccall((:nd_rhs, libnd), Cint,
                (Ptr{Cvoid}, Cint, CuPtr{T}, Int64, CuPtr{T}, Int64, CuPtr{T}, Int64, Cdouble, Ptr{Cvoid}),
                a.handle, dtype, pointer(du), length(du), pointer(u), length(u), pp, np, Float64(t),
                CUDA.stream().handle))
    nothing
end

# Sparsity pattern of ∂f/∂u, the method get_jac_prototype takes for GB300 networks
# (ext/NetworkDynamicsSparsityExt.jl:57-127 traces the RHS instead): the structural pattern
# of the library components from nd_jacobian_pattern, as the SparseMatrixCSC that
# set_jac_prototype! stores.
function NetworkDynamics.get_jac_prototype(nw::Network{<:GB300Execution}; kwargs...)
    a = nw.layer.aggregator
    a.handle == C_NULL && throw(ArgumentError("adapt the network with adapt(CuArray{T}, nw) first"))
    nnz = Ref{Int64}(0)
    check(ccall((:nd_jacobian_pattern, libnd), Cint, (Ptr{Cvoid}, Ref{Int64}, Ptr{Int32}, Ptr{Int32}),
                a.handle, nnz, C_NULL, C_NULL))
    n = NetworkDynamics.dim(nw)
    rowptr = Vector{Int32}(undef, n + 1)
    colidx = Vector{Int32}(undef, nnz[])
    check(ccall((:nd_jacobian_pattern, libnd), Cint, (Ptr{Cvoid}, Ref{Int64}, Ptr{Int32}, Ptr{Int32}),
                a.handle, nnz, rowptr, colidx))
    rows = Int[]
    for i in 1:n, _ in (rowptr[i] + 1):rowptr[i + 1]
        push!(rows, i)
    end
    SparseArrays.sparse(rows, Int.(colidx) .+ 1, trues(length(colidx)), n, n)
end

# find_fixpoint(nw, x0, p) for GB300 networks: Newton-GMRES on the device (nd_find_fixpoint)
# instead of a SteadyStateProblem on the host (src/initialization.jl:44-144).
function NetworkDynamics.find_fixpoint(nw::Network{<:GB300Execution}, x0::CuArray{Float64}, p::CuArray{Float64};
                                       t=NaN, tol=1e-10, maxiters=50, kwargs...)
    a = nw.layer.aggregator
    u = copy(x0)
    iters = Ref{Int32}(0)
    resid = Ref{Float64}(NaN)
    code = ccall((:nd_find_fixpoint, libnd), Cint,
                 (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Cdouble, Cdouble, Cint, Cint, Cint, Ref{Int32},
                  Ref{Float64}, Ptr{Cvoid}),
                 a.handle, pointer(u), pointer(p), Float64(t), tol, maxiters, 0, 0, iters, resid,
                 CUDA.stream().handle)
    code == Cint(-8) && throw(NetworkDynamics.NetworkInitError(last_error()))
    check(code)
    u
end

end # module
