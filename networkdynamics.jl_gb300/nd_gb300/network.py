"""Network construction and the GB300 right-hand side.

Python mirror of the reference's plug points (src/executionstyles.jl:13,
src/aggregators.jl:16-27, src/construction.jl:31-236): ``Network(g, vertexm, edgem;
execution=GB300Execution(), aggregator=GB300Aggregator(+))`` builds the flat layout, and
``adapt(nw, torch.float64)`` (the counterpart of ``adapt(CuArray{Float64}, nw)``,
ext/NetworkDynamicsCUDAExt.jl:16-45) creates the device handle in libnd_b200.so.  Calling
``nw(du, u, p, t)`` evaluates the RHS on the GPU through the C ABI.
"""
from __future__ import annotations

import ctypes as C
import operator
from typing import Sequence, Union

import numpy as np

from . import _capi as capi
from .components import EdgeModel, VertexModel
from .graphs import Graph


class ExecutionStyle:
    """Abstract execution style (src/executionstyles.jl:13)."""

    buffered = False


class GB300Execution(ExecutionStyle):
    """The RHS on one GB300 GPU.  Unbuffered: edges read vertex outputs straight from u
    (the lazy gather of src/gbufs.jl:37-65, done in registers).

    Keyword options, applied to the device handle when the network is adapted (the
    reference configures its execution styles by keyword and type parameter,
    src/executionstyles.jl:13-52):

    - ``sum_order``: "sequential" (default; the bits of SequentialAggregator, with the exact
      scan at hubs), "sequential_hw" (the same bits with hardware adds at hubs) or "tree"
      (a deterministic warp tree at hubs; not bitwise);
    - ``layout``: "auto" (two-phase edge-centric kernels for canonical edge lists, else the
      fused kernel) or "fused";
    - ``kernel_timing``: bracket every kernel with CUDA events for ``Network.kernel_times``.

    The precision is the dtype given to ``adapt``.  The degree buckets (light rows up to 32,
    heavy rows above 2048) and the FP32 Kahan threshold (rows longer than 32) are
    compile-time constants of the kernels."""

    buffered = False
    SUM_ORDERS = ("sequential", "sequential_hw", "tree")
    LAYOUTS = ("auto", "fused")

    def __init__(self, sum_order: str = "sequential", layout: str = "auto", kernel_timing: bool = False):
        if sum_order not in self.SUM_ORDERS:
            raise capi.ArgumentError(capi.ND_ERR_ARG, f"unknown sum_order {sum_order!r}: one of {self.SUM_ORDERS}")
        if layout not in self.LAYOUTS:
            raise capi.ArgumentError(capi.ND_ERR_ARG, f"unknown layout {layout!r}: one of {self.LAYOUTS}")
        self.sum_order = sum_order
        self.layout = layout
        self.kernel_timing = bool(kernel_timing)

    def __eq__(self, other):
        return isinstance(other, GB300Execution) and (self.sum_order, self.layout, self.kernel_timing) == (
            other.sum_order, other.layout, other.kernel_timing)

    def __hash__(self):
        return hash((self.sum_order, self.layout, self.kernel_timing))

    def __repr__(self):
        opts = [f"{k}={v!r}" for k, v, d in (("sum_order", self.sum_order, "sequential"),
                                             ("layout", self.layout, "auto"),
                                             ("kernel_timing", self.kernel_timing, False)) if v != d]
        return f"GB300Execution({', '.join(opts)})"


def iscudacompatible(x) -> bool:
    return isinstance(x, (GB300Execution, GB300Aggregator))


class GB300Aggregator:
    """Deterministic destination-sorted aggregation.  Like every reference aggregator,
    ``GB300Aggregator(+)`` is curried: it returns a constructor that the Network calls
    with its index layout (src/construction.jl:198).  Only ``+`` is supported, as for
    SparseAggregator (src/aggregators.jl:247-250)."""

    def __init__(self, f=operator.add):
        if f not in (operator.add, "+", sum):
            raise capi.ArgumentError(capi.ND_ERR_ARG, "GB300Aggregator only works with + as reducer.")
        self.f = operator.add

    def __repr__(self):
        return "GB300Aggregator(+)"


def get_aggr_constructor(agg: GB300Aggregator) -> GB300Aggregator:
    """src/aggregators.jl:287-292."""
    return GB300Aggregator(agg.f)


_TORCH_DT = None


def _dtype_code(dtype) -> int:
    import torch
    if dtype in (torch.float64, np.float64, "float64", "f64"):
        return capi.ND_F64
    if dtype in (torch.float32, np.float32, "float32", "f32"):
        return capi.ND_F32
    raise capi.ArgumentError(capi.ND_ERR_DTYPE,
                             f"Use adapt on Network with either float32 or float64, got {dtype}")


def _check_library(models, what):
    bad = next((m for m in models if m.kind is None), None)
    if bad is not None:
        raise capi.UnsupportedComponentError(
            capi.ND_ERR_UNSUPPORTED_COMPONENT,
            f"{what} model {bad.name!r} is not in the GB300 component library; "
            "GB300Execution has no CPU fallback")


def _check_no_external_inputs(vms, ems):
    """Networks with external inputs (the ExtMap gather of src/external_inputs.jl:51-80) or
    loopback edges (the injector copy of src/post_utils.jl:213-248, applied at
    src/coreloop.jl:47) are rejected by name: no library component reads external inputs or
    has a feed-forward output, so neither map can be built for a GB300 network."""
    bad = next((m for m in list(vms) + list(ems) if m.extin), None)
    if bad is not None:
        raise capi.ArgumentError(capi.ND_ERR_ARG,
                                 f"{bad.name!r} has external inputs; GB300Execution supports networks without "
                                 "external inputs only (no library component reads them)")
    bad = next((m for m in ems if m.loopback), None)
    if bad is not None:
        raise capi.ArgumentError(capi.ND_ERR_ARG,
                                 f"{bad.name!r} is a LoopbackConnection; GB300Execution supports networks without "
                                 "loopback edges only (no library vertex is an injector with a feed-forward output)")


def _mm_key(mm):
    """A hashable form of a component's mass matrix (components with different mass
    matrices are different components, in batches of their own)."""
    if mm is None:
        return None
    a = np.asarray(mm, dtype=np.float64)
    return (a.shape, tuple(a.ravel().tolist()))


def _batches(models, key):
    """Batches of identical components in order of first appearance, as find_identical
    groups them (src/utils.jl:197-216, src/construction.jl:155-168): the model of every
    batch and the batch index of every component."""
    index, reps = {}, []
    ids = np.empty(len(models), dtype=np.int32)
    for i, m in enumerate(models):
        k = key(m)
        b = index.get(k)
        if b is None:
            b = index[k] = len(reps)
            reps.append(m)
        ids[i] = b
    if len(reps) > capi.ND_MAX_BATCHES:
        raise capi.UnsupportedComponentError(capi.ND_ERR_UNSUPPORTED_COMPONENT,
                                             f"more than {capi.ND_MAX_BATCHES} different components")
    return reps, ids


class Network:
    """A network of library components on a graph, in the reference's flat layout
    (src/network_structure.jl:224-258): u = [vertex states batch by batch, edge states
    batch by batch], p = [vertex parameters batch by batch, edge parameters batch by
    batch]; components are batched by identity in order of first appearance, ascending
    index inside a batch.  With one vertex and one edge model that is vertex order and
    edges(g) order."""

    def __init__(self, g: Graph, vertexm: Union[VertexModel, Sequence[VertexModel]],
                 edgem: Union[EdgeModel, Sequence[EdgeModel]], execution: ExecutionStyle = None,
                 aggregator: GB300Aggregator = None, dtype=None):
        execution = GB300Execution() if execution is None else execution
        aggregator = GB300Aggregator() if aggregator is None else aggregator
        if not isinstance(execution, GB300Execution):
            raise capi.ArgumentError(capi.ND_ERR_ARG, f"Execution type {execution} not supported by this package")
        if not isinstance(aggregator, GB300Aggregator):
            raise capi.ArgumentError(capi.ND_ERR_ARG, f"Aggregator {aggregator} not supported by this package")
        vms = [vertexm] if isinstance(vertexm, VertexModel) else list(vertexm)
        ems = [edgem] if isinstance(edgem, EdgeModel) else list(edgem)
        if (not isinstance(vertexm, VertexModel) and len(vms) != g.nv) or \
                (not isinstance(edgem, EdgeModel) and len(ems) != g.ne):
            raise capi.ArgumentError(capi.ND_ERR_ARG, "one vertex model per vertex and one edge model per edge")
        if not ems:
            raise capi.ArgumentError(capi.ND_ERR_ARG,
                                     "a graph without edges needs the edge model passed as a single EdgeModel")
        _check_no_external_inputs(vms, ems)
        _check_library(vms, "vertex")
        _check_library(ems, "edge")
        # src/construction.jl:98-106
        if len({m.outdim for m in vms}) != 1:
            raise capi.ArgumentError(capi.ND_ERR_ARG, "All vertex models must have the same output dimension!")
        if len({m.outdim for m in ems}) != 1:
            raise capi.ArgumentError(capi.ND_ERR_ARG, "All edge models must have the same output dimension!")
        for m in ems:
            if m.coupling not in capi.COUPLINGS:
                raise capi.UnsupportedComponentError(capi.ND_ERR_UNSUPPORTED_COMPONENT,
                                                     f"unknown edge output wrapper {m.coupling!r}")
        self.graph = g
        if isinstance(vertexm, VertexModel):
            self.vertex_batches, self.vertex_batch = [vertexm], np.zeros(g.nv, dtype=np.int32)
        else:
            self.vertex_batches, self.vertex_batch = _batches(vms, lambda m: (m.kind, m.constants,
                                                                              _mm_key(m.mass_matrix)))
        if isinstance(edgem, EdgeModel):
            self.edge_batches, self.edge_batch = [edgem], np.zeros(g.ne, dtype=np.int32)
        else:
            self.edge_batches, self.edge_batch = _batches(ems, lambda m: (m.kind, m.coupling, _mm_key(m.mass_matrix)))
        # the single model of a one-batch network (None when there are several)
        self.vertexm = self.vertex_batches[0] if len(self.vertex_batches) == 1 else None
        self.edgem = self.edge_batches[0] if len(self.edge_batches) == 1 else None
        self.execution = execution
        self.aggregator = aggregator
        self._layout()
        self._handle = None
        self._dtype = None
        if dtype is not None:
            self._create(dtype)

    def _layout(self):
        """First state / parameter index of every component (register_vertices! /
        register_edges!, src/network_structure.jl:224-258)."""
        def place(batch, models, attr, start):
            order = np.argsort(batch, kind="stable")
            size = np.array([getattr(m, attr) for m in models], dtype=np.int64)[batch[order]]
            first = np.empty(len(batch), dtype=np.int64)
            first[order] = start + np.cumsum(size) - size
            return first, start + int(size.sum())
        self.v_data, nstate = place(self.vertex_batch, self.vertex_batches, "dim", 0)
        self.e_data, self.dim = place(self.edge_batch, self.edge_batches, "dim", nstate)
        self.v_para, npar = place(self.vertex_batch, self.vertex_batches, "pdim", 0)
        self.e_para, self.pdim = place(self.edge_batch, self.edge_batches, "pdim", npar)

    # --- layout helpers -------------------------------------------------------------------
    @property
    def nv(self) -> int:
        return self.graph.nv

    @property
    def ne(self) -> int:
        return self.graph.ne

    @property
    def homogeneous(self) -> bool:
        return len(self.vertex_batches) == 1 and len(self.edge_batches) == 1

    def vertex_state_index(self, v: int, k: int = 0) -> int:
        return int(self.v_data[v]) + k

    def edge_state_index(self, e: int, k: int = 0) -> int:
        return int(self.e_data[e]) + k

    def vertex_param_index(self, v: int, k: int = 0) -> int:
        return int(self.v_para[v]) + k

    def edge_param_index(self, e: int, k: int = 0) -> int:
        return int(self.e_para[e]) + k

    def pflat(self, vertex: dict | None = None, edge: dict | None = None) -> np.ndarray:
        """Flat parameter vector from per-symbol values (defaults where omitted).  A value
        is a scalar or an array over all vertices (edges), read at the components that
        have the symbol."""
        p = np.zeros(self.pdim, dtype=np.float64)
        for models, batch, first, given, what in (
                (self.vertex_batches, self.vertex_batch, self.v_para, vertex or {}, "vertex"),
                (self.edge_batches, self.edge_batch, self.e_para, edge or {}, "edge")):
            for b, m in enumerate(models):
                idx = np.flatnonzero(batch == b)
                for k, name in enumerate(m.psym):
                    val = given.get(name, m.pdef[k] if k < len(m.pdef) else None)
                    if val is None:
                        raise capi.ArgumentError(capi.ND_ERR_ARG, f"{what} parameter {name} has no default")
                    val = np.asarray(val, dtype=np.float64)
                    p[first[idx] + k] = val if val.ndim == 0 else val[idx]
        return p

    def mass_matrix(self):
        """The network's mass matrix as construct_mass_matrix builds it
        (src/construction.jl:409-467): None when every component has the identity (the
        reference's `I`), else its diagonal over the flat state vector, each component's own
        diagonal placed at its state range (v_data / e_data).  A component's mass matrix is a
        scalar for all its states or one entry per state; full matrices are not supported."""
        if all(m.mass_matrix is None for m in list(self.vertex_batches) + list(self.edge_batches)):
            return None
        diag = np.ones(self.dim)
        for models, batch, first in ((self.vertex_batches, self.vertex_batch, self.v_data),
                                     (self.edge_batches, self.edge_batch, self.e_data)):
            for b, m in enumerate(models):
                if m.mass_matrix is None or m.dim == 0:
                    continue
                mm = np.asarray(m.mass_matrix, dtype=np.float64)
                if mm.ndim > 1 or (mm.ndim == 1 and mm.shape[0] != m.dim):
                    raise capi.ArgumentError(capi.ND_ERR_ARG,
                                             f"Mass matrix must be a scalar or one entry per state (a diagonal); "
                                             f"got shape {mm.shape} in component :{m.name}.")
                idx = np.flatnonzero(batch == b)
                diag[first[idx][:, None] + np.arange(m.dim)] = np.broadcast_to(mm, (m.dim,))
        return diag

    # --- device handle -------------------------------------------------------------------
    def _create(self, dtype):
        code = _dtype_code(dtype)
        lib = capi.load()
        g = self.graph
        src = np.ascontiguousarray(g.src, dtype=np.int64)
        dst = np.ascontiguousarray(g.dst, dtype=np.int64)
        P = C.POINTER(C.c_int64)
        h = C.c_void_p()
        if self.homogeneous and not self.vertex_batches[0].constants:
            vm, em = self.vertex_batches[0], self.edge_batches[0]
            desc = capi.nd_network_desc(g.nv, g.ne, src.ctypes.data_as(P), dst.ctypes.data_as(P), vm.kind, em.kind,
                                        capi.COUPLINGS[em.coupling], 0)
            capi.check(lib.nd_create(C.byref(desc), code, C.byref(h)))
        else:
            vb = (capi.nd_batch * len(self.vertex_batches))(*[(m.kind, 0) for m in self.vertex_batches])
            eb = (capi.nd_batch * len(self.edge_batches))(
                *[(m.kind, capi.COUPLINGS[m.coupling]) for m in self.edge_batches])
            vbi = np.ascontiguousarray(self.vertex_batch, dtype=np.int32)
            ebi = np.ascontiguousarray(self.edge_batch, dtype=np.int32)
            P32 = C.POINTER(C.c_int32)
            nc = capi.ND_BATCH_CONSTANTS
            consts = np.zeros((len(self.vertex_batches), nc), dtype=np.float64)
            for b, m in enumerate(self.vertex_batches):
                consts[b, :len(m.constants)] = m.constants
            desc = capi.nd_batched_network_desc(g.nv, g.ne, src.ctypes.data_as(P), dst.ctypes.data_as(P),
                                                len(self.vertex_batches), len(self.edge_batches), vb, eb,
                                                vbi.ctypes.data_as(P32), ebi.ctypes.data_as(P32), 0, 0,
                                                consts.ctypes.data_as(C.POINTER(C.c_double)))
            capi.check(lib.nd_create_batched(C.byref(desc), code, C.byref(h)))
        self._handle = h
        self._dtype = code
        self._lib = lib

    @property
    def handle(self):
        if self._handle is None:
            raise capi.ArgumentError(capi.ND_ERR_ARG, "network is not adapted to the GPU: use adapt(nw, dtype)")
        return self._handle

    def info(self) -> capi.nd_info:
        out = capi.nd_info()
        capi.check(capi.load().nd_get_info(self.handle, C.byref(out)))
        return out

    def set_sum_order(self, order: str) -> None:
        code = {"sequential": capi.ND_ORDER_SEQUENTIAL, "tree": capi.ND_ORDER_TREE,
                "sequential_hw": capi.ND_ORDER_SEQUENTIAL_HW}[order]
        capi.check(capi.load().nd_set_sum_order(self.handle, code))

    def set_layout(self, layout: str) -> None:
        """'auto' (two-phase edge-centric kernels for canonical edge lists) or 'fused'."""
        code = {"auto": 0, "fused": 1}[layout]
        capi.check(capi.load().nd_set_layout(self.handle, code))

    def set_kernel_timing(self, on: bool) -> None:
        """Bracket every kernel that the RHS launches with CUDA events (off by default)."""
        capi.check(capi.load().nd_set_kernel_timing(self.handle, int(bool(on))))

    def kernel_times(self) -> dict:
        """{kind: (launches, total ms)} since the last read (waits for recorded events)."""
        n = len(capi.KERNEL_KINDS)
        launches = (C.c_int64 * n)()
        ms = (C.c_double * n)()
        capi.check(capi.load().nd_kernel_times(self.handle, launches, ms, n))
        return {k: (int(launches[i]), float(ms[i])) for i, k in enumerate(capi.KERNEL_KINDS)}

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and getattr(self, "_lib", None) is not None:
            try:
                self._lib.nd_destroy(h)
            except Exception:
                pass
            self._handle = None

    # --- the RHS ---------------------------------------------------------------------------
    def __call__(self, du, u, p, t=float("nan"), stream=None):
        """du = f(u, p, t) on the GPU.  du, u, p are contiguous CUDA tensors of the adapted
        dtype; the call is ordered on `stream` (default: torch's current stream)."""
        import torch
        for name, x in (("du", du), ("u", u)):
            if not (isinstance(x, torch.Tensor) and x.is_cuda and x.is_contiguous()):
                raise capi.ArgumentError(capi.ND_ERR_ARG, f"{name} must be a contiguous CUDA tensor")
        code = _dtype_code(u.dtype)
        if _dtype_code(du.dtype) != code:
            raise capi.ArgumentError(capi.ND_ERR_DTYPE, "du and u have different element types")
        if p is None or (hasattr(p, "numel") and p.numel() == 0):
            p_ptr, n_p = None, 0
        else:
            if not (isinstance(p, torch.Tensor) and p.is_cuda and p.is_contiguous()):
                raise capi.ArgumentError(capi.ND_ERR_ARG, "p must be a contiguous CUDA tensor")
            if _dtype_code(p.dtype) != code:
                raise capi.ArgumentError(capi.ND_ERR_DTYPE, "p has a different element type than u")
            p_ptr, n_p = p.data_ptr(), p.numel()
        s = stream if stream is not None else torch.cuda.current_stream()
        capi.check(self._lib.nd_rhs(self.handle, code, du.data_ptr(), du.numel(), u.data_ptr(), u.numel(),
                                    p_ptr, n_p, float(t), C.c_void_p(s.cuda_stream)))
        return None


def jvp(nw: Network, jv, u, p, v, t=0.0, stream=None):
    """jv = (∂f/∂u)(u, p, t) · v with the analytic library derivatives (CUDA tensors)."""
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    capi.check(nw._lib.nd_jvp(nw.handle, _dtype_code(u.dtype), jv.data_ptr(), u.data_ptr(),
                              p.data_ptr() if p is not None else None, v.data_ptr(), float(t),
                              C.c_void_p(s.cuda_stream)))


def jacobian_pattern(nw: Network):
    """CSR sparsity pattern of ∂f/∂u, the counterpart of get_jac_prototype(nw)
    (ext/NetworkDynamicsSparsityExt.jl:57-127): (rowptr [dim+1], colidx [nnz]) as int32
    numpy arrays, columns sorted per row."""
    lib = nw._lib
    nnz = C.c_int64()
    capi.check(lib.nd_jacobian_pattern(nw.handle, C.byref(nnz), None, None))
    rowptr = np.empty(nw.dim + 1, dtype=np.int32)
    colidx = np.empty(max(nnz.value, 1), dtype=np.int32)
    capi.check(lib.nd_jacobian_pattern(nw.handle, C.byref(nnz), rowptr.ctypes.data, colidx.ctypes.data))
    return rowptr, colidx[:nnz.value]


def jacobian(nw: Network, u, p, t=0.0, stream=None):
    """∂f/∂u at (u, p, t) with the analytic derivatives of the library components, as a
    torch sparse CSR tensor on u's device (values in the network's precision)."""
    import torch
    rowptr, colidx = jacobian_pattern(nw)
    values = torch.empty(len(colidx), dtype=u.dtype, device=u.device)
    s = stream if stream is not None else torch.cuda.current_stream()
    pp = p.data_ptr() if p is not None and p.numel() else None
    capi.check(nw._lib.nd_jacobian(nw.handle, _dtype_code(u.dtype), values.data_ptr(), u.data_ptr(), pp, float(t),
                                   C.c_void_p(s.cuda_stream)))
    return torch.sparse_csr_tensor(torch.from_numpy(rowptr.astype(np.int64)).to(u.device),
                                   torch.from_numpy(colidx.astype(np.int64)).to(u.device), values,
                                   size=(nw.dim, nw.dim))


def adapt(nw: Network, dtype) -> Network:
    """Counterpart of ``adapt(CuArray{T}, nw)``: a new Network whose handle lives on the
    current CUDA device with caches for element type `dtype` (float32 / float64)."""
    if not iscudacompatible(nw.execution) or not iscudacompatible(nw.aggregator):
        raise capi.ArgumentError(capi.ND_ERR_ARG,
                                 "The provided network has non-cuda compatible aggregator or execution strategies.")
    out = Network.__new__(Network)
    out.__dict__.update({k: v for k, v in nw.__dict__.items() if k not in ("_handle", "_dtype", "_lib")})
    out._handle = None
    out._dtype = None
    out._create(dtype)
    ex = nw.execution
    if ex.sum_order != "sequential":
        out.set_sum_order(ex.sum_order)
    if ex.layout != "auto":
        out.set_layout(ex.layout)
    if ex.kernel_timing:
        out.set_kernel_timing(True)
    return out
