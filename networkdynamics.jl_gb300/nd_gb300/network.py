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
    """Fused single-kernel RHS on one GB300 GPU.  Unbuffered: edges read vertex outputs
    straight from u (the lazy gather of src/gbufs.jl:37-65, done in registers)."""

    buffered = False

    def __repr__(self):
        return "GB300Execution()"


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


def _single_kind(models, what):
    kinds = {m.kind for m in models}
    if None in kinds:
        bad = next(m for m in models if m.kind is None)
        raise capi.UnsupportedComponentError(
            capi.ND_ERR_UNSUPPORTED_COMPONENT,
            f"{what} model {bad.name!r} is not in the GB300 component library; "
            "GB300Execution has no CPU fallback")
    if len(kinds) != 1:
        raise capi.UnsupportedComponentError(
            capi.ND_ERR_UNSUPPORTED_COMPONENT,
            f"GB300Execution needs one homogeneous {what} batch, got {len(kinds)} different {what} models")
    return models[0]


class Network:
    """A network of library components on a graph, in the reference's flat layout:
    u = [vertex states in vertex order], p = [vertex parameters in vertex order,
    edge parameters in edges(g) order] (src/network_structure.jl:224-258)."""

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
        self.graph = g
        self.vertexm = _single_kind(vms, "vertex")
        self.edgem = _single_kind(ems, "edge")
        if self.edgem.coupling != "AntiSymmetric":
            raise capi.UnsupportedComponentError(capi.ND_ERR_UNSUPPORTED_COMPONENT,
                                                 "only AntiSymmetric edges are in the GB300 library")
        self.execution = execution
        self.aggregator = aggregator
        self.dim = g.nv * self.vertexm.dim
        self.pdim = g.nv * self.vertexm.pdim + g.ne * self.edgem.pdim
        self._handle = None
        self._dtype = None
        if dtype is not None:
            self._create(dtype)

    # --- layout helpers -------------------------------------------------------------------
    @property
    def nv(self) -> int:
        return self.graph.nv

    @property
    def ne(self) -> int:
        return self.graph.ne

    def vertex_state_index(self, v: int, k: int = 0) -> int:
        return v * self.vertexm.dim + k

    def vertex_param_index(self, v: int, k: int = 0) -> int:
        return v * self.vertexm.pdim + k

    def edge_param_index(self, e: int, k: int = 0) -> int:
        return self.nv * self.vertexm.pdim + e * self.edgem.pdim + k

    def pflat(self, vertex: dict | None = None, edge: dict | None = None) -> np.ndarray:
        """Flat parameter vector from per-symbol arrays (defaults where omitted)."""
        p = np.zeros(self.pdim, dtype=np.float64)
        vp = self.vertexm.pdim
        for k, name in enumerate(self.vertexm.psym):
            val = (vertex or {}).get(name, self.vertexm.pdef[k] if k < len(self.vertexm.pdef) else None)
            if val is None:
                raise capi.ArgumentError(capi.ND_ERR_ARG, f"vertex parameter {name} has no default")
            p[k:self.nv * vp:vp] = val
        ep, off = self.edgem.pdim, self.nv * vp
        for k, name in enumerate(self.edgem.psym):
            val = (edge or {}).get(name, self.edgem.pdef[k] if k < len(self.edgem.pdef) else None)
            if val is None:
                raise capi.ArgumentError(capi.ND_ERR_ARG, f"edge parameter {name} has no default")
            p[off + k:off + self.ne * ep:ep] = val
        return p

    # --- device handle -------------------------------------------------------------------
    def _create(self, dtype):
        code = _dtype_code(dtype)
        lib = capi.load()
        g = self.graph
        src = np.ascontiguousarray(g.src, dtype=np.int64)
        dst = np.ascontiguousarray(g.dst, dtype=np.int64)
        P = C.POINTER(C.c_int64)
        desc = capi.nd_network_desc(g.nv, g.ne, src.ctypes.data_as(P), dst.ctypes.data_as(P),
                                    self.vertexm.kind, self.edgem.kind, capi.ND_ANTISYMMETRIC, 0)
        h = C.c_void_p()
        capi.check(lib.nd_create(C.byref(desc), code, C.byref(h)))
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
    return out
