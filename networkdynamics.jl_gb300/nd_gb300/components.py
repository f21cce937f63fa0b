"""Component models of the GB300 library.

Mirrors the reference's ``VertexModel``/``EdgeModel`` (src/component_functions.jl:251,306)
for the components the benchmarks use (test/ComponentLibrary.jl).  Each library
component carries a ``kind`` naming its hand-written CUDA implementation.  A model built
from a user function (``VertexModel(f=..., g=...)``) has no kind, and a GB300 network
that contains one is rejected at construction: the GB300 path never falls back to the
CPU.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

from . import _capi as capi


@dataclass
class VertexModel:
    name: str
    dim: int
    pdim: int
    sym: Sequence[str] = ()
    psym: Sequence[str] = ()
    pdef: Sequence[Optional[float]] = ()
    kind: Optional[int] = None          # ND_V_* of the CUDA implementation, None = user function
    f: Optional[Callable] = None
    g: object = 1                       # StateMask(1): the first state is the output
    outdim: int = 1                     # StateMask(1:outdim)
    # diagonal mass matrix: None (the identity), a scalar for every state (0: algebraic, as the
    # PQ bus) or one entry per state
    mass_matrix: Optional[object] = None
    constants: tuple = ()               # values the component function closes over
    extin: Optional[Sequence] = None    # external inputs (VIndex / EIndex of other components' states)


@dataclass
class EdgeModel:
    name: str
    pdim: int
    psym: Sequence[str] = ()
    pdef: Sequence[Optional[float]] = ()
    kind: Optional[int] = None          # ND_E_* of the CUDA implementation, None = user function
    coupling: str = "AntiSymmetric"
    dim: int = 0                        # static edges: no states
    f: Optional[Callable] = None
    g: Optional[Callable] = None
    outdim: int = 1                     # per side
    extin: Optional[Sequence] = None    # external inputs (VIndex / EIndex of other components' states)
    loopback: bool = False              # a LoopbackConnection: copies the dst output into the src input
    mass_matrix: Optional[object] = None  # diagonal mass matrix of the edge's states, as for vertices


# --- vertices (test/ComponentLibrary.jl) -------------------------------------------------

def diffusion_vertex() -> VertexModel:
    """diffusionvertex!: dv = Σ e   (test/ComponentLibrary.jl:42-46)."""
    return VertexModel("diffusion_vertex", dim=1, pdim=0, sym=("v",), kind=capi.ND_V_DIFFUSION)


def kuramoto_first() -> VertexModel:
    """kuramoto_vertex!: dθ = ω + Σ e   (test/ComponentLibrary.jl:69-72)."""
    return VertexModel("kuramoto_first", dim=1, pdim=1, sym=("θ",), psym=("ω",), pdef=(None,),
                       kind=capi.ND_V_KURAMOTO)


def kuramoto_second() -> VertexModel:
    """kuramoto_inertia! (swing): dδ = ω, dω = 1/M (Pm - D ω + Σ e)   (test/ComponentLibrary.jl:59-67)."""
    return VertexModel("kuramoto_second", dim=2, pdim=3, sym=("δ", "ω"), psym=("M", "D", "Pm"),
                       pdef=(1.0, 0.1, 1.0), kind=capi.ND_V_SWING)


swing_vertex = kuramoto_second


# --- edges ------------------------------------------------------------------------------

def diffusion_edge() -> EdgeModel:
    """diffusionedge!: e = p (v_s - v_d), AntiSymmetric   (test/ComponentLibrary.jl:8-13)."""
    return EdgeModel("diff_edge", pdim=1, psym=("p",), pdef=(1.0,), kind=capi.ND_E_DIFFUSION)


def diffusion_edge_unit() -> EdgeModel:
    """diffusion_edge!: e = v_s - v_d, AntiSymmetric   (test/diffusion_test.jl:57-60, 71)."""
    return EdgeModel("diff_edge_unit", pdim=0, kind=capi.ND_E_DIFFUSION_UNIT)


def kuramoto_edge() -> EdgeModel:
    """kuramoto_edge!: e = K sin(θ_s - θ_d), AntiSymmetric   (test/ComponentLibrary.jl:51-57)."""
    return EdgeModel("kuramoto_edge", pdim=1, psym=("K",), pdef=(None,), kind=capi.ND_E_KURAMOTO)


def static_line() -> EdgeModel:
    """Static power line P = K sin(θ_src - θ_dst) (line_mtk with active = 1,
    test/ComponentLibrary.jl:96-115); the same function as kuramoto_edge."""
    m = kuramoto_edge()
    m.name = "static_line"
    return m


def diffusion_edge_fid() -> EdgeModel:
    """diffusionedge_fid!: the two-sided g e_d = p (v_s - v_d), e_s = -e_d
    (test/ComponentLibrary.jl:22-28)."""
    return EdgeModel("diff_edge_fid", pdim=1, psym=("p",), pdef=(1.0,), kind=capi.ND_E_DIFFUSION,
                     coupling="Fiducial")


def diffusion_odeedge() -> EdgeModel:
    """diffusion_dedge!: ODE edge with states (e_dst, e_src),
    de1 = 1/τ (sin(v_s - v_d) - e1), de2 = 1/τ (sin(v_d - v_s) - e2), outputs
    Fiducial(dst=1:1, src=2:2)   (test/ComponentLibrary.jl:30-40)."""
    return EdgeModel("diff_edge_ode", pdim=1, psym=("τ",), pdef=(100.0,), kind=capi.ND_E_DIFFUSION_ODE,
                     coupling="Fiducial", dim=2)


def diffusion_dedge() -> EdgeModel:
    """The benchmarks' ODE edge: de = 100.0 (sin(..) - e), no parameters
    (benchmark/benchmark_models.jl:11-16)."""
    return EdgeModel("diffusion_dedge", pdim=0, kind=capi.ND_E_DIFFUSION_ODE_FIXED, coupling="Fiducial", dim=2)


def kuramoto_vertex_2d() -> VertexModel:
    """The benchmarks' second-order Kuramoto vertex: dθ = ω, dω = P - 1.0 ω + Σ e
    (benchmark/benchmark_models.jl:37-42)."""
    return VertexModel("kuramoto_vertex_2d", dim=2, pdim=1, sym=("θ", "ω"), psym=("P",), pdef=(None,),
                       kind=capi.ND_V_SWING_UNIT)


kuramoto_vertex_1d = kuramoto_first           # benchmark/benchmark_models.jl:32-35
static_kuramoto_edge = kuramoto_edge          # benchmark/benchmark_models.jl:27-30


# --- output wrappers (src/component_functions.jl:101-203) -----------------------------------

def _rewrap(m: EdgeModel, coupling: str) -> EdgeModel:
    if m.kind is None or m.dim != 0 or m.coupling == "Fiducial":
        raise capi.UnsupportedComponentError(
            capi.ND_ERR_UNSUPPORTED_COMPONENT,
            f"{coupling} wraps the single-sided g of a static library edge, not {m.name!r}")
    return EdgeModel(f"{coupling}({m.name})", pdim=m.pdim, psym=m.psym, pdef=m.pdef, kind=m.kind,
                     coupling=coupling)


def AntiSymmetric(m: EdgeModel) -> EdgeModel:
    """y_dst = g(...), y_src = -y_dst (src/component_functions.jl:117-126)."""
    return _rewrap(m, "AntiSymmetric")


def Symmetric(m: EdgeModel) -> EdgeModel:
    """y_dst = g(...), y_src = y_dst (src/component_functions.jl:142-151)."""
    return _rewrap(m, "Symmetric")


def Directed(m: EdgeModel) -> EdgeModel:
    """y_dst = g(...), no output for the source (y_src = 0) (src/component_functions.jl:167-175)."""
    return _rewrap(m, "Directed")


# --- power-grid components (benchmark/benchmark_models.jl:46-111) ----------------------------

def piline() -> EdgeModel:
    """piline!: π-line with series impedance R + iωL (ω = 2π·50) and shunt capacitances C1,
    C2; two-sided complex current outputs (benchmark/benchmark_models.jl:46-63)."""
    return EdgeModel("piline", pdim=4, psym=("L", "R", "C1", "C2"), pdef=(None, None, None, None),
                     kind=capi.ND_E_PILINE, coupling="Fiducial", outdim=2)


def pqnode() -> VertexModel:
    """pq!: algebraic PQ bus, du = S / conj(i) with S = P + iQ, mass matrix 0
    (benchmark/benchmark_models.jl:65-74)."""
    return VertexModel("pqnode", dim=2, pdim=2, sym=("u_r", "u_i"), psym=("P", "Q"), pdef=(None, None),
                       kind=capi.ND_V_PQ, outdim=2, mass_matrix=0.0)


def generator() -> VertexModel:
    """gen!: generator with states (u_r, u_i, θ, ω) and 11 parameters
    (benchmark/benchmark_models.jl:76-111).  The parameter names are the reference's psym;
    gen! itself unpacks the 8th and 9th parameters as X_q_dash, X_d_dash, and so does the
    GPU implementation."""
    return VertexModel("generator", dim=4, pdim=11, sym=("u_r", "u_i", "θ", "ω"),
                       psym=("H", "P", "D", "Ω", "E_f", "T_d_dash", "T_q_dash", "X_d_dash", "X_q_dash", "X_d",
                             "X_q"),
                       pdef=(None,) * 11, kind=capi.ND_V_GENERATOR, outdim=2)


def pqnode_inhomogeneous(P: float, Q: float) -> VertexModel:
    """pq! closing over its own P and Q (pqnode_inhomogeneous, benchmark/benchmark_models.jl:
    113-123): no parameters; every distinct (P, Q) is a component of its own, hence a batch
    of its own."""
    return VertexModel("pqnode_inhomogeneous", dim=2, pdim=0, sym=("u_r", "u_i"), kind=capi.ND_V_PQ_CONST, outdim=2,
                       mass_matrix=0.0, constants=(float(P), float(Q)))
