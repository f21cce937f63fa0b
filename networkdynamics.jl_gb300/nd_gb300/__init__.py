"""nd_gb300 — host side of the GB300 network right-hand side of NetworkDynamics.jl.

The compute path is libnd_b200.so (CUDA, sm_103a) behind the C ABI in include/nd_gb300.h;
this package mirrors the reference's Network / ExecutionStyle / Aggregator interface on
top of it.
"""
from . import _capi as capi
from ._capi import ArgumentError, NDError, NotConvergedError, UnsupportedComponentError
from .components import (AntiSymmetric, Directed, EdgeModel, Symmetric, VertexModel, diffusion_dedge, diffusion_edge,
                         diffusion_edge_fid, diffusion_edge_unit, diffusion_odeedge, diffusion_vertex, kuramoto_edge,
                         kuramoto_first, kuramoto_second, kuramoto_vertex_1d, kuramoto_vertex_2d, static_kuramoto_edge,
                         static_line, swing_vertex, piline, pqnode, pqnode_inhomogeneous, generator)
from .graphs import Graph, barabasi_albert, complete_graph, cycle_graph, random_geometric, simple_graph, watts_strogatz
from .network import (ExecutionStyle, GB300Aggregator, GB300Execution, Network, adapt, get_aggr_constructor,
                      iscudacompatible, jacobian, jacobian_pattern, jvp)
from .fixpoint import find_fixpoint
from .mpnn import MPNN

__all__ = [
    "capi", "ArgumentError", "NDError", "NotConvergedError", "UnsupportedComponentError",
    "AntiSymmetric", "Directed", "EdgeModel", "Symmetric", "VertexModel", "diffusion_dedge", "diffusion_edge",
    "diffusion_edge_fid", "diffusion_edge_unit", "diffusion_odeedge", "diffusion_vertex", "kuramoto_edge",
    "kuramoto_first", "kuramoto_second", "kuramoto_vertex_1d", "kuramoto_vertex_2d", "static_kuramoto_edge",
    "static_line", "swing_vertex", "piline", "pqnode", "pqnode_inhomogeneous", "generator",
    "Graph", "barabasi_albert", "complete_graph", "cycle_graph", "random_geometric", "simple_graph",
    "watts_strogatz",
    "ExecutionStyle", "GB300Aggregator", "GB300Execution", "Network", "adapt", "get_aggr_constructor",
    "iscudacompatible", "jacobian", "jacobian_pattern", "jvp", "MPNN", "find_fixpoint",
]
