"""Undirected simple graphs with Graphs.jl's edge order.

``Graph.src``/``Graph.dst`` list every edge once as (src < dst), sorted lexicographically:
the order of ``edges(g)`` for a Graphs.jl ``SimpleGraph``, which fixes the edge part of
the flat parameter vector and the aggregation order (src/network_structure.jl:240-250).
Vertices are 0-based here; the Julia shim converts from Julia's 1-based indices.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._capi import load_graphgen


@dataclass
class Graph:
    nv: int
    src: np.ndarray  # int64 [ne]
    dst: np.ndarray  # int64 [ne]

    @property
    def ne(self) -> int:
        return int(self.src.shape[0])

    def degree(self) -> np.ndarray:
        return (np.bincount(self.src, minlength=self.nv) + np.bincount(self.dst, minlength=self.nv)).astype(np.int64)

    def edges(self):
        return list(zip(self.src.tolist(), self.dst.tolist()))

    def laplacian(self) -> np.ndarray:
        """Dense graph Laplacian D - A (small graphs only)."""
        L = np.zeros((self.nv, self.nv))
        for s, d in zip(self.src, self.dst):
            L[s, d] -= 1
            L[d, s] -= 1
            L[s, s] += 1
            L[d, d] += 1
        return L


def simple_graph(nv: int, edges) -> Graph:
    """Graph from an iterable of (a, b) pairs; stored in edges(g) order, duplicates dropped."""
    pairs = {(min(a, b), max(a, b)) for a, b in edges if a != b}
    for a, b in pairs:
        if not (0 <= a < nv and 0 <= b < nv):
            raise ValueError(f"edge ({a}, {b}) out of range for {nv} vertices")
    arr = np.array(sorted(pairs), dtype=np.int64).reshape(-1, 2)
    return Graph(nv, np.ascontiguousarray(arr[:, 0]), np.ascontiguousarray(arr[:, 1]))


def complete_graph(n: int) -> Graph:
    return simple_graph(n, [(i, j) for i in range(n) for j in range(i + 1, n)])


def cycle_graph(n: int) -> Graph:
    return simple_graph(n, [(i, (i + 1) % n) for i in range(n)])


def _call_twice(fn, *args, xy=None):
    P = C.POINTER(C.c_int64)
    ne = fn(*args, P(), P(), 0, *([xy] if xy is not None else []))
    if ne < 0:
        raise ValueError("invalid graph generator arguments")
    src = np.empty(max(ne, 1), dtype=np.int64)
    dst = np.empty(max(ne, 1), dtype=np.int64)
    ne2 = fn(*args, src.ctypes.data_as(P), dst.ctypes.data_as(P), ne, *([xy] if xy is not None else []))
    assert ne2 == ne
    return src[:ne].copy(), dst[:ne].copy()


def watts_strogatz(n: int, k: int, beta: float, seed: int = 1) -> Graph:
    lib = load_graphgen()
    src, dst = _call_twice(lib.nd_gen_watts_strogatz, n, k, float(beta), seed)
    return Graph(n, src, dst)


def barabasi_albert(n: int, m: int, seed: int = 1) -> Graph:
    lib = load_graphgen()
    src, dst = _call_twice(lib.nd_gen_barabasi_albert, n, m, seed)
    return Graph(n, src, dst)


def random_geometric(n: int, radius: float, seed: int = 1, return_positions: bool = False):
    lib = load_graphgen()
    xy = np.zeros(2 * n, dtype=np.float64)
    src, dst = _call_twice(lib.nd_gen_random_geometric, n, float(radius), seed,
                           xy=xy.ctypes.data_as(C.POINTER(C.c_double)))
    g = Graph(n, src, dst)
    return (g, xy.reshape(n, 2)) if return_positions else g
