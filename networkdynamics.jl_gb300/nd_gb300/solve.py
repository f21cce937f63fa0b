"""Time integration on the GPU: the counterpart of
``solve(ODEProblem(nw, u0, (t0, t1), p), Tsit5(); reltol, abstol)`` (src/post_utils.jl:43-100
builds the ODEFunction around the network RHS; Tsit5 comes from OrdinaryDiffEqTsit5).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _capi as capi


@dataclass
class SolveStats:
    naccept: int
    nreject: int
    nf: int
    t_final: float
    status: int


def _as_device(x, dtype, device):
    import torch
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device=device)


def solve_tsit5(nw, u0, p, tspan, reltol=1e-3, abstol=1e-6, max_steps=0, stream=None):
    """Integrate the network from tspan[0] to tspan[1]; returns (u(t1) as an FP64 CUDA
    tensor, SolveStats).  The state is FP64; the RHS runs in the network's precision."""
    import torch
    lib = capi.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    u = _as_device(u0, torch.float64, dev).clone()
    if u.numel() != nw.dim:
        raise capi.ArgumentError(capi.ND_ERR_ARG, f"u0 does not have expected size {nw.dim}")
    pdt = torch.float64 if nw._dtype == capi.ND_F64 else torch.float32
    pt = _as_device(p, pdt, dev) if (p is not None and nw.pdim > 0) else None
    st = capi.nd_solve_stats()
    s = stream if stream is not None else torch.cuda.current_stream()
    capi.check(lib.nd_solve_tsit5(nw.handle, u.data_ptr(), pt.data_ptr() if pt is not None else None,
                                  float(tspan[0]), float(tspan[1]), float(reltol), float(abstol), int(max_steps),
                                  C.byref(st), C.c_void_p(s.cuda_stream)))
    return u, SolveStats(st.naccept, st.nreject, st.nf, st.t_final, st.status)


def solve_rosenbrock23(nw, u0, p, tspan, mass_matrix="auto", reltol=1e-3, abstol=1e-6, max_steps=0, stream=None):
    """Integrate M u' = f(u) by Rosenbrock23 on the GPU, the counterpart of
    ``solve(ODEProblem(nw, u0, tspan, p), Rosenbrock23())`` for networks whose components
    carry mass matrices.  mass_matrix: "auto" takes the network's own
    (``nw.mass_matrix()``, construct_mass_matrix of src/construction.jl:409-467), None is
    the identity, or a diagonal of length dim.  u0 must satisfy the algebraic rows.
    Returns (u(t1) as an FP64 CUDA tensor, SolveStats).  FP64 networks only."""
    return _solve_rosenbrock("nd_solve_rosenbrock23", nw, u0, p, tspan, mass_matrix, reltol, abstol, max_steps,
                             stream)


def solve_rodas4(nw, u0, p, tspan, mass_matrix="auto", reltol=1e-3, abstol=1e-6, max_steps=0, stream=None):
    """Integrate M u' = f(u) by Rodas4 (order 4, stiffly accurate) on the GPU, the
    counterpart of ``solve(ODEProblem(nw, u0, tspan, p), Rodas4())``.  Arguments and result
    as for solve_rosenbrock23; six linear solves per step instead of three, and far fewer
    steps at tight tolerances."""
    return _solve_rosenbrock("nd_solve_rodas4", nw, u0, p, tspan, mass_matrix, reltol, abstol, max_steps, stream)


def _solve_rosenbrock(entry, nw, u0, p, tspan, mass_matrix, reltol, abstol, max_steps, stream):
    import torch
    lib = capi.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    u = _as_device(u0, torch.float64, dev).clone()
    if u.numel() != nw.dim:
        raise capi.ArgumentError(capi.ND_ERR_ARG, f"u0 does not have expected size {nw.dim}")
    mm = nw.mass_matrix() if isinstance(mass_matrix, str) and mass_matrix == "auto" else mass_matrix
    md = None
    if mm is not None:
        md = _as_device(np.broadcast_to(np.asarray(mm, dtype=np.float64), (nw.dim,)).copy(), torch.float64, dev)
    pt = _as_device(p, torch.float64, dev) if (p is not None and nw.pdim > 0) else None
    st = capi.nd_solve_stats()
    s = stream if stream is not None else torch.cuda.current_stream()
    capi.check(getattr(lib, entry)(nw.handle, u.data_ptr(), pt.data_ptr() if pt is not None else None,
                                   md.data_ptr() if md is not None else None, float(tspan[0]), float(tspan[1]),
                                   float(reltol), float(abstol), int(max_steps), C.byref(st),
                                   C.c_void_p(s.cuda_stream)))
    return u, SolveStats(st.naccept, st.nreject, st.nf, st.t_final, st.status)
