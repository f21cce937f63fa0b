"""Steady states of one network on the GPU: the counterpart of the reference's
``find_fixpoint(nw, x0, p)`` (src/initialization.jl:44-144).  Homogeneous swing networks
use the batched swing Newton below; every other network of the library (power grids included) uses
Newton-GMRES on the sparse Jacobian (nd_find_fixpoint).

The swing solve is the batched Newton of ``Ensemble.fixpoint`` on an ensemble of one:
Newton's method on the power balance at ω = 0, each step's linear system solved by conjugate
gradients on the analytic Jacobian (the graph Laplacian weighted by K cos Δθ) with the
uniform phase shift projected out.  It stops at max |du| ≤ tol, the residual norm of the
reference (src/initialization.jl:129).  The initial phases come from ``x0`` (default
θ = 0, the reference's ``ufill=0`` start) or from a learned warm start.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi as capi
from .components import kuramoto_second
from .ensemble import Ensemble


def find_fixpoint(nw, p, x0=None, tol=1e-10, max_newton=50, max_cg=0, alg=None, t=float("nan"), krylov_dim=40,
                  max_restarts=20):
    """Steady state u* of the network `nw` with parameters p (flat reference layout), as an
    FP64 CUDA tensor; raises NotConvergedError (the reference's NetworkInitError) when
    Newton does not reach tol.  x0: initial state (default zeros, the reference's ufill=0).

    alg: "swing" -- Newton-CG on the power balance of a homogeneous swing network at ω = 0
    (default for such networks); "newton_gmres" -- Newton with restarted GMRES on the sparse
    Jacobian, for any network of the library (default for
    all others)."""
    import torch
    swing = nw.vertexm is not None and nw.edgem is not None and nw.vertexm.kind == capi.ND_V_SWING
    if alg is None:
        alg = "swing" if swing else "newton_gmres"
    if alg == "swing":
        if not swing:
            raise capi.ArgumentError(capi.ND_ERR_ARG,
                                     "find_fixpoint on the GPU supports homogeneous swing (kuramoto_second) networks")
        return _swing_fixpoint(nw, p, x0, tol, max_newton, max_cg)
    if alg != "newton_gmres":
        raise capi.ArgumentError(capi.ND_ERR_ARG, f"unknown fixpoint algorithm {alg!r}")
    pt = torch.as_tensor(np.asarray(p.cpu() if isinstance(p, torch.Tensor) else p, dtype=np.float64)).cuda()
    if pt.numel() != nw.pdim:
        raise capi.ArgumentError(capi.ND_ERR_ARG, f"p does not have expected size {nw.pdim}")
    u = torch.zeros(nw.dim, dtype=torch.float64, device="cuda")
    if x0 is not None:
        x = torch.as_tensor(np.asarray(x0.cpu() if isinstance(x0, torch.Tensor) else x0, dtype=np.float64)).cuda()
        if x.numel() != nw.dim:
            raise capi.ArgumentError(capi.ND_ERR_ARG, f"x0 does not have expected size {nw.dim}")
        u.copy_(x)
    iters, resid = C.c_int32(0), C.c_double(0.0)
    s = torch.cuda.current_stream()
    capi.check(nw._lib.nd_find_fixpoint(nw.handle, u.data_ptr(), pt.data_ptr() if pt.numel() else None, float(t),
                                        float(tol), int(max_newton), int(krylov_dim), int(max_restarts),
                                        C.byref(iters), C.byref(resid), C.c_void_p(s.cuda_stream)))
    find_fixpoint.last_stats = {"newton_iters": iters.value, "resid": resid.value}
    return u


def _swing_fixpoint(nw, p, x0, tol, max_newton, max_cg):
    import torch
    ens = Ensemble([nw.graph], kuramoto_second(), nw.edgem, torch.float64)
    pt = torch.as_tensor(np.asarray(p.cpu() if isinstance(p, torch.Tensor) else p, dtype=np.float64)).cuda()
    if pt.numel() != ens.pdim:
        raise capi.ArgumentError(capi.ND_ERR_ARG, f"p does not have expected size {ens.pdim}")
    u0 = torch.zeros(ens.dim, dtype=torch.float64, device="cuda")
    if x0 is not None:
        x = torch.as_tensor(np.asarray(x0.cpu() if isinstance(x0, torch.Tensor) else x0, dtype=np.float64)).cuda()
        if x.numel() != ens.dim:
            raise capi.ArgumentError(capi.ND_ERR_ARG, f"x0 does not have expected size {ens.dim}")
        u0[0::2] = x[0::2]
    r = ens.fixpoint(u0, pt, tol=tol, max_newton=max_newton, max_cg=max_cg)
    status = int(r.status.cpu().item())
    if status != capi.ND_OK:
        raise capi.NotConvergedError(status, f"find_fixpoint: residual {float(r.resid.cpu().item()):.3e} > {tol} "
                                             f"after {int(r.iters.cpu().item())} Newton iterations")
    find_fixpoint.last_stats = {"newton_iters": int(r.iters.cpu().item()), "resid": float(r.resid.cpu().item())}
    return r.u
