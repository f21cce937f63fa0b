"""Steady states of one network on the GPU: the counterpart of the reference's
``find_fixpoint(nw, x0, p)`` (src/initialization.jl:44-144) for swing networks.

The solve is the batched Newton of ``Ensemble.fixpoint`` on an ensemble of one: Newton's
method on the power balance at ω = 0, each step's linear system solved by conjugate
gradients on the analytic Jacobian (the graph Laplacian weighted by K cos Δθ) with the
uniform phase shift projected out.  It stops at max |du| ≤ tol, the residual norm of the
reference (src/initialization.jl:129).  The initial phases come from ``x0`` (default
θ = 0, the reference's ``ufill=0`` start) or from a learned warm start.
"""
from __future__ import annotations

import numpy as np

from . import _capi as capi
from .components import kuramoto_second
from .ensemble import Ensemble


def find_fixpoint(nw, p, x0=None, tol=1e-10, max_newton=50, max_cg=0):
    """Steady state u* of the swing network `nw` with parameters p (flat reference
    layout), as an FP64 CUDA tensor; raises NotConvergedError (the reference's
    NetworkInitError) when Newton does not reach tol.  x0: initial state (its phases are
    used; ω is 0 at any steady state)."""
    import torch
    if nw.vertexm is None or nw.edgem is None or nw.vertexm.kind != capi.ND_V_SWING:
        raise capi.ArgumentError(capi.ND_ERR_ARG,
                                 "find_fixpoint on the GPU supports homogeneous swing (kuramoto_second) networks")
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
    return r.u
