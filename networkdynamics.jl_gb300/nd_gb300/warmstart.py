"""Swing-network steady states on the GPU, cold-started and warm-started by the MPNN.

The instances follow the swing workload: one graph, per instance half of the vertices
generators with P ~ U(0.5, 1.5), the other half loads with P ~ -U(0.5, 1.5), P shifted to
zero sum, line weights K ~ U(5, 10), M = 1, D = 0.1.  Steady states come from the batched
Newton solve of ``Ensemble.fixpoint`` (the GPU find_fixpoint, src/initialization.jl:44-144),
started from θ = 0 (cold) or from the MPNN prediction (warm); warm-started instances that
do not converge are solved again from the cold start, and their iterations are counted
on both runs.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

from .components import kuramoto_second, static_line
from .ensemble import Ensemble
from .graphs import Graph

M_DEFAULT, D_DEFAULT = 1.0, 0.1


def swing_instances(g: Graph, n: int, seed: int):
    """P [n][nv] and K [n][ne] (float64) of n seeded instances on graph g.  P sums to zero
    over every connected component (a steady state exists only then; for connected
    graphs this is the plain zero-sum shift)."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import connected_components
    rng = np.random.default_rng(seed)
    A = sp.coo_matrix((np.ones(g.ne), (g.src, g.dst)), shape=(g.nv, g.nv))
    ncomp, label = connected_components(A, directed=False)
    count = np.bincount(label, minlength=ncomp)
    P = np.empty((n, g.nv))
    half = g.nv // 2
    for k in range(n):
        perm = rng.permutation(g.nv)
        mag = rng.uniform(0.5, 1.5, g.nv)
        P[k, perm[:half]] = mag[perm[:half]]
        P[k, perm[half:]] = -mag[perm[half:]]
        P[k] -= (np.bincount(label, weights=P[k], minlength=ncomp) / count)[label]
    K = rng.uniform(5.0, 10.0, (n, g.ne))
    return P, K


def swing_flat_params(g: Graph, P, K, M=M_DEFAULT, D=D_DEFAULT) -> np.ndarray:
    """Packed parameters of the instances: per instance (M, D, Pm) per vertex, then K."""
    n = P.shape[0]
    pv = np.empty((n, g.nv, 3))
    pv[:, :, 0] = M
    pv[:, :, 1] = D
    pv[:, :, 2] = P
    return np.concatenate([pv.reshape(n, -1), K], axis=1).ravel()


@dataclass
class FixpointBatch:
    theta: np.ndarray     # [n][nv] steady-state phases
    iters: np.ndarray     # Newton iterations per instance
    cg_iters: np.ndarray  # conjugate-gradient iterations per instance
    resid: np.ndarray     # final max |du|
    status: np.ndarray    # nd_status per instance
    seconds: float        # wall time of the solves (synchronised)


def fixpoints(g: Graph, P, K, theta0=None, tol=1e-10, max_newton=50, chunk=2000) -> FixpointBatch:
    """Steady states of the instances (P, K) by the batched GPU Newton, `chunk` instances
    per ensemble, started from theta0 [n][nv] (default θ = 0)."""
    import torch
    n = P.shape[0]
    out = FixpointBatch(np.empty((n, g.nv)), np.empty(n, np.int64), np.empty(n, np.int64), np.empty(n),
                        np.empty(n, np.int64), 0.0)
    ens = None
    for lo in range(0, n, chunk):
        hi = min(n, lo + chunk)
        if ens is None or ens.n != hi - lo:
            ens = Ensemble([g] * (hi - lo), kuramoto_second(), static_line(), torch.float64)
        p = torch.from_numpy(swing_flat_params(g, P[lo:hi], K[lo:hi])).cuda()
        u0 = torch.zeros(ens.dim, dtype=torch.float64, device="cuda")
        if theta0 is not None:
            th = theta0[lo:hi]
            th = th if isinstance(th, torch.Tensor) else torch.from_numpy(np.asarray(th))
            u0.view(hi - lo, g.nv, 2)[:, :, 0] = th.to(device="cuda", dtype=torch.float64)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = ens.fixpoint(u0, p, tol=tol, max_newton=max_newton)
        torch.cuda.synchronize()
        out.seconds += time.perf_counter() - t0
        out.theta[lo:hi] = r.u.view(hi - lo, g.nv, 2)[:, :, 0].cpu().numpy()
        out.iters[lo:hi] = r.iters.cpu().numpy()
        out.cg_iters[lo:hi] = r.cg_iters.cpu().numpy()
        out.resid[lo:hi] = r.resid.cpu().numpy()
        out.status[lo:hi] = r.status.cpu().numpy()
    return out


def warm_vs_cold(model, g: Graph, P, K, tol=1e-10, max_newton=50, chunk=2000) -> dict:
    """Newton iterations, CG iterations and wall time from the cold start and from the
    MPNN prediction (prediction time included), on the same instances."""
    import torch
    cold = fixpoints(g, P, K, None, tol, max_newton, chunk)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pred = torch.cat([model.forward(P[i:i + chunk], K[i:i + chunk]) for i in range(0, P.shape[0], chunk)])
    torch.cuda.synchronize()
    t_pred = time.perf_counter() - t0
    warm = fixpoints(g, P, K, pred, tol, max_newton, chunk)
    bad = np.nonzero(warm.status != 0)[0]
    iters = warm.iters.copy()
    cg = warm.cg_iters.copy()
    t_fallback = 0.0
    converged = int((warm.status == 0).sum())
    if bad.size:
        fb = fixpoints(g, P[bad], K[bad], None, tol, max_newton, chunk)
        iters[bad] += fb.iters
        cg[bad] += fb.cg_iters
        t_fallback = fb.seconds
        converged += int((fb.status == 0).sum())
    pc = pred.double().cpu().numpy()
    tc = cold.theta - cold.theta.mean(axis=1, keepdims=True)
    err = np.abs(pc - tc).max(axis=1)
    return {
        "instances": int(P.shape[0]),
        "cold": {"newton_iters_mean": float(cold.iters.mean()), "newton_iters_max": int(cold.iters.max()),
                 "cg_iters_mean": float(cold.cg_iters.mean()), "seconds": cold.seconds,
                 "converged": int((cold.status == 0).sum())},
        "warm": {"newton_iters_mean": float(iters.mean()), "newton_iters_max": int(iters.max()),
                 "cg_iters_mean": float(cg.mean()), "seconds": warm.seconds + t_pred + t_fallback,
                 "predict_seconds": t_pred, "fallbacks": int(bad.size),
                 "converged": converged},
        "newton_iter_ratio": float(cold.iters.mean() / max(iters.mean(), 1e-12)),
        "cg_iter_ratio": float(cold.cg_iters.mean() / max(cg.mean(), 1e-12)),
        "prediction_max_abs_err": {"mean": float(err.mean()), "max": float(err.max())},
    }
