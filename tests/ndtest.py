"""Shared helpers of the parity tests."""
from __future__ import annotations

import numpy as np

import nd_gb300 as nd
from oracle import oracle as O


def random_inputs(nw_or_on, vk, rng, dtype=np.float64):
    """Seeded u, p for a network: states N(0,1) (phases U(-π,π)), parameters U(0.5,1.5)
    with swing M = 1, D = 0.1, Pm = ±U(0.5,1.5) shifted to zero sum."""
    dim, pdim = nw_or_on.dim, nw_or_on.pdim
    nv = nw_or_on.nv
    u = rng.normal(size=dim)
    p = rng.uniform(0.5, 1.5, size=pdim)
    if vk == O.V_SWING:
        u[0::2] = rng.uniform(-np.pi, np.pi, size=nv)
        pm = rng.uniform(0.5, 1.5, size=nv) * np.where(np.arange(nv) % 2 == 0, 1, -1)
        pm -= pm.mean()
        p[:3 * nv] = np.stack([np.ones(nv), np.full(nv, 0.1), pm], 1).ravel()
        p[3 * nv:] = rng.uniform(5, 10, size=pdim - 3 * nv)
    return u.astype(dtype), p.astype(dtype)


def gpu_rhs(nw, u, p, device, dtype):
    import torch
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    du = torch.full((nw.dim,), float("nan"), dtype=tdt, device=device)
    ut = torch.from_numpy(np.ascontiguousarray(u, dtype=dtype)).to(device)
    pt = torch.from_numpy(np.ascontiguousarray(p, dtype=dtype)).to(device) if p is not None and len(p) else None
    nw(du, ut, pt, float("nan"))
    return du.cpu().numpy()


def exact_rows(g, vk, ek, u, p, vertices):
    """Sequential-order RHS entries for selected vertices only (exact oracle at any size):
    each row's incident edges in ascending edge id, summed left to right."""
    vertices = np.asarray(vertices, dtype=np.int64)
    dv = O.VDIM[vk]
    pv = O.VPDIM[vk]
    th = u[::dv]
    pe = p[g.nv * pv:] if p is not None else None
    sel = np.zeros(g.nv, dtype=bool)
    sel[vertices] = True
    e_s = np.nonzero(sel[g.src])[0]
    e_d = np.nonzero(sel[g.dst])[0]
    out = {}
    rows = {int(v): [] for v in vertices}
    for e in e_s:
        rows[int(g.src[e])].append((int(e), True))
    for e in e_d:
        rows[int(g.dst[e])].append((int(e), False))
    for v, lst in rows.items():
        lst.sort()
        acc = 0.0
        for e, is_src in lst:
            s, d = int(g.src[e]), int(g.dst[e])
            diff = th[s] - th[d]
            if ek == O.E_DIFFUSION:
                y = pe[e] * diff
            elif ek == O.E_DIFFUSION_UNIT:
                y = diff
            else:
                y = pe[e] * np.sin(diff)
            acc = acc + (-y if is_src else y)
        if vk == O.V_DIFFUSION:
            out[v] = (acc,)
        elif vk == O.V_KURAMOTO:
            out[v] = (p[v] + acc,)
        else:
            M, D, Pm = p[3 * v:3 * v + 3]
            w = u[2 * v + 1]
            out[v] = (w, 1.0 / M * (Pm - D * w + acc))
    return out


def fd_jacobian(on, u, p):
    """Dense central-difference Jacobian of the oracle RHS (FP64).  An entry whose state does
    not enter a row's arithmetic is exactly 0: both perturbed evaluations give the same
    bits."""
    u = np.asarray(u, dtype=np.float64)
    J = np.zeros((on.dim, on.dim))
    for i in range(on.dim):
        h = 1e-6 * max(1.0, abs(u[i]))
        up, um = u.copy(), u.copy()
        up[i] += h
        um[i] -= h
        J[:, i] = (on.rhs(up, p) - on.rhs(um, p)) / (up[i] - um[i])
    return J
