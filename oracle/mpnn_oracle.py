"""CPU oracle of the warm-start message-passing network (test infrastructure only).

float64 numpy restatement of the forward pass, the loss and its gradient for the
network in networkdynamics.jl_gb300/csrc/nd_mpnn.cu, used to check the CUDA forward,
backward and Adam kernels.  The network has no reference counterpart (the reference's
find_fixpoint, src/initialization.jl:44-144, starts Newton from a caller-given guess), so
parity here means agreement with this restatement, whose gradient is itself checked
against central finite differences in the CPU tests.

Layout (identical to the CUDA side): parameters = W_in[H][2], b_in[H], per layer
W_s[H][H], W_m[H][H], b[H], then w_out[H], b_out; rows of a weight matrix are output
units.  Per instance and vertex i (κ = 10):
    s_i = Σ_j K_ij / κ,  x_i = [P_i, log(1 + s_i)],  h0 = tanh(W_in x + b_in)
    m = M^hops h with (M h)_i = (1 / s_i) Σ_j (K_ij / κ) h_j,  a = tanh(W_s h + W_m m + b),  h' = h + a
    y = w_out · h + b_out,  θ̂ = y - mean(y)
    loss = mean over instances and vertices of (θ̂ - (θ* - mean θ*))²
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

H = 64
KAPPA = 10.0


def offsets(L: int, h: int = H) -> dict:
    o = {"W_in": 0, "b_in": 2 * h}
    base = 3 * h
    for l in range(L):
        o[f"W_s{l}"] = base
        o[f"W_m{l}"] = base + h * h
        o[f"b{l}"] = base + 2 * h * h
        base += 2 * h * h + h
    o["w_out"] = base
    o["b_out"] = base + h
    o["n"] = base + h + 1
    return o


def unpack(params: np.ndarray, L: int, h: int = H) -> dict:
    o = offsets(L, h)
    p = np.asarray(params, dtype=np.float64)
    d = {"W_in": p[0:2 * h].reshape(h, 2), "b_in": p[2 * h:3 * h]}
    for l in range(L):
        d[f"W_s{l}"] = p[o[f"W_s{l}"]:o[f"W_s{l}"] + h * h].reshape(h, h)
        d[f"W_m{l}"] = p[o[f"W_m{l}"]:o[f"W_m{l}"] + h * h].reshape(h, h)
        d[f"b{l}"] = p[o[f"b{l}"]:o[f"b{l}"] + h]
    d["w_out"] = p[o["w_out"]:o["w_out"] + h]
    d["b_out"] = p[o["b_out"]]
    return d


def random_params(L: int, rng, scale: float = 0.3, h: int = H) -> np.ndarray:
    return rng.uniform(-scale, scale, offsets(L, h)["n"])


def _adjacency(nv, src, dst, k):
    A = sp.coo_matrix((np.concatenate([k, k]), (np.concatenate([dst, src]), np.concatenate([src, dst]))),
                      shape=(nv, nv))
    return A.tocsr()


def forward(params, L, nv, src, dst, P, K, keep=False, hops=1):
    """θ̂ [B][nv] (and the activations when keep); messages are M^hops h."""
    d = unpack(params, L)
    P = np.atleast_2d(np.asarray(P, np.float64))
    K = np.atleast_2d(np.asarray(K, np.float64))
    out, caches = [], []
    for b in range(P.shape[0]):
        A = _adjacency(nv, src, dst, K[b] / KAPPA)
        s = np.asarray(A.sum(axis=1)).ravel()
        inv_s = np.where(s > 0, 1.0 / np.where(s > 0, s, 1.0), 0.0)
        x = np.stack([P[b], np.log1p(s)], 1)
        h = np.tanh(x @ d["W_in"].T + d["b_in"])
        hs, ms, As = [h], [], []
        for l in range(L):
            m = h
            for _ in range(hops):
                m = inv_s[:, None] * (A @ m)
            a = np.tanh(h @ d[f"W_s{l}"].T + m @ d[f"W_m{l}"].T + d[f"b{l}"])
            h = h + a
            ms.append(m)
            As.append(a)
            hs.append(h)
        y = h @ d["w_out"] + d["b_out"]
        out.append(y - y.mean())
        caches.append((A, inv_s, x, hs, ms, As, y, hops))
    th = np.stack(out)
    return (th, caches) if keep else th


def loss_grad(params, L, nv, src, dst, P, K, target, hops=1):
    """(loss, gradient) of the mean squared centred error, gradient in the flat layout."""
    d = unpack(params, L)
    o = offsets(L)
    th, caches = forward(params, L, nv, src, dst, P, K, keep=True, hops=hops)
    T = np.atleast_2d(np.asarray(target, np.float64))
    Tc = T - T.mean(axis=1, keepdims=True)
    B = th.shape[0]
    count = B * nv
    e = th - Tc
    loss = float((e * e).sum() / count)
    g = np.zeros(o["n"])
    for b in range(B):
        A, inv_s, x, hs, ms, As, y, hops = caches[b]
        dy = 2.0 * (e[b] - e[b].mean()) / count
        g[o["w_out"]:o["w_out"] + H] += hs[L].T @ dy
        g[o["b_out"]] += dy.sum()
        dh = np.outer(dy, d["w_out"])
        for l in range(L - 1, -1, -1):
            dz = dh * (1.0 - As[l] ** 2)
            g[o[f"W_s{l}"]:o[f"W_s{l}"] + H * H] += (dz.T @ hs[l]).ravel()
            g[o[f"W_m{l}"]:o[f"W_m{l}"] + H * H] += (dz.T @ ms[l]).ravel()
            g[o[f"b{l}"]:o[f"b{l}"] + H] += dz.sum(0)
            dm = dz @ d[f"W_m{l}"]
            for _ in range(hops):  # (M^hops)^T = (A diag(1/s))^hops
                dm = A.T @ (inv_s[:, None] * dm)
            dh = dh + dz @ d[f"W_s{l}"] + dm
        dz0 = dh * (1.0 - hs[0] ** 2)
        g[0:2 * H] += (dz0.T @ x).ravel()
        g[2 * H:3 * H] += dz0.sum(0)
    return loss, g


def loss_only(params, L, nv, src, dst, P, K, target, hops=1):
    th = forward(params, L, nv, src, dst, P, K, hops=hops)
    T = np.atleast_2d(np.asarray(target, np.float64))
    e = th - (T - T.mean(axis=1, keepdims=True))
    return float((e * e).sum() / e.size)


def adam(params, grad, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One bias-corrected Adam step (Kingma & Ba 2015, Algorithm 1); returns (params, m, v)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    p = params - lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
    return p, m, v
