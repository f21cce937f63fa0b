"""Learned warm start for swing-network steady states (libnd_b200.so, nd_mpnn_* entry points).

``MPNN(g)`` is a message-passing network on the fixed graph ``g`` that maps per-instance
power injections P and line weights K to steady-state phases.  Its forward, backward and
Adam kernels are hand-written CUDA (FP32); this module only moves tensors.  The
prediction is used as the initial guess of the GPU Newton solve (``Ensemble.fixpoint``),
the place where the reference's find_fixpoint takes the caller's guess
(src/initialization.jl:44-144).

Weights are saved as a flat binary: the 8-byte magic ``NDMPNN02``, six little-endian
int64 (nv, ne, layers, hidden, hops, nparams), then nparams float32 values.
"""
from __future__ import annotations

import ctypes as C
import struct
from pathlib import Path

import numpy as np

from . import _capi as capi
from .graphs import Graph

MAGIC = b"NDMPNN02"


class MPNN:
    def __init__(self, g: Graph, layers: int = 4, hidden: int = 64, seed: int = 0, hops: int = 1):
        self.graph = g
        self.layers, self.hidden, self.hops = int(layers), int(hidden), int(hops)
        self._lib = capi.load()
        src = np.ascontiguousarray(g.src, dtype=np.int64)
        dst = np.ascontiguousarray(g.dst, dtype=np.int64)
        P = C.POINTER(C.c_int64)
        h = C.c_void_p()
        capi.check(self._lib.nd_mpnn_create(g.nv, g.ne, src.ctypes.data_as(P), dst.ctypes.data_as(P), self.layers,
                                            self.hidden, C.c_uint64(seed), C.byref(h)))
        self._h = h
        capi.check(self._lib.nd_mpnn_set_hops(h, self.hops))
        n = C.c_int64()
        capi.check(self._lib.nd_mpnn_num_params(h, C.byref(n)))
        self.nparams = n.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None:
            try:
                self._lib.nd_mpnn_destroy(h)
            except Exception:
                pass
            self._h = None

    @staticmethod
    def _stream(stream):
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        return C.c_void_p(s.cuda_stream)

    @staticmethod
    def _f32(x, shape, name):
        import torch
        t = x if isinstance(x, torch.Tensor) else torch.as_tensor(np.asarray(x))
        t = t.to(device="cuda", dtype=torch.float32).contiguous()
        if tuple(t.shape) != tuple(shape):
            raise capi.ArgumentError(capi.ND_ERR_ARG, f"{name} must have shape {tuple(shape)}, got {tuple(t.shape)}")
        return t

    # --- parameters ---------------------------------------------------------------------
    def get_params(self, stream=None):
        import torch
        out = torch.empty(self.nparams, dtype=torch.float32, device="cuda")
        capi.check(self._lib.nd_mpnn_get_params(self._h, out.data_ptr(), self._stream(stream)))
        return out

    def set_params(self, params, stream=None):
        t = self._f32(params, (self.nparams,), "params")
        capi.check(self._lib.nd_mpnn_set_params(self._h, t.data_ptr(), self._stream(stream)))

    def get_grads(self, stream=None):
        import torch
        out = torch.empty(self.nparams, dtype=torch.float32, device="cuda")
        capi.check(self._lib.nd_mpnn_get_grads(self._h, out.data_ptr(), self._stream(stream)))
        return out

    # --- compute ------------------------------------------------------------------------
    def forward(self, P, K, stream=None):
        """Centred phase prediction [batch][nv] (float32 CUDA tensor)."""
        import torch
        g = self.graph
        Pt = self._f32(P, (len(P), g.nv), "P")
        Kt = self._f32(K, (len(P), g.ne), "K")
        out = torch.empty_like(Pt)
        capi.check(self._lib.nd_mpnn_forward(self._h, Pt.shape[0], Pt.data_ptr(), Kt.data_ptr(), out.data_ptr(),
                                             self._stream(stream)))
        return out

    def loss_grad(self, P, K, theta_star, stream=None):
        """Loss (device float32 scalar tensor); the gradients stay in the handle."""
        import torch
        g = self.graph
        Pt = self._f32(P, (len(P), g.nv), "P")
        Kt = self._f32(K, (len(P), g.ne), "K")
        Tt = self._f32(theta_star, (len(P), g.nv), "theta_star")
        loss = torch.empty((), dtype=torch.float32, device="cuda")
        capi.check(self._lib.nd_mpnn_loss_grad(self._h, Pt.shape[0], Pt.data_ptr(), Kt.data_ptr(), Tt.data_ptr(),
                                               loss.data_ptr(), self._stream(stream)))
        return loss

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, stream=None):
        capi.check(self._lib.nd_mpnn_adam(self._h, float(lr), float(beta1), float(beta2), float(eps),
                                          self._stream(stream)))

    def reset_optimizer(self, stream=None):
        capi.check(self._lib.nd_mpnn_reset_optimizer(self._h, self._stream(stream)))

    def fit(self, P, K, theta_star, epochs=10, batch=64, lr=1e-3, lr_final=None, seed=0):
        """Minibatch Adam over the training set (device tensors or arrays [n][·]); the
        learning rate decays geometrically from lr to lr_final.  Returns the mean loss
        of each epoch."""
        import torch
        g = self.graph
        Pt = self._f32(P, (len(P), g.nv), "P")
        Kt = self._f32(K, (len(P), g.ne), "K")
        Tt = self._f32(theta_star, (len(P), g.nv), "theta_star")
        n = Pt.shape[0]
        steps = epochs * ((n + batch - 1) // batch)
        lr_final = lr if lr_final is None else lr_final
        decay = (lr_final / lr) ** (1.0 / max(steps - 1, 1))
        gen = torch.Generator(device="cpu")
        gen.manual_seed(seed)
        hist, k = [], 0
        for _ in range(epochs):
            perm = torch.randperm(n, generator=gen).to(Pt.device)
            tot = torch.zeros((), dtype=torch.float64, device=Pt.device)
            nb = 0
            for i in range(0, n, batch):
                idx = perm[i:i + batch]
                loss = self.loss_grad(Pt[idx], Kt[idx], Tt[idx])
                self.adam_step(lr * decay ** k)
                tot += loss.double()
                nb += 1
                k += 1
            hist.append(float(tot.item()) / nb)
        return hist

    # --- persistence --------------------------------------------------------------------
    def save(self, path):
        p = self.get_params().cpu().numpy().astype("<f4")
        with open(path, "wb") as f:
            f.write(MAGIC)
            f.write(struct.pack("<6q", self.graph.nv, self.graph.ne, self.layers, self.hidden, self.hops,
                                self.nparams))
            f.write(p.tobytes())

    def load(self, path):
        data = Path(path).read_bytes()
        if data[:8] != MAGIC:
            raise capi.ArgumentError(capi.ND_ERR_ARG, f"{path} is not an MPNN weight file")
        shape = struct.unpack("<6q", data[8:56])
        if shape != (self.graph.nv, self.graph.ne, self.layers, self.hidden, self.hops, self.nparams):
            raise capi.ArgumentError(capi.ND_ERR_ARG, f"{path} holds a network of another shape")
        n = shape[-1]
        self.set_params(np.frombuffer(data[56:56 + 4 * n], dtype="<f4").astype(np.float32))
