"""Ensembles of networks on the GPU: many instances of one component pair on different
graphs (basin-stability perturbations, parameter sweeps), packed one after another.

Each instance keeps the reference's flat layout, so ``ens.u_slice(i)`` / ``ens.p_slice(i)``
of the packed vectors are exactly the ``u`` / ``p`` of ``Network(graphs[i], vm, em)``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _capi as capi
from .components import EdgeModel, VertexModel
from .network import _dtype_code as _network_dtype_code


def _dtype_code(dtype) -> int:
    """torch.float64 / torch.float32 as for networks, or "f32x2": FP64 buffers with the
    RHS computed in double-float on the FP32 pipe (ensembles only)."""
    if isinstance(dtype, str) and dtype.lower() in ("f32x2", "float32x2", "double-float"):
        return capi.ND_F32X2
    return _network_dtype_code(dtype)


@dataclass
class EnsembleSolveResult:
    u: object          # packed FP64 CUDA tensor
    status: np.ndarray  # per instance nd_status
    nsteps: np.ndarray  # per instance steps
    control: object = None  # per instance (t, dt, qold), FP64 CUDA tensor [n, 3] (snapshot solves)

    def save_snapshot(self, directory) -> None:
        """Write the state and step control as .npy files (u, control, status, nsteps), to
        continue the solve later with ``Ensemble.solve_tsit5(..., snapshot=load_snapshot(dir))``."""
        from pathlib import Path
        if self.control is None:
            raise capi.ArgumentError(capi.ND_ERR_ARG, "solve with snapshot=True to record the step control")
        d = Path(directory)
        d.mkdir(parents=True, exist_ok=True)
        np.save(d / "u.npy", self.u.cpu().numpy())
        np.save(d / "control.npy", self.control.cpu().numpy())
        np.save(d / "status.npy", _host(self.status))
        np.save(d / "nsteps.npy", _host(self.nsteps))


@dataclass
class EnsembleSnapshot:
    u: np.ndarray        # packed FP64 state at the snapshot time
    control: np.ndarray  # [n, 3]: time reached, next step size, error history

    @property
    def t(self) -> float:
        return float(self.control[:, 0].min()) if len(self.control) else 0.0


def load_snapshot(directory) -> EnsembleSnapshot:
    from pathlib import Path
    d = Path(directory)
    return EnsembleSnapshot(np.load(d / "u.npy"), np.load(d / "control.npy"))


def _host(x):
    return x.cpu().numpy() if hasattr(x, "cpu") else np.asarray(x)


@dataclass
class FixpointResult:
    u: object
    iters: np.ndarray
    resid: np.ndarray
    status: np.ndarray
    cg_iters: np.ndarray


class Ensemble:
    def __init__(self, graphs, vertexm: VertexModel, edgem: EdgeModel, dtype):
        import torch
        if vertexm.kind is None or edgem.kind is None:
            raise capi.UnsupportedComponentError(capi.ND_ERR_UNSUPPORTED_COMPONENT,
                                                 "ensemble components must come from the GB300 library")
        self.graphs = list(graphs)
        self.vertexm, self.edgem = vertexm, edgem
        self.n = len(self.graphs)
        nvs = np.array([g.nv for g in self.graphs], dtype=np.int64)
        nes = np.array([g.ne for g in self.graphs], dtype=np.int64)
        self.v_offset = np.concatenate([[0], np.cumsum(nvs)]).astype(np.int64)
        self.e_offset = np.concatenate([[0], np.cumsum(nes)]).astype(np.int64)
        src = np.concatenate([g.src for g in self.graphs]).astype(np.int64) if nes.sum() else np.zeros(1, np.int64)
        dst = np.concatenate([g.dst for g in self.graphs]).astype(np.int64) if nes.sum() else np.zeros(1, np.int64)
        P = C.POINTER(C.c_int64)
        desc = capi.nd_ensemble_desc(self.n, self.v_offset.ctypes.data_as(P), self.e_offset.ctypes.data_as(P),
                                     src.ctypes.data_as(P), dst.ctypes.data_as(P), vertexm.kind, edgem.kind,
                                     capi.ND_ANTISYMMETRIC, 0)
        self._lib = capi.load()
        h = C.c_void_p()
        capi.check(self._lib.nd_ensemble_create(C.byref(desc), _dtype_code(dtype), C.byref(h)))
        self._h = h
        self.dtype_code = _dtype_code(dtype)
        # element type of p and of the RHS buffers (the state is FP64 in every precision)
        self.torch_dtype = torch.float32 if self.dtype_code == capi.ND_F32 else torch.float64
        dim, pdim = C.c_int64(), C.c_int64()
        capi.check(self._lib.nd_ensemble_get_info(h, C.byref(dim), C.byref(pdim)))
        self.dim, self.pdim = dim.value, pdim.value
        self.u_offset = self.v_offset * vertexm.dim
        self.p_offset = self.v_offset * vertexm.pdim + self.e_offset * edgem.pdim

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None:
            try:
                self._lib.nd_ensemble_destroy(h)
            except Exception:
                pass
            self._h = None

    def u_slice(self, i):
        return slice(int(self.u_offset[i]), int(self.u_offset[i + 1]))

    def p_slice(self, i):
        return slice(int(self.p_offset[i]), int(self.p_offset[i + 1]))

    def _stream(self, stream):
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        return C.c_void_p(s.cuda_stream)

    def rhs(self, du, u, p, stream=None):
        capi.check(self._lib.nd_ensemble_rhs(self._h, self.dtype_code, du.data_ptr(), u.data_ptr(),
                                             p.data_ptr() if p is not None else None, self._stream(stream)))

    def solve_tsit5(self, u0, p, tspan, reltol=1e-6, abstol=1e-8, max_steps=0, threads=0, stream=None,
                    snapshot=False):
        """Tsit5 of every instance over tspan.  max_steps is the per-instance step budget;
        0 means capi.ND_ENSEMBLE_DEFAULT_MAX_STEPS (1e5, SciML's default maxiters).  An
        instance that runs out gets status ND_ERR_MAXITERS.

        snapshot=True records each instance's step control (result.control) so that the
        result can be saved and continued; snapshot=<EnsembleSnapshot> (from
        load_snapshot) continues a saved solve: u0 defaults to the snapshot's state, and
        every instance starts with the snapshot's step size and error history instead of
        the initial-step heuristic."""
        import torch
        resume = isinstance(snapshot, EnsembleSnapshot)
        if resume and u0 is None:
            u0 = snapshot.u
        u = u0.to(torch.float64).clone() if isinstance(u0, torch.Tensor) else torch.tensor(u0, dtype=torch.float64,
                                                                                           device="cuda")
        dev = u.device
        status = torch.zeros(self.n, dtype=torch.int32, device=dev)
        nsteps = torch.zeros(self.n, dtype=torch.int64, device=dev)
        control = None
        if resume:
            if snapshot.control.shape != (self.n, 3):
                raise capi.ArgumentError(capi.ND_ERR_ARG, f"snapshot control must have shape ({self.n}, 3)")
            if np.any(snapshot.control[:, 0] != snapshot.control[0, 0]):
                # an instance that stopped early (step budget, step underflow) has no state at
                # the snapshot time
                raise capi.ArgumentError(capi.ND_ERR_ARG, "snapshot instances ended at different times")
            control = torch.from_numpy(np.ascontiguousarray(snapshot.control, dtype=np.float64)).to(dev)
        elif snapshot:
            control = torch.zeros((self.n, 3), dtype=torch.float64, device=dev)
        capi.check(self._lib.nd_ensemble_solve_tsit5_ex(
            self._h, u.data_ptr(), p.data_ptr() if p is not None else None, float(tspan[0]), float(tspan[1]),
            float(reltol), float(abstol), int(max_steps), int(threads), status.data_ptr(), nsteps.data_ptr(),
            control.data_ptr() if control is not None else None, int(resume), self._stream(stream)))
        return EnsembleSolveResult(u, status, nsteps, control)

    def autotune(self, u0, p, t0=0.0, t_probe=0.5, reltol=1e-6, abstol=1e-8, stream=None, cache=True):
        """Pick the threads per instance of the solver by timing a short solve with each
        candidate block size (synchronous), and use it for threads = 0.  With ``cache``,
        a block size that an earlier process picked for the same workload on the same
        device is taken from the autotuner cache file instead (nd_gb300.tuning)."""
        import torch
        from .tuning import AutotuneCache, workload_key
        key = store = None
        if cache:
            key = workload_key(torch.cuda.get_device_name(u0.device), int(self._lib.nd_version()), self.vertexm.kind,
                               self.edgem.kind, self.dtype_code, self.n, int(self.v_offset[-1]),
                               int(self.e_offset[-1]), float(reltol), float(abstol), float(t_probe))
            store = AutotuneCache()
            hit = store.get(key)
            if hit in (64, 128, 256, 512):  # the block sizes the solver takes
                self.set_threads(hit)
                return hit
        chosen = C.c_int()
        capi.check(self._lib.nd_ensemble_autotune(self._h, u0.data_ptr(), p.data_ptr() if p is not None else None,
                                                  float(t0), float(t_probe), float(reltol), float(abstol),
                                                  C.byref(chosen), self._stream(stream)))
        if store is not None:
            store.put(key, chosen.value)
        return chosen.value

    def set_threads(self, threads):
        capi.check(self._lib.nd_ensemble_set_threads(self._h, int(threads)))

    def fixpoint(self, u0, p, tol=1e-10, max_newton=50, max_cg=0, stream=None):
        import torch
        u = u0.to(torch.float64).clone()
        dev = u.device
        iters = torch.zeros(self.n, dtype=torch.int32, device=dev)
        resid = torch.zeros(self.n, dtype=torch.float64, device=dev)
        status = torch.zeros(self.n, dtype=torch.int32, device=dev)
        cg = torch.zeros(self.n, dtype=torch.int32, device=dev)
        capi.check(self._lib.nd_ensemble_fixpoint(self._h, u.data_ptr(), p.data_ptr(), float(tol), int(max_newton),
                                                  int(max_cg), iters.data_ptr(), resid.data_ptr(), status.data_ptr(),
                                                  cg.data_ptr(), self._stream(stream)))
        return FixpointResult(u, iters, resid, status, cg)
