"""ORACLE — test infrastructure, not product code.

Python side of the CPU oracle:

* ``OracleNetwork``   — ctypes wrapper of oracle/nd_oracle.c (the C restatement of the
  reference RHS, src/coreloop.jl:1-102 with src/aggregators.jl:133-151), its threaded
  Polyester restatement, and the CPU Tsit5.
* ``rhs_numpy``       — an independent numpy mirror of the same RHS for small cases.  It
  uses ``np.add.at``, which applies the additions in index order, to reproduce
  SequentialAggregator's order.
* ``newton_fixpoint`` — dense Newton on the swing/Kuramoto steady state, the restated
  find_fixpoint (src/initialization.jl:44-144) for small networks.
* ``collect_externals`` / ``gen_loopback_map`` / ``apply_loopback`` — the external-input
  and loopback copies of the core loop (src/external_inputs.jl, src/post_utils.jl).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "nd_oracle.c"
BUILD_DIR = HERE / "_build"
LIB = BUILD_DIR / "liboracle.so"

V_DIFFUSION, V_KURAMOTO, V_SWING, V_SWING_UNIT, V_PQ, V_GENERATOR, V_PQ_CONST = 1, 2, 3, 4, 5, 6, 7
E_DIFFUSION, E_DIFFUSION_UNIT, E_KURAMOTO, E_DIFFUSION_ODE, E_DIFFUSION_ODE_FIXED, E_PILINE = 1, 2, 3, 4, 5, 6
C_ANTISYMMETRIC, C_SYMMETRIC, C_DIRECTED, C_FIDUCIAL = 1, 2, 3, 4

VDIM = {V_DIFFUSION: 1, V_KURAMOTO: 1, V_SWING: 2, V_SWING_UNIT: 2, V_PQ: 2, V_GENERATOR: 4, V_PQ_CONST: 2}
VPDIM = {V_DIFFUSION: 0, V_KURAMOTO: 1, V_SWING: 3, V_SWING_UNIT: 1, V_PQ: 2, V_GENERATOR: 11, V_PQ_CONST: 0}
EDIM = {E_DIFFUSION: 0, E_DIFFUSION_UNIT: 0, E_KURAMOTO: 0, E_DIFFUSION_ODE: 2, E_DIFFUSION_ODE_FIXED: 2,
        E_PILINE: 0}
EPDIM = {E_DIFFUSION: 1, E_DIFFUSION_UNIT: 0, E_KURAMOTO: 1, E_DIFFUSION_ODE: 1, E_DIFFUSION_ODE_FIXED: 0,
         E_PILINE: 4}


def build_oracle(force: bool = False) -> Path:
    """Compile the C restatement (no FMA contraction, OpenMP for the threaded variant)."""
    BUILD_DIR.mkdir(exist_ok=True)
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp", str(SRC),
           "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


class Tsit5Stats(C.Structure):
    _fields_ = [("naccept", C.c_int64), ("nreject", C.c_int64), ("nf", C.c_int64),
                ("t_final", C.c_double), ("dt_last", C.c_double), ("status", C.c_int)]


_lib = None


def load():
    global _lib
    if _lib is None:
        build_oracle()
        lib = C.CDLL(str(LIB))
        vp, i64 = C.c_void_p, C.c_int64
        P64 = C.POINTER(C.c_int64)
        P32 = C.POINTER(C.c_int32)
        lib.nd_oracle_layout_new.restype = vp
        lib.nd_oracle_layout_new.argtypes = [i64, i64, P64, P64, P32, P32]
        lib.nd_oracle_layout_new_batched.restype = vp
        lib.nd_oracle_layout_new_batched.argtypes = [i64, i64, P64, P64, C.c_int, P32, P32, C.c_int, P32, P32, P32,
                                                     vp]
        lib.nd_oracle_layout_free.argtypes = [vp]
        lib.nd_oracle_gen_barabasi_albert.restype = i64
        lib.nd_oracle_gen_barabasi_albert.argtypes = [i64, i64, C.c_uint64, P64, P64, i64]
        for fn in ("nd_oracle_dim", "nd_oracle_pdim"):
            getattr(lib, fn).restype = i64
            getattr(lib, fn).argtypes = [vp]
        lib.nd_oracle_depth.restype = C.c_int
        lib.nd_oracle_depth.argtypes = [vp]
        for fn in ("nd_oracle_n_out", "nd_oracle_n_aggr"):
            getattr(lib, fn).restype = i64
            getattr(lib, fn).argtypes = [vp]
        for fn in ("nd_oracle_v_data", "nd_oracle_v_para", "nd_oracle_e_para", "nd_oracle_e_data"):
            getattr(lib, fn).restype = i64
            getattr(lib, fn).argtypes = [vp, i64]
        for fn in ("nd_oracle_rhs_f64", "nd_oracle_rhs_f32", "nd_oracle_rhs_poly_f64", "nd_oracle_rhs_poly_f32"):
            getattr(lib, fn).restype = None
            getattr(lib, fn).argtypes = [vp, vp, vp, vp, vp, vp]
        lib.nd_oracle_num_threads.restype = C.c_int
        lib.nd_oracle_set_num_threads.argtypes = [C.c_int]
        for fn in (lib.nd_oracle_tsit5, lib.nd_oracle_tsit5_threaded):
            fn.restype = C.c_int
            fn.argtypes = [vp, vp, vp, C.c_double, C.c_double, C.c_double, C.c_double, i64, C.POINTER(Tsit5Stats)]
        lib.nd_oracle_tsit5_tableau.argtypes = [vp, vp, vp]
        _lib = lib
    return _lib


class EdgeList:
    """An undirected graph as the oracle's generators return it: 0-based (src < dst) pairs in
    edges(g) order."""

    def __init__(self, nv, src, dst):
        self.nv, self.src, self.dst = int(nv), src, dst

    @property
    def ne(self):
        return int(self.src.shape[0])


def barabasi_albert(n, m, seed=1):
    """The package's seeded Barabási–Albert graph, generated by the oracle's own copy of the
    generator (the benchmark's CPU reference arm uses it so that it loads nothing of the
    package)."""
    lib = load()
    P64 = C.POINTER(C.c_int64)
    ne = lib.nd_oracle_gen_barabasi_albert(n, m, seed, P64(), P64(), 0)
    if ne < 0:
        raise ValueError("invalid Barabasi-Albert arguments" if ne == -1 else "out of memory")
    src = np.empty(max(ne, 1), dtype=np.int64)
    dst = np.empty(max(ne, 1), dtype=np.int64)
    lib.nd_oracle_gen_barabasi_albert(n, m, seed, src.ctypes.data_as(P64), dst.ctypes.data_as(P64), ne)
    return EdgeList(n, src[:ne].copy(), dst[:ne].copy())


def tsit5_tableau():
    lib = load()
    c = np.zeros(7)
    a = np.zeros((7, 6))
    bt = np.zeros(7)
    lib.nd_oracle_tsit5_tableau(c.ctypes.data, a.ctypes.data, bt.ctypes.data)
    return c, a, bt


def _ptr(x):
    return x.ctypes.data if x is not None and x.size else None


class OracleNetwork:
    """Reference layout + sequential RHS for a graph (0-based src/dst in edges(g) order).
    ``vkind``/``ekind`` are scalars (one batch) or per-vertex / per-edge arrays."""

    def __init__(self, nv, src, dst, vkind, ekind):
        self.lib = load()
        self.nv = int(nv)
        self.src = np.ascontiguousarray(src, dtype=np.int64)
        self.dst = np.ascontiguousarray(dst, dtype=np.int64)
        self.ne = int(self.src.shape[0])
        self.vkind = np.ascontiguousarray(np.broadcast_to(np.asarray(vkind, dtype=np.int32), (self.nv,)))
        self.ekind = np.ascontiguousarray(np.broadcast_to(np.asarray(ekind, dtype=np.int32), (self.ne,)))
        P64 = C.POINTER(C.c_int64)
        P32 = C.POINTER(C.c_int32)
        self.L = self.lib.nd_oracle_layout_new(self.nv, self.ne, self.src.ctypes.data_as(P64),
                                               self.dst.ctypes.data_as(P64), self.vkind.ctypes.data_as(P32),
                                               self.ekind.ctypes.data_as(P32))
        self._finish()

    def _finish(self):
        if not self.L:
            raise ValueError("all vertex models and all edge models must have the same output dimension")
        self.dim = int(self.lib.nd_oracle_dim(self.L))
        self.pdim = int(self.lib.nd_oracle_pdim(self.L))
        self.depth = int(self.lib.nd_oracle_depth(self.L))
        self.n_out = int(self.lib.nd_oracle_n_out(self.L))
        self.n_aggr = int(self.lib.nd_oracle_n_aggr(self.L))

    @classmethod
    def from_graph(cls, g, vkind, ekind):
        return cls(g.nv, g.src, g.dst, vkind, ekind)

    @classmethod
    def from_batches(cls, nv, src, dst, vertex_batches, vertex_batch, edge_batches, edge_batch, vertex_constants=None):
        """Network with explicit batches (the reference's order of first appearance):
        ``vertex_batches`` lists the vertex kind of every batch, ``edge_batches`` the
        (edge kind, coupling) of every batch; ``vertex_batch`` / ``edge_batch`` give each
        component's batch."""
        self = cls.__new__(cls)
        self.lib = load()
        self.nv = int(nv)
        self.src = np.ascontiguousarray(src, dtype=np.int64)
        self.dst = np.ascontiguousarray(dst, dtype=np.int64)
        self.ne = int(self.src.shape[0])
        vbk = np.ascontiguousarray(vertex_batches, dtype=np.int32)
        ebk = np.ascontiguousarray([k for k, _ in edge_batches] or [0], dtype=np.int32)
        ebc = np.ascontiguousarray([c for _, c in edge_batches] or [0], dtype=np.int32)
        vb = np.ascontiguousarray(vertex_batch, dtype=np.int32)
        eb = np.ascontiguousarray(edge_batch if self.ne else np.zeros(1), dtype=np.int32)
        self.vkind = vbk[vb]
        self.ekind = ebk[eb[:self.ne]] if self.ne else np.zeros(0, dtype=np.int32)
        self._vconst = (None if vertex_constants is None
                        else np.ascontiguousarray(vertex_constants, dtype=np.float64).reshape(-1))
        P64 = C.POINTER(C.c_int64)
        P32 = C.POINTER(C.c_int32)
        self.L = self.lib.nd_oracle_layout_new_batched(
            self.nv, self.ne, self.src.ctypes.data_as(P64), self.dst.ctypes.data_as(P64), len(vbk),
            vbk.ctypes.data_as(P32), vb.ctypes.data_as(P32), len(edge_batches), ebk.ctypes.data_as(P32),
            ebc.ctypes.data_as(P32), eb.ctypes.data_as(P32), _ptr(self._vconst))
        self._finish()
        return self

    def __del__(self):
        if getattr(self, "L", None):
            self.lib.nd_oracle_layout_free(self.L)
            self.L = None

    def _rhs(self, fn, dtype, u, p):
        u = np.ascontiguousarray(u, dtype=dtype)
        p = np.ascontiguousarray(p if p is not None else np.zeros(0), dtype=dtype)
        assert u.shape == (self.dim,) and p.shape == (self.pdim,)
        du = np.empty(self.dim, dtype=dtype)
        o = np.empty(self.n_out + 1, dtype=dtype)
        ab = np.empty(self.n_aggr + 1, dtype=dtype)
        fn(self.L, du.ctypes.data, u.ctypes.data, _ptr(p), o.ctypes.data, ab.ctypes.data)
        return du

    def rhs(self, u, p, dtype=np.float64):
        fn = self.lib.nd_oracle_rhs_f64 if dtype == np.float64 else self.lib.nd_oracle_rhs_f32
        return self._rhs(fn, dtype, u, p)

    def rhs_poly(self, u, p, dtype=np.float64):
        fn = self.lib.nd_oracle_rhs_poly_f64 if dtype == np.float64 else self.lib.nd_oracle_rhs_poly_f32
        return self._rhs(fn, dtype, u, p)

    def tsit5(self, u0, p, t0, t1, reltol=1e-8, abstol=1e-10, maxsteps=10_000_000, threaded=False):
        """Tsit5 from t0 to t1.  ``threaded`` runs the RHS and the stage updates on all host
        threads; the result has the same bits as the sequential solve."""
        u = np.array(u0, dtype=np.float64, copy=True)
        p = np.ascontiguousarray(p if p is not None else np.zeros(0), dtype=np.float64)
        st = Tsit5Stats()
        fn = self.lib.nd_oracle_tsit5_threaded if threaded else self.lib.nd_oracle_tsit5
        fn(self.L, u.ctypes.data, _ptr(p), t0, t1, reltol, abstol, maxsteps, C.byref(st))
        return u, st

    def abs_terms(self, u, p):
        """Σ|terms| per state entry of du: the scale against which rounding differences
        of a reordered sum are bounded (used for tolerance reporting)."""
        uo = np.asarray(u, dtype=np.float64)
        p = np.asarray(p if p is not None else np.zeros(0), dtype=np.float64)
        vk = int(self.vkind[0])
        ek = int(self.ekind[0]) if self.ne else E_DIFFUSION_UNIT
        dv = VDIM[vk]
        th = uo[::dv] if dv > 1 else uo
        vs, vd = th[self.src], th[self.dst]
        pe = p[self.nv * VPDIM[vk]:]
        if ek == E_DIFFUSION:
            y = pe * (vs - vd)
        elif ek == E_DIFFUSION_UNIT:
            y = vs - vd
        else:
            y = pe * np.sin(vs - vd)
        s = np.zeros(self.nv)
        np.add.at(s, self.src, np.abs(y))
        np.add.at(s, self.dst, np.abs(y))
        out = np.zeros(self.dim)
        if vk == V_SWING:
            pv = p[:3 * self.nv].reshape(-1, 3)
            out[1::2] = (s + np.abs(pv[:, 2]) + np.abs(pv[:, 1] * uo[1::2])) / np.abs(pv[:, 0])
            out[0::2] = np.abs(uo[1::2])
        elif vk == V_KURAMOTO:
            out[:] = s + np.abs(p[:self.nv])
        else:
            out[:] = s
        return out


def rosenbrock23(rhs, jac, u0, t0, t1, reltol, abstol, mass=None, max_steps=100_000):
    """Rosenbrock23 (Shampine & Reichelt 1997, ode23s) for M u' = rhs(u) with a diagonal mass
    matrix (None: identity), dense: W = M - h d J, d = 1/(2+√2), e32 = 6+√2;
    k1 = W⁻¹ f0, k2 = W⁻¹ (f(u + h/2 k1) - M k1) + k1, u1 = u + h k2,
    k3 = W⁻¹ (f(u1) - e32 (M k2 - f1) - 2 (M k1 - f0)), error h/6 (k1 - 2 k2 + k3) in the
    scaled RMS norm, step factor min(5, max(0.2, 0.9 err^(-1/3))), first step
    min(1e-3 (t1 - t0), 1e-2).  The restatement the GPU solver is checked against.
    Returns (u(t1), accepted steps, rejected steps)."""
    u = np.array(u0, dtype=np.float64, copy=True)
    n = u.size
    M = np.ones(n) if mass is None else np.broadcast_to(np.asarray(mass, dtype=np.float64), (n,))
    d, e32 = 1.0 / (2.0 + np.sqrt(2.0)), 6.0 + np.sqrt(2.0)
    f0 = rhs(u)
    t, dt = t0, min(1e-3 * (t1 - t0), 1e-2)
    na = nr = 0
    while t < t1 and na + nr < max_steps:
        if t + dt * (1 + 1e-12) > t1:
            dt = t1 - t
        W = np.diag(M) - dt * d * jac(u)
        k1 = np.linalg.solve(W, f0)
        f1 = rhs(u + 0.5 * dt * k1)
        k2 = np.linalg.solve(W, f1 - M * k1) + k1
        u1 = u + dt * k2
        f2 = rhs(u1)
        k3 = np.linalg.solve(W, f2 - e32 * (M * k2 - f1) - 2.0 * (M * k1 - f0))
        err = dt / 6.0 * (k1 - 2.0 * k2 + k3)
        E = np.sqrt(np.mean((err / (abstol + reltol * np.maximum(np.abs(u), np.abs(u1)))) ** 2))
        if not E == E:
            E = 1e10
        fac = min(5.0, max(0.2, 0.9 * max(E, 1e-10) ** (-1.0 / 3.0)))
        if E <= 1.0:
            t = t1 if abs(t1 - (t + dt)) <= 1e-14 * max(1.0, abs(t1)) else t + dt
            u, f0 = u1, f2
            na += 1
        else:
            nr += 1
        dt *= fac
    return u, na, nr


# Rodas4 (Hairer & Wanner, Solving ODEs II, section VI.4; the RODAS code's first method),
# in the transformed variables that need no matrix-vector product with J: gamma, the stage
# coefficients a_ij (applied to the k's) and C_ij (divided by h), and the stiffly accurate
# solution u5 + k5 + k6 with the embedded error estimate k6.
RODAS4_GAMMA = 0.25
RODAS4_A = ((), (1.544,), (0.9466785280815826, 0.2557011698983284),
            (3.314825187068521, 2.896124015972201, 0.9986419139977817),
            (1.221224509226641, 6.019134481288629, 12.53708332932087, -0.6878860361058950))
RODAS4_C = ((), (-5.6688,), (-2.430093356833875, -0.2063599157091915),
            (-0.1073529058151375, -9.594562251023355, -20.47028614809616),
            (7.496443313967647, -10.24680431464352, -33.99990352819905, 11.70890893206160),
            (8.083246795921522, -7.981132988064893, -31.52159432874371, 16.31930543123136, -6.058818238834054))


def rodas4_step(rhs, jac, u, f0, dt, M):
    """One Rodas4 step of M u' = rhs(u) (autonomous, diagonal M): returns (u_new, err, f at
    u_new is not evaluated).  W = M/(h γ) - J; k_i = W⁻¹ (f(U_i) + M Σ_j C_ij k_j / h) with
    U_1 = u, U_i = u + Σ_j a_ij k_j (i <= 5), U_6 = U_5 + k_5; u_new = U_6 + k_6, err = k_6."""
    W = np.diag(M / (dt * RODAS4_GAMMA)) - jac(u)
    ks = []
    U = u
    for i in range(6):
        if i == 0:
            f = f0
        else:
            if i < 5:
                U = u + sum(a * k for a, k in zip(RODAS4_A[i], ks))
            else:
                U = U + ks[4]
            f = rhs(U)
        b = f + M * sum(c * k for c, k in zip(RODAS4_C[i], ks)) / dt if i else f
        ks.append(np.linalg.solve(W, b))
    return U + ks[5], ks[5]


def rodas4(rhs, jac, u0, t0, t1, reltol, abstol, mass=None, max_steps=100_000, fixed_dt=None):
    """Rodas4 for M u' = rhs(u) with a diagonal mass matrix (None: identity), dense.  Error
    in the scaled RMS norm of k6 against abstol + reltol max(|u|, |u_new|); step factor
    min(6, max(0.2, 0.9 err^(-1/4))); first step min(1e-3 (t1 - t0), 1e-2).  fixed_dt
    takes steps of that size, accepting every one (for convergence-order checks).  The
    restatement the GPU solver is checked against.  Returns (u(t1), accepted, rejected)."""
    u = np.array(u0, dtype=np.float64, copy=True)
    n = u.size
    M = np.ones(n) if mass is None else np.broadcast_to(np.asarray(mass, dtype=np.float64), (n,))
    f0 = rhs(u)
    t = t0
    dt = fixed_dt if fixed_dt else min(1e-3 * (t1 - t0), 1e-2)
    na = nr = 0
    while t < t1 and na + nr < max_steps:
        if t + dt * (1 + 1e-12) > t1:
            dt = t1 - t
        u1, err = rodas4_step(rhs, jac, u, f0, dt, M)
        E = np.sqrt(np.mean((err / (abstol + reltol * np.maximum(np.abs(u), np.abs(u1)))) ** 2))
        if not E == E:
            E = 1e10
        if fixed_dt or E <= 1.0:
            t = t1 if abs(t1 - (t + dt)) <= 1e-14 * max(1.0, abs(t1)) else t + dt
            u = u1
            f0 = rhs(u)
            na += 1
        else:
            nr += 1
        if not fixed_dt:
            dt *= min(6.0, max(0.2, 0.9 * max(E, 1e-10) ** (-0.25)))
    return u, na, nr


def rhs_numpy(nv, src, dst, vk, ek, u, p, dtype=np.float64):
    """Independent numpy restatement of the sequential RHS for one homogeneous batch."""
    src = np.asarray(src, dtype=np.int64)
    dst = np.asarray(dst, dtype=np.int64)
    ne = src.shape[0]
    u = np.asarray(u, dtype=dtype)
    p = np.asarray(p if p is not None else np.zeros(0), dtype=dtype)
    dv, pv = VDIM[vk], VPDIM[vk]
    o_v = u[::dv].copy()                              # vertex g: StateMask(1)
    vs, vd = o_v[src], o_v[dst]
    pe = p[nv * pv:]
    if ek == E_DIFFUSION:
        y = pe * (vs - vd)
    elif ek == E_DIFFUSION_UNIT:
        y = vs - vd
    else:
        y = pe * (np.sin(vs - vd) if dtype == np.float64 else np.sin(vs - vd).astype(dtype))
    # output buffer order per edge: src slot, then dst slot (AntiSymmetric: y_src = -y_dst)
    vals = np.empty(2 * ne, dtype=dtype)
    vals[0::2] = -y
    vals[1::2] = y
    targets = np.empty(2 * ne, dtype=np.int64)
    targets[0::2] = src
    targets[1::2] = dst
    agg = np.zeros(nv, dtype=dtype)
    np.add.at(agg, targets, vals)                     # SequentialAggregator order
    du = np.zeros(nv * dv, dtype=dtype)
    if vk == V_DIFFUSION:
        du[:] = agg
    elif vk == V_KURAMOTO:
        du[:] = p[:nv] + agg
    else:
        P = p[:3 * nv].reshape(-1, 3)
        M, D, Pm = P[:, 0], P[:, 1], P[:, 2]
        w = u[1::2]
        du[0::2] = w
        du[1::2] = dtype(1) / M * (Pm - D * w + agg)
    return du


def layout_batched(nv, src, dst, vertex_batches, vertex_batch, edge_batches, edge_batch):
    """Flat layout of a batched network (src/network_structure.jl:224-258), restated in
    numpy: vertex batches then edge batches, components ascending inside a batch.
    Returns the per-component first state / parameter indices and the edge order."""
    vb = np.asarray(vertex_batch)
    eb = np.asarray(edge_batch) if len(src) else np.zeros(0, dtype=np.int64)
    vorder = np.concatenate([np.flatnonzero(vb == b) for b in range(len(vertex_batches))])
    eorder = (np.concatenate([np.flatnonzero(eb == b) for b in range(len(edge_batches))])
              if len(edge_batches) else np.zeros(0, dtype=np.int64))
    v_data = np.zeros(nv, dtype=np.int64)
    v_para = np.zeros(nv, dtype=np.int64)
    e_data = np.zeros(len(src), dtype=np.int64)
    e_para = np.zeros(len(src), dtype=np.int64)
    st = par = 0
    for v in vorder:
        k = vertex_batches[vb[v]]
        v_data[v], v_para[v] = st, par
        st += VDIM[k]
        par += VPDIM[k]
    for e in eorder:
        k = edge_batches[eb[e]][0]
        e_data[e], e_para[e] = st, par
        st += EDIM[k]
        par += EPDIM[k]
    return dict(v_data=v_data, v_para=v_para, e_data=e_data, e_para=e_para, eorder=eorder, dim=st, pdim=par)


def rhs_numpy_batched(nv, src, dst, vertex_batches, vertex_batch, edge_batches, edge_batch, u, p,
                      dtype=np.float64, vertex_constants=None):
    """Independent numpy restatement of the sequential RHS of a batched network (several
    vertex / edge batches, ODE edges, Symmetric / Directed / Fiducial outputs)."""
    src = np.asarray(src, dtype=np.int64)
    dst = np.asarray(dst, dtype=np.int64)
    L = layout_batched(nv, src, dst, vertex_batches, vertex_batch, edge_batches, edge_batch)
    u = np.asarray(u, dtype=dtype)
    p = np.asarray(p if p is not None else np.zeros(0), dtype=dtype)
    sin = (lambda x: np.sin(x)) if dtype == np.float64 else (lambda x: np.sin(x).astype(dtype))
    du = np.zeros(L["dim"], dtype=dtype)
    if any(k in (V_PQ, V_GENERATOR, V_PQ_CONST) for k in vertex_batches):
        return _rhs_numpy_powergrid(nv, src, dst, vertex_batches, vertex_batch, edge_batches, edge_batch, u, p, L,
                                    du, vertex_constants)
    ov = u[L["v_data"]]                                # vertex g: StateMask(1)
    eo = L["eorder"]
    eb = np.asarray(edge_batch, dtype=np.int64)
    ne = len(src)
    ysrc = np.zeros(ne, dtype=dtype)
    ydst = np.zeros(ne, dtype=dtype)
    for b, (k, c) in enumerate(edge_batches):
        es = np.flatnonzero(eb == b)
        vs, vd = ov[src[es]], ov[dst[es]]
        if k in (E_DIFFUSION_ODE, E_DIFFUSION_ODE_FIXED):
            x0, x1 = u[L["e_data"][es]], u[L["e_data"][es] + 1]
            rate = dtype(1) / p[L["e_para"][es]] if k == E_DIFFUSION_ODE else dtype(100.0)
            du[L["e_data"][es]] = rate * (sin(vs - vd) - x0)
            du[L["e_data"][es] + 1] = rate * (sin(vd - vs) - x1)
            ydst[es], ysrc[es] = x0, x1                # Fiducial(dst=1:1, src=2:2)
            continue
        w = p[L["e_para"][es]] if EPDIM[k] else None
        y = (w * (vs - vd) if k == E_DIFFUSION else (vs - vd) if k == E_DIFFUSION_UNIT else w * sin(vs - vd))
        ydst[es] = y
        ysrc[es] = y if c == C_SYMMETRIC else (np.zeros_like(y) if c == C_DIRECTED else -y)
    # output buffer: per edge in batch order, src slot then dst slot; SequentialAggregator
    vals = np.empty(2 * ne, dtype=dtype)
    vals[0::2], vals[1::2] = ysrc[eo], ydst[eo]
    tg = np.empty(2 * ne, dtype=np.int64)
    tg[0::2], tg[1::2] = src[eo], dst[eo]
    agg = np.zeros(nv, dtype=dtype)
    np.add.at(agg, tg, vals)
    vbatch = np.asarray(vertex_batch)
    for b, k in enumerate(vertex_batches):
        vs_ = np.flatnonzero(vbatch == b)
        s, q, a = L["v_data"][vs_], L["v_para"][vs_], agg[vs_]
        if k == V_DIFFUSION:
            du[s] = a
        elif k == V_KURAMOTO:
            du[s] = p[q] + a
        elif k == V_SWING:
            w = u[s + 1]
            du[s] = w
            du[s + 1] = dtype(1) / p[q] * (p[q + 2] - p[q + 1] * w + a)
        else:
            w = u[s + 1]
            du[s] = w
            du[s + 1] = (p[q].astype(np.float64) - 1.0 * w.astype(np.float64)).astype(dtype) + a
    return du


def _rhs_numpy_powergrid(nv, src, dst, vertex_batches, vertex_batch, edge_batches, edge_batch, u, p, L, du,
                         vertex_constants=None):
    """The power-grid components (benchmark/benchmark_models.jl:46-109) in numpy complex
    arithmetic: vertex outputs and edge outputs are complex numbers (depth 2)."""
    v_data, v_para, e_para = L["v_data"], L["v_para"], L["e_para"]
    V = u[v_data] + 1j * u[v_data + 1]                 # StateMask(1:2)
    w = 2 * np.pi * 50
    ne = len(src)
    isrc = np.zeros(ne, dtype=np.complex128)
    idst = np.zeros(ne, dtype=np.complex128)
    eb = np.asarray(edge_batch, dtype=np.int64)
    for b, (k, c) in enumerate(edge_batches):
        assert k == E_PILINE
        es = np.flatnonzero(eb == b)
        Lh, R, C1, C2 = (p[e_para[es] + j] for j in range(4))
        Vs, Vd = V[src[es]], V[dst[es]]
        imain = (Vs - Vd) / (R + 1j * w * Lh)
        i_src = -(imain + Vs * 1j * w * C1)
        i_dst = imain - Vd * 1j * w * C2
        isrc[es], idst[es] = -i_src, -i_dst
    eo = L["eorder"]
    vals = np.empty(2 * ne, dtype=np.complex128)
    vals[0::2], vals[1::2] = isrc[eo], idst[eo]
    tg = np.empty(2 * ne, dtype=np.int64)
    tg[0::2], tg[1::2] = src[eo], dst[eo]
    re, im = np.zeros(nv), np.zeros(nv)                # SequentialAggregator, per component
    np.add.at(re, tg, vals.real)
    np.add.at(im, tg, vals.imag)
    isum = re + 1j * im
    vbatch = np.asarray(vertex_batch)
    for b, k in enumerate(vertex_batches):
        vs = np.flatnonzero(vbatch == b)
        s, q, i = v_data[vs], v_para[vs], isum[vs]
        if k in (V_PQ, V_PQ_CONST):
            S = (p[q] + 1j * p[q + 1]) if k == V_PQ else complex(*np.asarray(vertex_constants).reshape(-1, 2)[b])
            uc = S / np.conj(i)
            du[s], du[s + 1] = uc.real, uc.imag
            continue
        assert k == V_GENERATOR
        H, P, D, Om, E_f, T_d_dash, T_q_dash, X_q_dash, X_d_dash, X_d, X_q = (p[q + j] for j in range(11))
        uc = u[s] + 1j * u[s + 1]
        th, om = u[s + 2], u[s + 3]
        i_c = 1j * i * np.exp(-1j * th)
        e_c = 1j * uc * np.exp(-1j * th)
        pw = (uc * np.conj(i)).real
        de_d = (1 / T_q_dash) * (-e_c.real + (X_q - X_q_dash) * i_c.imag)
        de_q = (1 / T_d_dash) * (-e_c.imag - (X_d - X_d_dash) * i_c.real + E_f)
        dU = -1j * (de_d + 1j * de_q) * np.exp(1j * th) + uc * 1j * om
        du[s], du[s + 1], du[s + 2] = dU.real, dU.imag, om
        du[s + 3] = (P - D * om - pw - (X_q_dash - X_d_dash) * i_c.real * i_c.imag) * (Om / (2 * H))
    return du


def swing_residual_theta(theta, src, dst, K, P):
    """Power balance P_i + Σ_in K sin(θ_src-θ_dst) (with AntiSymmetric signs) at ω = 0."""
    y = K * np.sin(theta[src] - theta[dst])
    r = P.copy()
    np.add.at(r, dst, y)
    np.add.at(r, src, -y)
    return r


def newton_fixpoint(nv, src, dst, K, P, theta0=None, tol=1e-10, maxiter=50):
    """Dense Newton on the swing / first-order Kuramoto steady state with ω = 0.

    The state is θ; the Jacobian of the power balance is a weighted graph Laplacian with
    weights K cos(θ_src - θ_dst), singular along the uniform phase shift, so θ_0 is pinned
    (the gauge).  Returns (θ, iterations, final max-norm residual)."""
    src = np.asarray(src)
    dst = np.asarray(dst)
    th = np.zeros(nv) if theta0 is None else np.array(theta0, dtype=np.float64)
    th = th - th[0]
    it = 0
    res = np.max(np.abs(swing_residual_theta(th, src, dst, K, P)))
    while res > tol and it < maxiter:
        w = K * np.cos(th[src] - th[dst])
        J = np.zeros((nv, nv))
        # r_dst += K sin(θs-θd): ∂/∂θs = w, ∂/∂θd = -w ; r_src -= ...: ∂/∂θs = -w, ∂/∂θd = w
        np.add.at(J, (dst, src), w)
        np.add.at(J, (dst, dst), -w)
        np.add.at(J, (src, src), -w)
        np.add.at(J, (src, dst), w)
        r = swing_residual_theta(th, src, dst, K, P)
        delta = np.zeros(nv)
        delta[1:] = np.linalg.solve(J[1:, 1:], -r[1:])
        th = th + delta
        it += 1
        res = np.max(np.abs(swing_residual_theta(th, src, dst, K, P)))
    return th, it, res


def collect_externals(from_state, idx, u, o):
    """The ExtMap gather collect_externals! (src/external_inputs.jl:51-64, CPU loop):
    entry k reads u[idx[k]] for a StateBufIdx, o[idx[k]] for an OutBufIdx.  0-based."""
    ext = np.empty(len(idx), dtype=np.result_type(u, o))
    for k, (st, i) in enumerate(zip(from_state, idx)):
        ext[k] = u[i] if st else o[i]
    return ext


def gen_loopback_map(src, dst, loopback, v_out, v_aggr):
    """gen_loopback_map (src/post_utils.jl:213-224): for each loopback edge in edge order,
    the destination vertex's output indices and the source vertex's aggregation indices,
    appended range by range.  v_out[v] / v_aggr[v] are index sequences (0-based)."""
    out_idx, agg_idx = [], []
    for e in range(len(src)):
        if not loopback[e]:
            continue
        out_idx.extend(v_out[dst[e]])
        agg_idx.extend(v_aggr[src[e]])
    return np.asarray(out_idx, dtype=np.int64), np.asarray(agg_idx, dtype=np.int64)


def apply_loopback(aggbuf, obuf, out_idx, agg_idx):
    """_apply_loopback! on the CPU (src/post_utils.jl:230-236): aggbuf[agg] = obuf[out] in
    map order (a later entry wins where agg repeats)."""
    agg = np.array(aggbuf, copy=True)
    for oi, ai in zip(out_idx, agg_idx):
        agg[ai] = obuf[oi]
    return agg
