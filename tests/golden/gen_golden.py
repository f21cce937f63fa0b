"""Generate the golden fixtures in this folder from the CPU oracle.

Each .npz holds a graph (0-based src/dst in edges(g) order), inputs and the oracle's
outputs.  The known answers they are checked against come from the reference's own tests:

* ``diffusion_ba10_5.npz``   du = -L·x for unit diffusion on a BA(10, 5) graph
                             (test/diffusion_test.jl:80-90), 30 random x.
* ``kuramoto_ws1000.npz``    first-order Kuramoto on WS(1000, 10, 0.1), ω ~ N(0,1), K = 3,
                             θ ~ U(-π, π): one RHS and the Tsit5 state at t = 10
                             (reltol 1e-8, abstol 1e-10).
* ``swing_ws4.npz``          the 4-node swing fixpoint of test/initialization_test.jl:15-38
                             (P = [1,-1,1,-1], K = 6 on watts_strogatz(4, 2, 0) = C4).
* ``swing_ba200.npz``        swing + static line on BA(200, 2): one RHS in F64 and F32.
* ``batched_gpu_test.npz``   the network of test/GPU_test.jl:12-21 (complete graph on 4
                             vertices; swing and diffusion vertices; ODE, Kuramoto and
                             two-sided fiducial edges) with its batches, x0, p ~ U(0, 1): one RHS.
* ``powergrid_ws300.npz``    PQ buses and generators with π-lines on WS(300, 4, 0.5): one RHS.

Run: python tests/golden/gen_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "networkdynamics.jl_gb300"))
sys.path.insert(0, str(ROOT))

import nd_gb300 as nd  # noqa: E402
from oracle import oracle as O  # noqa: E402


def main():
    rng = np.random.default_rng(42)

    g = nd.barabasi_albert(10, 5, seed=42)
    on = O.OracleNetwork.from_graph(g, O.V_DIFFUSION, O.E_DIFFUSION_UNIT)
    xs = rng.normal(size=(30, g.nv))
    dus = np.stack([on.rhs(x, None) for x in xs])
    np.savez(HERE / "diffusion_ba10_5.npz", nv=g.nv, src=g.src, dst=g.dst, x=xs, du=dus)

    g = nd.watts_strogatz(1000, 10, 0.1, seed=1)
    on = O.OracleNetwork.from_graph(g, O.V_KURAMOTO, O.E_KURAMOTO)
    theta = rng.uniform(-np.pi, np.pi, size=g.nv)
    omega = rng.normal(size=g.nv)
    p = np.concatenate([omega, np.full(g.ne, 3.0)])
    du = on.rhs(theta, p)
    uT, st = on.tsit5(theta, p, 0.0, 10.0, reltol=1e-8, abstol=1e-10)
    np.savez(HERE / "kuramoto_ws1000.npz", nv=g.nv, src=g.src, dst=g.dst, u=theta, p=p, du=du, u_t10=uT,
             naccept=st.naccept, nreject=st.nreject)

    g = nd.cycle_graph(4)
    P = np.array([1.0, -1.0, 1.0, -1.0])
    th, it, res = O.newton_fixpoint(4, g.src, g.dst, 6.0, P)
    np.savez(HERE / "swing_ws4.npz", nv=4, src=g.src, dst=g.dst, P=P, K=6.0, theta=th, iters=it, res=res)

    g = nd.barabasi_albert(200, 2, seed=7)
    on = O.OracleNetwork.from_graph(g, O.V_SWING, O.E_KURAMOTO)
    u = np.empty(on.dim)
    u[0::2] = rng.uniform(-np.pi, np.pi, size=g.nv)
    u[1::2] = rng.normal(size=g.nv)
    pv = np.stack([np.ones(g.nv), np.full(g.nv, 0.1), rng.uniform(-1.5, 1.5, size=g.nv)], axis=1).ravel()
    p = np.concatenate([pv, rng.uniform(5, 10, size=g.ne)])
    np.savez(HERE / "swing_ba200.npz", nv=g.nv, src=g.src, dst=g.dst, u=u, p=p, du=on.rhs(u, p),
             du32=on.rhs(u, p, dtype=np.float32))
    batched_fixtures()
    print("golden fixtures written to", HERE)


def batched_fixtures():
    rng = np.random.default_rng(7)
    g = nd.complete_graph(4)
    vb, vbi = [O.V_SWING, O.V_DIFFUSION], np.array([0, 1, 0, 1], dtype=np.int32)
    eb = np.array([(O.E_DIFFUSION_ODE, O.C_FIDUCIAL), (O.E_KURAMOTO, O.C_ANTISYMMETRIC),
                   (O.E_DIFFUSION, O.C_FIDUCIAL)], dtype=np.int32)
    ebi = np.array([0, 1, 1, 2, 0, 2], dtype=np.int32)
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, vbi, [tuple(x) for x in eb], ebi)
    x0, p = rng.random(on.dim), rng.random(on.pdim)
    np.savez(HERE / "batched_gpu_test.npz", nv=g.nv, src=g.src, dst=g.dst, vb=np.array(vb), vbi=vbi, eb=eb,
             ebi=ebi, u=x0, p=p, du=on.rhs(x0, p))

    g = nd.watts_strogatz(300, 4, 0.5, seed=3)
    kinds = rng.integers(0, 2, g.nv)
    order = list(dict.fromkeys(kinds.tolist()))
    vb = np.array([[O.V_PQ, O.V_GENERATOR][k] for k in order], dtype=np.int32)
    vbi = np.array([order.index(k) for k in kinds], dtype=np.int32)
    eb = np.array([(O.E_PILINE, O.C_FIDUCIAL)], dtype=np.int32)
    ebi = np.zeros(g.ne, dtype=np.int32)
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, vbi, [tuple(x) for x in eb], ebi)
    u, p = 1.0 + 0.1 * rng.normal(size=on.dim), rng.uniform(0.5, 1.5, size=on.pdim)
    np.savez(HERE / "powergrid_ws300.npz", nv=g.nv, src=g.src, dst=g.dst, vb=vb, vbi=vbi, eb=eb, ebi=ebi, u=u,
             p=p, du=on.rhs(u, p))


if __name__ == "__main__":
    main()
