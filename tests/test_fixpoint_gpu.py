"""find_fixpoint on the GPU for any network of output dimension 1: Newton with restarted
GMRES on the sparse Jacobian (nd_find_fixpoint), against known answers, the oracle's dense
Newton and the oracle RHS at the solution.  The reference solves the same
SteadyStateProblem with NonlinearSolve (src/initialization.jl:44-144) and raises
NetworkInitError when it fails or the RHS gives NaN."""
import numpy as np
import pytest

import nd_gb300 as nd
from nd_gb300 import _capi as capi
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def adapt(net):
    import torch
    return nd.adapt(net, torch.float64)


def test_reference_swing_network_both_solvers(cuda):
    """The 4-node swing network of test/initialization_test.jl:15-38 (K = 6, P = ±1):
    neighbouring phases differ by asin(1/12), with either solver."""
    g4 = nd.cycle_graph(4)
    net = nd.Network(g4, nd.kuramoto_second(), nd.static_line())
    P = np.array([1.0, -1.0, 1.0, -1.0])
    p = np.concatenate([np.stack([np.ones(4), np.full(4, 0.1), P], 1).ravel(), np.full(4, 6.0)])
    u = nd.find_fixpoint(adapt(net), p, alg="newton_gmres").cpu().numpy()
    np.testing.assert_allclose(np.abs(np.diff(u[0::2])), np.arcsin(1 / 12), atol=1e-11)
    assert np.max(np.abs(u[1::2])) <= 1e-10
    on = O.OracleNetwork.from_graph(g4, O.V_SWING, O.E_KURAMOTO)
    assert np.max(np.abs(on.rhs(u, p))) <= 1e-10
    u_swing = nd.find_fixpoint(net, p).cpu().numpy()
    np.testing.assert_allclose(np.diff(u[0::2]), np.diff(u_swing[0::2]), atol=1e-11)


def test_kuramoto_matches_dense_newton(cuda):
    """First-order Kuramoto with zero-sum natural frequencies: the phase differences along
    every edge agree with the oracle's dense Newton (the phases are fixed up to a shift)."""
    g = nd.watts_strogatz(300, 6, 0.2, seed=2)
    rng = np.random.default_rng(2)
    om = rng.uniform(-1, 1, g.nv)
    om -= om.mean()
    K = rng.uniform(4, 6, g.ne)
    net = nd.Network(g, nd.kuramoto_first(), nd.kuramoto_edge())
    p = np.concatenate([om, K])
    u = nd.find_fixpoint(adapt(net), p).cpu().numpy()
    st = nd.find_fixpoint.last_stats
    assert st["resid"] <= 1e-10 and 1 <= st["newton_iters"] <= 20
    th, it, res = O.newton_fixpoint(g.nv, g.src, g.dst, K, om)
    assert res <= 1e-10
    np.testing.assert_allclose(u[g.src] - u[g.dst], th[g.src] - th[g.dst], atol=1e-9)
    on = O.OracleNetwork.from_graph(g, O.V_KURAMOTO, O.E_KURAMOTO)
    assert np.max(np.abs(on.rhs(u, p))) <= 1e-10


def test_diffusion_converges_to_the_weighted_mean(cuda):
    """du = -L u: every consensus state is a fixpoint.  The Newton step from u0 lies in
    D^-1 range(L) (GMRES from 0, right-preconditioned by the diagonal D of the weighted
    Laplacian), which keeps Σ d_i u_i: the solve lands on the degree-weighted mean of u0."""
    g = nd.barabasi_albert(2000, 3, seed=5)
    net = nd.Network(g, nd.diffusion_vertex(), nd.diffusion_edge())
    rng = np.random.default_rng(5)
    u0 = rng.normal(size=g.nv)
    w = rng.uniform(0.5, 1.5, g.ne)
    u = nd.find_fixpoint(adapt(net), w, x0=u0).cpu().numpy()
    d = np.bincount(g.src, weights=w, minlength=g.nv) + np.bincount(g.dst, weights=w, minlength=g.nv)
    np.testing.assert_allclose(u, (d * u0).sum() / d.sum(), atol=1e-9)


def test_batched_network_with_ode_edges(cuda):
    """Kuramoto vertices with ODE edges: at the fixpoint the edge states equal the sine
    couplings and the oracle RHS vanishes."""
    g = nd.watts_strogatz(200, 4, 0.3, seed=7)
    rng = np.random.default_rng(7)
    kinds = rng.integers(0, 2, g.ne)
    em = [nd.diffusion_odeedge() if k else nd.kuramoto_edge() for k in kinds]
    net = nd.Network(g, nd.kuramoto_first(), em)
    om = rng.uniform(-0.5, 0.5, g.nv)
    om -= om.mean()
    p = net.pflat(vertex={"ω": om}, edge={"τ": 0.5, "K": 3.0})
    u = nd.find_fixpoint(adapt(net), p).cpu().numpy()
    eb = [(m.kind, capi.COUPLINGS[m.coupling]) for m in net.edge_batches]
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, [O.V_KURAMOTO], net.vertex_batch, eb, net.edge_batch)
    assert np.max(np.abs(on.rhs(u, p))) <= 1e-10
    ode = np.flatnonzero(kinds)
    th = u[:g.nv]
    e1 = u[net.e_data[ode]]
    np.testing.assert_allclose(e1, np.sin(th[g.src[ode]] - th[g.dst[ode]]), atol=1e-10)


def test_failures_raise(cuda):
    """No fixpoint (frequencies that do not sum to zero) and NaN in the parameters raise."""
    g = nd.cycle_graph(20)
    net = adapt(nd.Network(g, nd.kuramoto_first(), nd.kuramoto_edge()))
    p = np.concatenate([np.full(20, 0.3), np.full(20, 2.0)])
    with pytest.raises(nd.NotConvergedError):
        nd.find_fixpoint(net, p, max_newton=15)
    p_nan = np.concatenate([np.zeros(20), np.full(20, 2.0)])
    p_nan[3] = np.nan
    with pytest.raises(nd.NotConvergedError, match="NaN"):
        nd.find_fixpoint(net, p_nan)
