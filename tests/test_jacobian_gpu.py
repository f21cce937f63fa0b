"""The sparse Jacobian on the GPU: its pattern against the dependencies the oracle RHS
actually has (the reference checks its traced pattern against a ForwardDiff Jacobian the
same way, _assert_conservative_pattern in ext/NetworkDynamicsSparsityExt.jl), its values
against central differences of the oracle, against the analytic JVP, and against the
Laplacian for diffusion."""
import numpy as np
import pytest

import nd_gb300 as nd
from nd_gb300 import _capi as capi
from oracle import oracle as O

from ndtest import fd_jacobian
from test_batched_gpu import ALL_EDGES, VKINDS, build

pytestmark = pytest.mark.gpu


def dense(nw, u, p, cuda, dtype):
    import torch
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    ut = torch.from_numpy(np.asarray(u, dtype=dtype)).to(cuda)
    pt = torch.from_numpy(np.asarray(p, dtype=dtype)).to(cuda) if len(p) else None
    J = nd.jacobian(nw, ut, pt)
    return J.to_dense().cpu().numpy().astype(np.float64)


def pattern_dense(nw):
    rowptr, colidx = nd.jacobian_pattern(nw)
    P = np.zeros((nw.dim, nw.dim), dtype=bool)
    for i in range(nw.dim):
        cols = colidx[rowptr[i]:rowptr[i + 1]]
        assert np.all(np.diff(cols) > 0)  # sorted, unique
        P[i, cols] = True
    return P


def check(nw_host, on, u, p, cuda):
    import torch
    nw = nd.adapt(nw_host, torch.float64)
    fd = fd_jacobian(on, u, p)
    P = pattern_dense(nw)
    # conservative: every dependency the RHS has is in the pattern ...
    assert not (fd != 0)[~P].any()
    J = dense(nw, u, p, cuda, np.float64)
    assert not J[~P].any()
    # ... and an entry the finite differences see as exactly zero is one whose derivatives
    # cancel (e.g. an own-output column reached through edges of opposite signs)
    assert np.abs(J[P & (fd == 0)]).max(initial=0.0) <= 1e-12
    assert (P & (fd == 0)).sum() <= max(2, P.sum() // 1000)
    np.testing.assert_allclose(J, fd, rtol=1e-6, atol=1e-7)
    J32 = dense(nd.adapt(nw_host, torch.float32), u, p, cuda, np.float32)
    np.testing.assert_allclose(J32, J, rtol=1e-5, atol=1e-5 * np.abs(J).max())
    return nw, J


def test_reference_gpu_test_network(cuda):
    g = nd.complete_graph(4)
    vf = [nd.kuramoto_second(), nd.diffusion_vertex(), nd.kuramoto_second(), nd.diffusion_vertex()]
    ef = [nd.diffusion_odeedge(), nd.kuramoto_edge(), nd.kuramoto_edge(), nd.diffusion_edge_fid(),
          nd.diffusion_odeedge(), nd.diffusion_edge_fid()]
    net = nd.Network(g, vf, ef)
    vb = [m.kind for m in net.vertex_batches]
    eb = [(m.kind, capi.COUPLINGS[m.coupling]) for m in net.edge_batches]
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, net.vertex_batch, eb, net.edge_batch)
    rng = np.random.default_rng(1)
    check(net, on, rng.random(net.dim), rng.random(net.pdim) + 0.5, cuda)


@pytest.mark.parametrize("seed", [0, 1])
def test_random_batched_network(cuda, seed):
    g = nd.barabasi_albert(200, 3, seed=seed)
    rng = np.random.default_rng(seed)
    net, on = build(g, VKINDS, ALL_EDGES, vassign=rng.integers(0, 4, g.nv),
                    eassign=rng.integers(0, len(ALL_EDGES), g.ne))
    check(net, on, rng.normal(size=net.dim), rng.uniform(0.5, 1.5, size=net.pdim), cuda)


@pytest.mark.parametrize("vm,em,vk,ek", [(nd.kuramoto_second, nd.static_line, O.V_SWING, O.E_KURAMOTO),
                                         (nd.kuramoto_first, nd.diffusion_edge, O.V_KURAMOTO, O.E_DIFFUSION)])
def test_homogeneous_networks(cuda, vm, em, vk, ek):
    g = nd.watts_strogatz(150, 6, 0.2, seed=3)
    net = nd.Network(g, vm(), em())
    on = O.OracleNetwork.from_graph(g, vk, ek)
    rng = np.random.default_rng(3)
    check(net, on, rng.normal(size=net.dim), rng.uniform(0.5, 1.5, size=net.pdim), cuda)


def test_diffusion_jacobian_is_minus_laplacian(cuda):
    """du = -L x (test/diffusion_test.jl:80-90), so ∂f/∂u = -L exactly."""
    import torch
    g = nd.barabasi_albert(500, 4, seed=9)
    nw = nd.adapt(nd.Network(g, nd.diffusion_vertex(), nd.diffusion_edge_unit()), torch.float64)
    u = np.random.default_rng(9).normal(size=g.nv)
    np.testing.assert_array_equal(dense(nw, u, np.zeros(0), cuda, np.float64), -g.laplacian())


def test_jacobian_times_vector_equals_jvp(cuda):
    """Large swing network: the assembled Jacobian times v against nd_jvp (both analytic)."""
    import torch
    g = nd.barabasi_albert(100_000, 2, seed=4)
    net = nd.Network(g, nd.kuramoto_second(), nd.static_line())
    nw = nd.adapt(net, torch.float64)
    rng = np.random.default_rng(4)
    u = torch.from_numpy(rng.normal(size=nw.dim)).cuda()
    p = torch.from_numpy(net.pflat(vertex={"Pm": rng.normal(size=g.nv)}, edge={"K": rng.uniform(5, 10, g.ne)})).cuda()
    v = torch.from_numpy(rng.normal(size=nw.dim)).cuda()
    J = nd.jacobian(nw, u, p)
    rowptr, _ = nd.jacobian_pattern(nw)
    assert len(rowptr) == nw.dim + 1
    jv = torch.empty_like(u)
    nd.jvp(nw, jv, u, p, v)
    got = (J @ v.unsqueeze(1)).squeeze(1)
    scale = (J.abs() @ v.abs().unsqueeze(1)).squeeze(1)
    assert torch.all((got - jv).abs() <= 1e-13 * (scale + 1e-300)).item()


def test_directed_edges_leave_sources_out(cuda):
    """A Directed edge has no source output (y_src = 0), so a source row does not depend
    on it: on a directed path the Jacobian is strictly lower bidiagonal plus the diagonal."""
    import torch
    n = 8
    g = nd.Graph(n, np.arange(n - 1, dtype=np.int64), np.arange(1, n, dtype=np.int64))
    nw = nd.adapt(nd.Network(g, nd.diffusion_vertex(), nd.Directed(nd.diffusion_edge_unit())), torch.float64)
    J = dense(nw, np.arange(n, dtype=np.float64), np.zeros(0), cuda, np.float64)
    exp = np.zeros((n, n))
    for e in range(n - 1):
        exp[e + 1, e] += 1.0      # y_dst = u_src - u_dst
        exp[e + 1, e + 1] -= 1.0
    np.testing.assert_array_equal(J, exp)


@pytest.mark.parametrize("pq_only", [False, True])
def test_powergrid_jacobian(cuda, pq_only):
    """Power grids (PQ buses, generators, π-lines; complex outputs): the pattern holds every
    dependency of the oracle RHS and the dual-number values match its central differences,
    as for the networks with real outputs.  The reference covers power grids with its
    traced prototype (ext/NetworkDynamicsSparsityExt.jl:57-127) and ForwardDiff values."""
    import torch
    from test_batched_gpu import powergrid_network
    g, net, on = powergrid_network(40, 3, pq_only)
    rng = np.random.default_rng(9)
    p = net.pflat(vertex={"P": rng.uniform(-1, 1, g.nv), "Q": rng.uniform(-1, 1, g.nv), "H": 5.0, "D": 0.1,
                          "Ω": 2 * np.pi * 50, "E_f": 1.0, "T_d_dash": 7.0, "T_q_dash": 0.5, "X_d_dash": 0.3,
                          "X_q_dash": 0.6, "X_d": 1.8, "X_q": 1.7},
                  edge={"L": 1e-3, "R": 0.05, "C1": 1e-5, "C2": 1e-5})
    u = 1.0 + 0.1 * rng.normal(size=net.dim)
    nw = nd.adapt(net, torch.float64)
    fd = fd_jacobian(on, u, p)
    P = pattern_dense(nw)
    assert not (np.abs(fd) > 1e-9 * np.abs(fd).max())[~P].any()
    J = dense(nw, u, p, cuda, np.float64)
    assert not J[~P].any()
    np.testing.assert_allclose(J, fd, rtol=1e-5, atol=1e-7 * np.abs(fd).max())
    # the JVP of the network, through the assembled Jacobian
    v = rng.normal(size=net.dim)
    jv = torch.empty(net.dim, dtype=torch.float64, device=cuda)
    nd.jvp(nw, jv, torch.from_numpy(u).to(cuda), torch.from_numpy(p).to(cuda), torch.from_numpy(v).to(cuda))
    np.testing.assert_allclose(jv.cpu().numpy(), J @ v, rtol=1e-12, atol=1e-12 * np.abs(J).sum(1).max())
