"""Rosenbrock23 with a mass matrix on the GPU (nd_solve_rosenbrock23): the reference hands
networks with mass matrices (construct_mass_matrix, src/construction.jl:409-467) to SciML's
Rosenbrock solvers.  Checked against known answers: exp(-tL) x0 for diffusion
(test/diffusion_test.jl:119-129), the exact solution of the linear DAE obtained by
eliminating algebraic vertices, and the oracle's dense Rosenbrock23 restatement on a
nonlinear swing network."""
import dataclasses

import numpy as np
import pytest
import scipy.linalg

import nd_gb300 as nd
from nd_gb300.solve import solve_rodas4, solve_rosenbrock23
from oracle import oracle as O

from ndtest import random_inputs

pytestmark = pytest.mark.gpu


def test_diffusion_known_answer(cuda):
    import torch
    g = nd.barabasi_albert(40, 3, seed=42)
    L = g.laplacian()
    nw = nd.adapt(nd.Network(g, nd.diffusion_vertex(), nd.diffusion_edge_unit()), torch.float64)
    x0 = np.random.default_rng(3).normal(size=g.nv)
    for T in (0.5, 5.0):
        u, st = solve_rosenbrock23(nw, x0, None, (0.0, T), reltol=1e-6, abstol=1e-9)
        assert st.status == 0 and st.t_final == T and st.naccept > 0
        assert np.max(np.abs(u.cpu().numpy() - scipy.linalg.expm(-T * L) @ x0)) < 1e-5


def test_dae_with_algebraic_vertices(cuda):
    """Diffusion with every fifth vertex algebraic (mass_matrix = 0): such a vertex holds
    the weighted mean of its neighbours, 0 = Σ w (u_n - u_v).  The exact solution
    eliminates those vertices: x' = (A_xx - A_xz A_zz⁻¹ A_zx) x, z = -A_zz⁻¹ A_zx x."""
    import torch
    g = nd.watts_strogatz(60, 4, 0.2, seed=5)
    rng = np.random.default_rng(5)
    w = rng.uniform(0.5, 1.5, g.ne)
    alg = np.arange(g.nv) % 5 == 0
    vm = [dataclasses.replace(nd.diffusion_vertex(), mass_matrix=0) if a else nd.diffusion_vertex() for a in alg]
    net = nd.Network(g, vm, nd.diffusion_edge())
    mm = net.mass_matrix()
    idx = net.v_data  # state of each vertex (algebraic vertices form their own batch)
    assert np.all(mm[idx[alg]] == 0) and np.all(mm[idx[~alg]] == 1)
    # A = -L_w in vertex order
    A = np.zeros((g.nv, g.nv))
    for e, (s, d) in enumerate(zip(g.src, g.dst)):
        A[s, d] += w[e]
        A[d, s] += w[e]
        A[s, s] -= w[e]
        A[d, d] -= w[e]
    X, Z = np.nonzero(~alg)[0], np.nonzero(alg)[0]
    Azz_inv_Azx = np.linalg.solve(A[np.ix_(Z, Z)], A[np.ix_(Z, X)])
    S = A[np.ix_(X, X)] - A[np.ix_(X, Z)] @ Azz_inv_Azx
    x0 = rng.normal(size=len(X))
    v0 = np.zeros(g.nv)
    v0[X] = x0
    v0[Z] = -Azz_inv_Azx @ x0  # consistent algebraic values
    u0 = np.empty(net.dim)
    u0[idx] = v0
    nw = nd.adapt(net, torch.float64)
    T = 2.0
    u, st = solve_rosenbrock23(nw, u0, w, (0.0, T), reltol=1e-6, abstol=1e-9)
    assert st.status == 0 and st.t_final == T
    got = u.cpu().numpy()[idx]
    xT = scipy.linalg.expm(S * T) @ x0
    np.testing.assert_allclose(got[X], xT, atol=1e-5)
    np.testing.assert_allclose(got[Z], -Azz_inv_Azx @ xT, atol=1e-5)
    # identity mass matrix given explicitly: the algebraic vertices then move
    u2, _ = solve_rosenbrock23(nw, u0, w, (0.0, T), mass_matrix=None, reltol=1e-6, abstol=1e-9)
    assert np.max(np.abs(u2.cpu().numpy()[idx][Z] - got[Z])) > 1e-3


def test_swing_against_oracle_rosenbrock(cuda):
    """A nonlinear network (swing on BA(100, 2), identity mass matrix) against the oracle's
    dense Rosenbrock23 restatement driven by the oracle RHS and its central-difference
    Jacobian: the same step sequence (within 2) and the same end state.  Rosenbrock23 is of
    order 2, so both sit ~N_steps · tol from the exact solution; the oracle's Tsit5 at
    1e-10 checks that distance."""
    import torch
    from ndtest import fd_jacobian
    g = nd.barabasi_albert(100, 2, seed=6)
    on = O.OracleNetwork.from_graph(g, O.V_SWING, O.E_KURAMOTO)
    u0, p = random_inputs(on, O.V_SWING, np.random.default_rng(6))
    u0[0::2] *= 0.1
    u0[1::2] = 0.0
    nw = nd.adapt(nd.Network(g, nd.kuramoto_second(), nd.static_line()), torch.float64)
    u, st = solve_rosenbrock23(nw, u0, p, (0.0, 0.5), reltol=1e-7, abstol=1e-9)
    ref, na, nr = O.rosenbrock23(lambda x: on.rhs(x, p), lambda x: fd_jacobian(on, x, p), u0, 0.0, 0.5, 1e-7, 1e-9)
    assert st.status == 0 and st.t_final == 0.5
    assert abs(st.naccept - na) <= 2 and abs(st.nreject - nr) <= 2
    np.testing.assert_allclose(u.cpu().numpy(), ref, atol=1e-8, rtol=0)
    exact, rst = on.tsit5(u0, p, 0.0, 0.5, reltol=1e-10, abstol=1e-12)
    assert np.max(np.abs(u.cpu().numpy() - exact)) <= 1e4 * 1e-7 * max(1.0, np.abs(exact).max())


def test_rosenbrock_rejects_bad_arguments(cuda):
    import torch
    g = nd.cycle_graph(5)
    net = nd.Network(g, nd.diffusion_vertex(), nd.diffusion_edge_unit())
    with pytest.raises(nd.ArgumentError):
        solve_rosenbrock23(nd.adapt(net, torch.float32), np.zeros(5), None, (0.0, 1.0))
    nw = nd.adapt(net, torch.float64)
    with pytest.raises(nd.ArgumentError):
        solve_rosenbrock23(nw, np.zeros(5), None, (1.0, 0.0))
    with pytest.raises(nd.NotConvergedError):
        solve_rosenbrock23(nw, np.arange(5.0), None, (0.0, 100.0), reltol=1e-12, abstol=1e-14, max_steps=3)


def test_rodas4_diffusion_and_dae_known_answers(cuda):
    """Rodas4 on the GPU: exp(-tL) x0 for diffusion, and the eliminated solution of the
    linear DAE with algebraic vertices, at a tight tolerance where it needs far fewer steps
    than Rosenbrock23 (order 4 against 2)."""
    import torch
    g = nd.barabasi_albert(40, 3, seed=42)
    L = g.laplacian()
    nw = nd.adapt(nd.Network(g, nd.diffusion_vertex(), nd.diffusion_edge_unit()), torch.float64)
    x0 = np.random.default_rng(3).normal(size=g.nv)
    u, st = solve_rodas4(nw, x0, None, (0.0, 5.0), reltol=1e-8, abstol=1e-10)
    assert st.status == 0 and st.t_final == 5.0
    assert np.max(np.abs(u.cpu().numpy() - scipy.linalg.expm(-5.0 * L) @ x0)) < 1e-7
    _, st23 = solve_rosenbrock23(nw, x0, None, (0.0, 5.0), reltol=1e-8, abstol=1e-10)
    assert 4 * st.naccept < st23.naccept
    # the DAE of test_dae_with_algebraic_vertices
    g = nd.watts_strogatz(60, 4, 0.2, seed=5)
    rng = np.random.default_rng(5)
    w = rng.uniform(0.5, 1.5, g.ne)
    alg = np.arange(g.nv) % 5 == 0
    vm = [dataclasses.replace(nd.diffusion_vertex(), mass_matrix=0) if a else nd.diffusion_vertex() for a in alg]
    net = nd.Network(g, vm, nd.diffusion_edge())
    idx = net.v_data
    A = np.zeros((g.nv, g.nv))
    for e, (s_, d) in enumerate(zip(g.src, g.dst)):
        A[s_, d] += w[e]
        A[d, s_] += w[e]
        A[s_, s_] -= w[e]
        A[d, d] -= w[e]
    X, Z = np.nonzero(~alg)[0], np.nonzero(alg)[0]
    Azz_inv_Azx = np.linalg.solve(A[np.ix_(Z, Z)], A[np.ix_(Z, X)])
    S = A[np.ix_(X, X)] - A[np.ix_(X, Z)] @ Azz_inv_Azx
    x0 = rng.normal(size=len(X))
    v0 = np.zeros(g.nv)
    v0[X] = x0
    v0[Z] = -Azz_inv_Azx @ x0
    u0 = np.empty(net.dim)
    u0[idx] = v0
    u, st = solve_rodas4(nd.adapt(net, torch.float64), u0, w, (0.0, 2.0), reltol=1e-8, abstol=1e-10)
    assert st.status == 0 and st.t_final == 2.0
    got = u.cpu().numpy()[idx]
    xT = scipy.linalg.expm(S * 2.0) @ x0
    np.testing.assert_allclose(got[X], xT, atol=1e-7)
    np.testing.assert_allclose(got[Z], -Azz_inv_Azx @ xT, atol=1e-7)


def test_rodas4_swing_against_oracle(cuda):
    """Swing on BA(100, 2) against the oracle's dense Rodas4 restatement (central-difference
    Jacobian): the same step sequence (within 2) and the same end state; both within the
    tolerance of the oracle's Tsit5 at 1e-11."""
    import torch
    from ndtest import fd_jacobian
    g = nd.barabasi_albert(100, 2, seed=6)
    on = O.OracleNetwork.from_graph(g, O.V_SWING, O.E_KURAMOTO)
    u0, p = random_inputs(on, O.V_SWING, np.random.default_rng(6))
    u0[0::2] *= 0.1
    u0[1::2] = 0.0
    nw = nd.adapt(nd.Network(g, nd.kuramoto_second(), nd.static_line()), torch.float64)
    u, st = solve_rodas4(nw, u0, p, (0.0, 0.5), reltol=1e-7, abstol=1e-9)
    ref, na, nr = O.rodas4(lambda x: on.rhs(x, p), lambda x: fd_jacobian(on, x, p), u0, 0.0, 0.5, 1e-7, 1e-9)
    assert st.status == 0 and st.t_final == 0.5
    assert abs(st.naccept - na) <= 2 and abs(st.nreject - nr) <= 2
    np.testing.assert_allclose(u.cpu().numpy(), ref, atol=1e-8, rtol=0)
    exact, _ = on.tsit5(u0, p, 0.0, 0.5, reltol=1e-11, abstol=1e-13)
    assert np.max(np.abs(u.cpu().numpy() - exact)) <= 1e3 * 1e-7 * max(1.0, np.abs(exact).max())
