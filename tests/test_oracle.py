"""Pins of the CPU oracle against the reference's own known answers and fixtures.

The reference cannot run here (no Julia), so the oracle is pinned by the analytic answers
its tests use: du = -L·x for diffusion (test/diffusion_test.jl:80-90), Tsit5 against
exp(-tL)·x0 (test/diffusion_test.jl:119-129), the 4-node swing fixpoint
(test/initialization_test.jl:15-38), and by an independent numpy restatement.
"""
import numpy as np
import pytest
import scipy.linalg

import nd_gb300 as nd
from oracle import oracle as O

GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"


def test_diffusion_equals_minus_laplacian():
    d = np.load(GOLDEN / "diffusion_ba10_5.npz")
    g = nd.Graph(int(d["nv"]), d["src"], d["dst"])
    L = g.laplacian()
    on = O.OracleNetwork.from_graph(g, O.V_DIFFUSION, O.E_DIFFUSION_UNIT)
    for x, du in zip(d["x"], d["du"]):
        got = on.rhs(x, None)
        np.testing.assert_array_equal(got, du)              # fixture
        np.testing.assert_allclose(got, -L @ x, atol=1e-12)  # known answer


def test_tsit5_diffusion_known_answer():
    """solve(prob, Tsit5(); reltol=1e-5) matches exp(-tL)x0 to < 1e-6."""
    g = nd.barabasi_albert(10, 5, seed=42)
    L = g.laplacian()
    on = O.OracleNetwork.from_graph(g, O.V_DIFFUSION, O.E_DIFFUSION_UNIT)
    x0 = np.random.default_rng(3).normal(size=g.nv)
    for T in (0.5, 2.0, 5.0):
        uT, st = on.tsit5(x0, None, 0.0, T, reltol=1e-5, abstol=1e-8)
        assert st.status == 0
        assert np.max(np.abs(uT - scipy.linalg.expm(-T * L) @ x0)) < 1e-6


def test_tsit5_tableau_order_conditions():
    c, a, bt = O.tsit5_tableau()
    b = a[6, :6]
    b = np.append(b, 0.0)
    A = np.zeros((7, 7))
    A[:, :6] = a
    np.testing.assert_allclose(A.sum(axis=1), c, atol=1e-14)  # row-sum condition
    # order 5 conditions of the propagating weights b (FSAL: b = last row of A)
    assert abs(b.sum() - 1) < 1e-14
    assert abs(b @ c - 1 / 2) < 1e-14
    assert abs(b @ c**2 - 1 / 3) < 1e-14
    assert abs(b @ (A @ c) - 1 / 6) < 1e-14
    assert abs(b @ c**3 - 1 / 4) < 1e-13
    assert abs(b @ (c * (A @ c)) - 1 / 8) < 1e-13
    assert abs(b @ (A @ c**2) - 1 / 12) < 1e-13
    assert abs(b @ (A @ (A @ c)) - 1 / 24) < 1e-13
    assert abs(b @ c**4 - 1 / 5) < 1e-13
    # embedded 4th-order weights bhat = b - btilde
    bhat = b - bt
    assert abs(bhat.sum() - 1) < 1e-14
    assert abs(bhat @ c - 1 / 2) < 1e-13
    assert abs(bhat @ c**2 - 1 / 3) < 1e-13
    assert abs(bhat @ c**3 - 1 / 4) < 1e-13
    assert abs(bt.sum()) < 1e-14


def test_swing_fixpoint_known_answer():
    """C4 with P = [1,-1,1,-1], K = 6: each generator sends 1/2 to each neighbour,
    so neighbouring phases differ by asin(1/12)."""
    d = np.load(GOLDEN / "swing_ws4.npz")
    th, it, res = O.newton_fixpoint(4, d["src"], d["dst"], 6.0, d["P"])
    assert res <= 1e-10
    np.testing.assert_allclose(np.abs(np.diff(th)), np.arcsin(1 / 12), atol=1e-12)
    np.testing.assert_allclose(th, d["theta"], atol=1e-12)
    # at the fixpoint the full swing RHS vanishes
    g = nd.Graph(4, d["src"], d["dst"])
    on = O.OracleNetwork.from_graph(g, O.V_SWING, O.E_KURAMOTO)
    u = np.zeros(8)
    u[0::2] = th
    p = np.concatenate([np.stack([np.ones(4), np.full(4, 0.1), d["P"]], 1).ravel(), np.full(4, 6.0)])
    assert np.max(np.abs(on.rhs(u, p))) <= 1e-10


@pytest.mark.parametrize("vk,ek", [(1, 1), (1, 2), (1, 3), (2, 1), (2, 3), (3, 3), (3, 1), (3, 2)])
def test_c_oracle_matches_numpy_mirror(vk, ek):
    g = nd.barabasi_albert(700, 3, seed=vk * 10 + ek)
    on = O.OracleNetwork.from_graph(g, vk, ek)
    rng = np.random.default_rng(vk + ek)
    u = rng.normal(size=on.dim)
    p = rng.uniform(0.5, 1.5, size=on.pdim)
    for dt in (np.float64, np.float32):
        a = on.rhs(u, p, dtype=dt)
        b = O.rhs_numpy(g.nv, g.src, g.dst, vk, ek, u, p, dtype=dt)
        if dt == np.float64 or ek != 3:
            np.testing.assert_array_equal(a, b)
        else:  # numpy's float32 sin is not libm's sinf
            np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-5)
    np.testing.assert_array_equal(on.rhs_poly(u, p), on.rhs(u, p))


def test_heterogeneous_batches_layout():
    """Vertex batches are laid out batch-major in order of first appearance
    (src/construction.jl:155-195 with find_identical, src/utils.jl:197-216)."""
    g = nd.cycle_graph(6)
    vk = np.array([O.V_SWING, O.V_KURAMOTO, O.V_SWING, O.V_KURAMOTO, O.V_SWING, O.V_KURAMOTO], dtype=np.int32)
    on = O.OracleNetwork(6, g.src, g.dst, vk, O.E_KURAMOTO)
    lib = on.lib
    starts = [lib.nd_oracle_v_data(on.L, v) for v in range(6)]
    assert starts == [0, 6, 2, 7, 4, 8]
    assert on.dim == 9 and on.pdim == 3 * 3 + 3 + 6


def test_golden_fixtures_reproduce():
    d = np.load(GOLDEN / "kuramoto_ws1000.npz")
    on = O.OracleNetwork(int(d["nv"]), d["src"], d["dst"], O.V_KURAMOTO, O.E_KURAMOTO)
    np.testing.assert_array_equal(on.rhs(d["u"], d["p"]), d["du"])
    d = np.load(GOLDEN / "swing_ba200.npz")
    on = O.OracleNetwork(int(d["nv"]), d["src"], d["dst"], O.V_SWING, O.E_KURAMOTO)
    np.testing.assert_array_equal(on.rhs(d["u"], d["p"]), d["du"])


def test_threaded_tsit5_equals_sequential_tsit5():
    """The threaded oracle Tsit5 (PolyesterExecution restatement of the RHS, parallel stage
    updates) takes the same steps and ends in the same bits as the sequential one: the GPU
    tests use it for long solves on large networks."""
    g = nd.barabasi_albert(3000, 2, seed=7)
    on = O.OracleNetwork.from_graph(g, O.V_SWING, O.E_KURAMOTO)
    rng = np.random.default_rng(3)
    u0 = np.zeros(on.dim)
    u0[0::2] = rng.uniform(-np.pi, np.pi, g.nv)
    pm = rng.uniform(0.5, 1.5, g.nv) * np.where(np.arange(g.nv) % 2 == 0, 1, -1)
    pm -= pm.mean()
    p = np.concatenate([np.stack([np.ones(g.nv), np.full(g.nv, 0.1), pm], 1).ravel(),
                        rng.uniform(5, 10, g.ne)])
    a, sa = on.tsit5(u0, p, 0.0, 1.0, reltol=1e-8, abstol=1e-10)
    b, sb = on.tsit5(u0, p, 0.0, 1.0, reltol=1e-8, abstol=1e-10, threaded=True)
    assert (sa.naccept, sa.nreject, sa.status) == (sb.naccept, sb.nreject, sb.status)
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("n,m,seed", [(10, 5, 42), (1000, 1, 3), (20_000, 4, 1), (5000, 3, 9)])
def test_oracle_barabasi_albert_equals_package_generator(n, m, seed):
    """The oracle's copy of the seeded Barabási–Albert generator (used by the benchmark's CPU
    reference arm) returns the package generator's edge list."""
    a = O.barabasi_albert(n, m, seed)
    b = nd.barabasi_albert(n, m, seed=seed)
    assert a.nv == b.nv
    np.testing.assert_array_equal(a.src, b.src)
    np.testing.assert_array_equal(a.dst, b.dst)


def test_oracle_rosenbrock23_known_answer():
    """The oracle's dense Rosenbrock23 (the restatement the GPU solver is checked against)
    reproduces exp(-tL) x0 for diffusion (test/diffusion_test.jl:119-129), and with a zero
    mass-matrix entry keeps that vertex on its algebraic constraint."""
    import scipy.linalg
    g = nd.barabasi_albert(20, 3, seed=4)
    L = g.laplacian()
    on = O.OracleNetwork.from_graph(g, O.V_DIFFUSION, O.E_DIFFUSION_UNIT)
    x0 = np.random.default_rng(1).normal(size=g.nv)
    rhs, jac = (lambda x: on.rhs(x, None)), (lambda x: -L)
    u, na, nr = O.rosenbrock23(rhs, jac, x0, 0.0, 1.0, 1e-6, 1e-9)
    assert na > 0 and np.max(np.abs(u - scipy.linalg.expm(-L) @ x0)) < 1e-5
    mass = np.ones(g.nv)
    mass[0] = 0.0
    x0[0] = -L[0, 1:] @ x0[1:] / L[0, 0]  # consistent: (L x)_0 = 0
    u, _, _ = O.rosenbrock23(rhs, jac, x0, 0.0, 1.0, 1e-6, 1e-9, mass=mass)
    assert abs(L[0] @ u) < 1e-10


def test_oracle_rodas4_is_fourth_order():
    """The Rodas4 restatement (the coefficients the GPU solver uses) converges with order 4
    at fixed steps on a nonlinear ODE (y' = -y², y(1) = 1/2), a stiff linear system and an
    index-1 DAE with a nonlinear algebraic row (mass matrix diag(1, 0)): halving the step
    divides the error by ~16."""
    def ratios(f, jac, y0, exact, mass=None):
        errs = [np.abs(O.rodas4(f, jac, y0, 0.0, 1.0, 1.0, 1.0, mass=mass, fixed_dt=h)[0] - exact).max()
                for h in (0.1, 0.05, 0.025)]
        return [errs[i] / errs[i + 1] for i in range(2)]

    for r in ratios(lambda y: -y ** 2, lambda y: np.diag(-2 * y), np.array([1.0]), 0.5):
        assert 14.0 < r < 19.0
    A = np.array([[-1.0, 1.0], [0.0, -100.0]])
    y0 = np.array([1.0, 1.0])
    for r in ratios(lambda y: A @ y, lambda y: A, y0, scipy.linalg.expm(A) @ y0):
        assert 14.0 < r < 19.0
    f = lambda y: np.array([-y[0] + y[1], y[0] - 2 * y[1] + 0.1 * y[1] ** 2])
    jac = lambda y: np.array([[-1.0, 1.0], [1.0, -2.0 + 0.2 * y[1]]])
    z0 = np.array([1.0, (2 - np.sqrt(3.6)) / 0.2])  # consistent: 0 = y1 - 2 y2 + 0.1 y2²
    ref = O.rodas4(f, jac, z0, 0.0, 1.0, 1e-13, 1e-13, mass=[1.0, 0.0])[0]
    for r in ratios(f, jac, z0, ref, mass=[1.0, 0.0]):
        assert 14.0 < r < 19.0
    # adaptive: the algebraic row stays satisfied and the steps follow tol^(-1/4)
    y, na, _ = O.rodas4(f, jac, z0, 0.0, 1.0, 1e-6, 1e-8, mass=[1.0, 0.0])
    assert abs(y[0] - 2 * y[1] + 0.1 * y[1] ** 2) < 1e-9 and np.abs(y - ref).max() < 1e-6
