"""GPU Tsit5 against the CPU oracle's Tsit5 (same tableau, controller and operation order)
and against the reference's known answer exp(-tL)x0 (test/diffusion_test.jl:119-129)."""
import numpy as np
import pytest
import scipy.linalg

import nd_gb300 as nd
from nd_gb300.solve import solve_tsit5
from oracle import oracle as O

from ndtest import random_inputs

pytestmark = pytest.mark.gpu

GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"


def test_diffusion_known_answer(cuda):
    import torch
    g = nd.barabasi_albert(10, 5, seed=42)
    L = g.laplacian()
    nw = nd.adapt(nd.Network(g, nd.diffusion_vertex(), nd.diffusion_edge_unit()), torch.float64)
    x0 = np.random.default_rng(3).normal(size=g.nv)
    on = O.OracleNetwork.from_graph(g, O.V_DIFFUSION, O.E_DIFFUSION_UNIT)
    for T in (0.5, 5.0):
        u, st = solve_tsit5(nw, x0, None, (0.0, T), reltol=1e-5, abstol=1e-8)
        assert st.status == 0 and st.t_final == T
        got = u.cpu().numpy()
        assert np.max(np.abs(got - scipy.linalg.expm(-T * L) @ x0)) < 1e-6
        ref, rst = on.tsit5(x0, None, 0.0, T, reltol=1e-5, abstol=1e-8)
        assert (st.naccept, st.nreject) == (rst.naccept, rst.nreject)
        assert np.max(np.abs(got - ref)) < 1e-12


def test_kuramoto_ws1000_golden_trajectory(cuda):
    """First-order Kuramoto on WS(1000, 10, 0.1), Tsit5 to t = 10 at reltol 1e-8,
    abstol 1e-10: the GPU solve follows the oracle's step sequence and state."""
    import torch
    d = np.load(GOLDEN / "kuramoto_ws1000.npz")
    g = nd.Graph(int(d["nv"]), d["src"], d["dst"])
    nw = nd.adapt(nd.Network(g, nd.kuramoto_first(), nd.kuramoto_edge()), torch.float64)
    u, st = solve_tsit5(nw, d["u"], d["p"], (0.0, 10.0), reltol=1e-8, abstol=1e-10)
    assert st.status == 0
    assert abs(st.naccept - int(d["naccept"])) <= 2 and st.nreject <= int(d["nreject"]) + 2
    np.testing.assert_allclose(u.cpu().numpy(), d["u_t10"], atol=1e-7, rtol=0)


def test_swing_ba20k_against_oracle(cuda):
    import torch
    g = nd.barabasi_albert(20_000, 2, seed=4)
    on = O.OracleNetwork.from_graph(g, O.V_SWING, O.E_KURAMOTO)
    u0, p = random_inputs(on, O.V_SWING, np.random.default_rng(9))
    u0[1::2] = 0.0
    nw = nd.adapt(nd.Network(g, nd.kuramoto_second(), nd.static_line()), torch.float64)
    u, st = solve_tsit5(nw, u0, p, (0.0, 2.0), reltol=1e-6, abstol=1e-8)
    ref, rst = on.tsit5(u0, p, 0.0, 2.0, reltol=1e-6, abstol=1e-8)
    assert st.status == 0 and rst.status == 0
    assert abs(st.naccept - rst.naccept) <= 2
    np.testing.assert_allclose(u.cpu().numpy(), ref, atol=1e-5, rtol=0)
    # FP32 RHS with FP64 state: within the tolerance's reach of the FP64 solve
    nw32 = nd.adapt(nd.Network(g, nd.kuramoto_second(), nd.static_line()), torch.float32)
    u32, st32 = solve_tsit5(nw32, u0, p, (0.0, 2.0), reltol=1e-6, abstol=1e-8)
    assert st32.status == 0
    assert np.max(np.abs(u32.cpu().numpy() - ref)) < 1e-3


def test_swing_ba100k_t20_against_oracle(cuda):
    """The swing workload of the plain GPU method: BA(1e5, m=2), K ~ U(5,10), P = ±U(0.5,1.5)
    zero-sum, Tsit5 to t = 20 at reltol 1e-8, abstol 1e-10, against the oracle's Tsit5 on the
    host cores (the threaded restatement gives the sequential solve's bits).

    * From the steady state with every phase perturbed by N(0, 0.05²): the dynamics
      contract, and the final states agree to 1e-7 (ten times the relative tolerance at
      |θ| ~ 1) with step counts within 2.
    * From random phases U(-π, π) the network desynchronises and the dynamics are chaotic:
      the 1-ulp differences between CUDA's and libm's sines grow to O(1) by t = 20, as two
      CPU solves whose RHS differ in one last bit do.  The step sequences still agree
      (within 2 accepted / rejected steps), and so does the one exact invariant,
      Σω(t) = Σω(0) e^{-Dt} with ΣP = 0 and M = 1 (the couplings cancel in pairs)."""
    import torch
    g = nd.barabasi_albert(100_000, 2, seed=1)
    on = O.OracleNetwork.from_graph(g, O.V_SWING, O.E_KURAMOTO)
    u0, p = random_inputs(on, O.V_SWING, np.random.default_rng(9))
    u0[1::2] = 0.0
    nw = nd.adapt(nd.Network(g, nd.kuramoto_second(), nd.static_line()), torch.float64)
    # near the steady state
    ufix = nd.find_fixpoint(nw, p).cpu().numpy()
    us = ufix.copy()
    us[0::2] += 0.05 * np.random.default_rng(10).normal(size=g.nv)
    u, st = solve_tsit5(nw, us, p, (0.0, 20.0), reltol=1e-8, abstol=1e-10)
    ref, rst = on.tsit5(us, p, 0.0, 20.0, reltol=1e-8, abstol=1e-10, threaded=True)
    assert st.status == 0 and rst.status == 0 and st.t_final == 20.0
    assert abs(st.naccept - rst.naccept) <= 2 and abs(st.nreject - rst.nreject) <= 2
    np.testing.assert_allclose(u.cpu().numpy(), ref, atol=1e-7, rtol=0)
    # random phases: chaotic; compare the step sequence and the exact invariant
    u0[1::2] = np.random.default_rng(11).normal(size=g.nv)
    u, st = solve_tsit5(nw, u0, p, (0.0, 20.0), reltol=1e-8, abstol=1e-10)
    ref, rst = on.tsit5(u0, p, 0.0, 20.0, reltol=1e-8, abstol=1e-10, threaded=True)
    assert st.status == 0 and rst.status == 0
    assert abs(st.naccept - rst.naccept) <= 2 and abs(st.nreject - rst.nreject) <= 2
    want = u0[1::2].sum() * np.exp(-0.1 * 20.0)
    scale = np.abs(u0[1::2]).sum()
    got = u.cpu().numpy()
    assert abs(got[1::2].sum() - want) <= 1e-6 * scale and abs(ref[1::2].sum() - want) <= 1e-6 * scale


def test_solve_rejects_bad_arguments(cuda):
    import torch
    g = nd.cycle_graph(5)
    nw = nd.adapt(nd.Network(g, nd.diffusion_vertex(), nd.diffusion_edge_unit()), torch.float64)
    with pytest.raises(nd.ArgumentError):
        solve_tsit5(nw, np.zeros(4), None, (0.0, 1.0))
    with pytest.raises(nd.ArgumentError):
        solve_tsit5(nw, np.zeros(5), None, (1.0, 0.0))
    with pytest.raises(nd.NotConvergedError):
        solve_tsit5(nw, np.arange(5.0), None, (0.0, 100.0), reltol=1e-12, abstol=1e-14, max_steps=5)
