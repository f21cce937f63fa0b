"""The CPU oracle on batched networks (several vertex / edge batches, ODE edges, the
Symmetric / Directed / Fiducial outputs): the layout the reference builds, and the RHS
against the independent numpy restatement.

The network of the reference's GPU test (test/GPU_test.jl:12-21) is the first case: a
complete graph on 4 vertices with swing and diffusion vertices and ODE, Kuramoto and
two-sided Fiducial edges.
"""
from pathlib import Path

import numpy as np
import pytest

import nd_gb300 as nd
from oracle import oracle as O

ALL_EDGE_BATCHES = [
    (O.E_DIFFUSION, O.C_ANTISYMMETRIC), (O.E_DIFFUSION_UNIT, O.C_SYMMETRIC), (O.E_KURAMOTO, O.C_DIRECTED),
    (O.E_DIFFUSION_ODE, O.C_FIDUCIAL), (O.E_DIFFUSION, O.C_FIDUCIAL), (O.E_KURAMOTO, O.C_ANTISYMMETRIC),
    (O.E_DIFFUSION_ODE_FIXED, O.C_FIDUCIAL), (O.E_DIFFUSION_UNIT, O.C_DIRECTED),
]
ALL_VERTEX_BATCHES = [O.V_SWING, O.V_DIFFUSION, O.V_KURAMOTO, O.V_SWING_UNIT]


def gpu_test_network():
    """complete_graph(4), vf = [swing, diffusion, swing, diffusion],
    ef = [odeedge, kuramoto, kuramoto, edge_fid, odeedge, edge_fid] (test/GPU_test.jl:13-20),
    as batches in order of first appearance."""
    g = nd.complete_graph(4)
    vbatches = [O.V_SWING, O.V_DIFFUSION]
    vbatch = [0, 1, 0, 1]
    ebatches = [(O.E_DIFFUSION_ODE, O.C_FIDUCIAL), (O.E_KURAMOTO, O.C_ANTISYMMETRIC), (O.E_DIFFUSION, O.C_FIDUCIAL)]
    ebatch = [0, 1, 1, 2, 0, 2]
    return g, vbatches, vbatch, ebatches, ebatch


def random_batched(nv=300, m=3, seed=0, vbatches=ALL_VERTEX_BATCHES, ebatches=ALL_EDGE_BATCHES):
    g = nd.barabasi_albert(nv, m, seed=seed)
    rng = np.random.default_rng(seed)
    return (g, list(vbatches), rng.integers(0, len(vbatches), g.nv).astype(np.int32), list(ebatches),
            rng.integers(0, len(ebatches), g.ne).astype(np.int32))


def _inputs(on, seed):
    rng = np.random.default_rng(seed)
    u = rng.normal(size=on.dim)
    p = rng.uniform(0.5, 1.5, size=on.pdim)
    return u, p


def test_gpu_test_network_layout():
    """dim 10 / pdim 12; vertex states batch-major (swing 0, 2 then diffusion 1, 3), the
    ODE edges' states after every vertex state (src/network_structure.jl:224-258)."""
    g, vb, vbi, eb, ebi = gpu_test_network()
    assert list(zip(g.src.tolist(), g.dst.tolist())) == [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, vbi, eb, ebi)
    assert on.dim == 10 and on.pdim == 12
    assert [on.lib.nd_oracle_v_data(on.L, v) for v in range(4)] == [0, 4, 2, 5]
    assert [on.lib.nd_oracle_v_para(on.L, v) for v in range(4)] == [0, 6, 3, 6]
    assert [on.lib.nd_oracle_e_data(on.L, e) for e in (0, 4)] == [6, 8]
    # edge parameters: ODE τ (edges 0, 4), then K (1, 2), then the fiducial p (3, 5)
    assert [on.lib.nd_oracle_e_para(on.L, e) for e in range(6)] == [6, 8, 9, 10, 7, 11]
    L = O.layout_batched(g.nv, g.src, g.dst, vb, vbi, eb, ebi)
    assert L["dim"] == 10 and L["pdim"] == 12
    assert L["v_data"].tolist() == [0, 4, 2, 5] and L["e_para"].tolist() == [6, 8, 9, 10, 7, 11]


def test_gpu_test_network_rhs_hand_computed():
    """Every entry of du of the reference's GPU-test network computed by hand from the
    component functions (test/ComponentLibrary.jl) and the layout above."""
    g, vb, vbi, eb, ebi = gpu_test_network()
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, vbi, eb, ebi)
    u, p = _inputs(on, 1)
    du = on.rhs(u, p)
    th = {0: u[0], 1: u[4], 2: u[2], 3: u[5]}          # vertex outputs
    tau = {0: p[6], 4: p[7]}
    K = {1: p[8], 2: p[9]}
    w = {3: p[10], 5: p[11]}
    es = {0: (u[6], u[7]), 4: (u[8], u[9])}
    edges = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    ysrc, ydst = {}, {}
    for e, (s, d) in enumerate(edges):
        if e in es:
            ydst[e], ysrc[e] = es[e]
        elif e in K:
            ydst[e] = K[e] * np.sin(th[s] - th[d])
            ysrc[e] = -ydst[e]
        else:
            ydst[e] = w[e] * (th[s] - th[d])
            ysrc[e] = -ydst[e]
    agg = [0.0] * 4
    order = [0, 4, 1, 2, 3, 5]                          # out order: edge batches, src then dst
    for e in order:
        s, d = edges[e]
        agg[s] = agg[s] + ysrc[e]
        agg[d] = agg[d] + ydst[e]
    exp = np.zeros(10)
    for v, (st, q) in {0: (0, 0), 2: (2, 3)}.items():
        M, D, Pm = p[q:q + 3]
        exp[st] = u[st + 1]
        exp[st + 1] = 1 / M * (Pm - D * u[st + 1] + agg[v])
    exp[4], exp[5] = agg[1], agg[3]
    for e, s0 in ((0, 6), (4, 8)):
        s, d = edges[e]
        exp[s0] = 1 / tau[e] * (np.sin(th[s] - th[d]) - u[s0])
        exp[s0 + 1] = 1 / tau[e] * (np.sin(th[d] - th[s]) - u[s0 + 1])
    np.testing.assert_allclose(du, exp, rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_batched_rhs_matches_numpy(seed):
    g, vb, vbi, eb, ebi = random_batched(seed=seed)
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, vbi, eb, ebi)
    u, p = _inputs(on, seed)
    ref = O.rhs_numpy_batched(g.nv, g.src, g.dst, vb, vbi, eb, ebi, u, p)
    np.testing.assert_allclose(on.rhs(u, p), ref, rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(on.rhs_poly(u, p), ref, rtol=1e-13, atol=1e-13)
    ref32 = O.rhs_numpy_batched(g.nv, g.src, g.dst, vb, vbi, eb, ebi, u, p, dtype=np.float32)
    np.testing.assert_allclose(on.rhs(u, p, dtype=np.float32), ref32, rtol=2e-5, atol=2e-5)


def test_batched_without_sine_is_bitwise():
    """No transcendental functions: the C oracle and numpy agree bit for bit (the same
    operations in the same order)."""
    vb = [O.V_DIFFUSION, O.V_KURAMOTO, O.V_SWING, O.V_SWING_UNIT]
    eb = [(O.E_DIFFUSION, O.C_ANTISYMMETRIC), (O.E_DIFFUSION_UNIT, O.C_SYMMETRIC), (O.E_DIFFUSION, O.C_DIRECTED),
          (O.E_DIFFUSION, O.C_FIDUCIAL)]
    g, vb, vbi, eb, ebi = random_batched(nv=500, m=4, seed=5, vbatches=vb, ebatches=eb)
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, vbi, eb, ebi)
    u, p = _inputs(on, 5)
    np.testing.assert_array_equal(on.rhs(u, p), O.rhs_numpy_batched(g.nv, g.src, g.dst, vb, vbi, eb, ebi, u, p))


def test_kind_constructor_equals_first_appearance_batches():
    g = nd.watts_strogatz(60, 4, 0.2, seed=3)
    rng = np.random.default_rng(3)
    vk = rng.choice([O.V_SWING, O.V_KURAMOTO, O.V_DIFFUSION], g.nv).astype(np.int32)
    ek = rng.choice([O.E_KURAMOTO, O.E_DIFFUSION], g.ne).astype(np.int32)
    a = O.OracleNetwork(g.nv, g.src, g.dst, vk, ek)
    vb = list(dict.fromkeys(vk.tolist()))
    eb = list(dict.fromkeys(ek.tolist()))
    b = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, [vb.index(k) for k in vk], [(k, O.C_ANTISYMMETRIC) for k in eb],
                                     [eb.index(k) for k in ek])
    assert (a.dim, a.pdim) == (b.dim, b.pdim)
    u, p = _inputs(a, 3)
    np.testing.assert_array_equal(a.rhs(u, p), b.rhs(u, p))


def test_ode_edge_relaxes_to_the_static_sine_coupling():
    """Known answer: the ODE edge's states have the fixed point e1 = sin(θs - θd),
    e2 = sin(θd - θs) (de = (sin(..) - e)/τ); there every vertex receives the unit-sine
    coupling of its neighbours, and at e = 0 the state derivatives are sin(..)/τ."""
    g = nd.cycle_graph(5)
    vb, vbi = [O.V_KURAMOTO], [0] * 5
    eb, ebi = [(O.E_DIFFUSION_ODE, O.C_FIDUCIAL)], [0] * 5
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, vbi, eb, ebi)
    rng = np.random.default_rng(0)
    th = rng.uniform(-1, 1, 5)
    u = np.concatenate([th, np.zeros(10)])
    p = np.concatenate([np.zeros(5), np.full(5, 0.5)])  # ω = 0, τ = 0.5
    du = on.rhs(u, p)
    s, d = g.src, g.dst
    np.testing.assert_allclose(du[5::2], 2.0 * np.sin(th[s] - th[d]), rtol=1e-15)
    np.testing.assert_allclose(du[6::2], 2.0 * np.sin(th[d] - th[s]), rtol=1e-15)
    u[5::2], u[6::2] = np.sin(th[s] - th[d]), np.sin(th[d] - th[s])
    du = on.rhs(u, p)
    np.testing.assert_allclose(du[5:], 0.0, atol=1e-16)
    exp = np.zeros(5)
    np.add.at(exp, d, np.sin(th[s] - th[d]))
    np.add.at(exp, s, np.sin(th[d] - th[s]))
    np.testing.assert_allclose(du[:5], exp, atol=1e-15)


def powergrid(nv=300, seed=0, pq_only=False):
    """A power-grid network: PQ buses and generators on a Watts-Strogatz graph with π-line
    edges (benchmark/benchmark_cases.jl:68-79)."""
    g = nd.watts_strogatz(nv, 4, 0.5, seed=seed)
    rng = np.random.default_rng(seed)
    kinds = np.zeros(nv, dtype=int) if pq_only else rng.integers(0, 2, nv)
    order = list(dict.fromkeys(kinds.tolist()))          # batches in order of first appearance
    vb = [[O.V_PQ, O.V_GENERATOR][k] for k in order]
    vbi = np.array([order.index(k) for k in kinds], dtype=np.int32)
    return g, vb, vbi, [(O.E_PILINE, O.C_FIDUCIAL)], np.zeros(g.ne, dtype=np.int32)


@pytest.mark.parametrize("pq_only", [False, True])
def test_powergrid_oracle_matches_numpy_complex(pq_only):
    """The C restatement of piline!, pq! and gen! (real arithmetic in Julia's operation order)
    against numpy's complex arithmetic."""
    g, vb, vbi, eb, ebi = powergrid(pq_only=pq_only)
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, vbi, eb, ebi)
    assert on.depth == 2 and on.n_out == 2 * (g.nv + 2 * g.ne)
    rng = np.random.default_rng(1)
    u, p = rng.normal(size=on.dim), rng.uniform(0.5, 1.5, size=on.pdim)
    ref = O.rhs_numpy_batched(g.nv, g.src, g.dst, vb, vbi, eb, ebi, u, p)
    scale = 1 + np.abs(ref)
    assert np.max(np.abs(on.rhs(u, p) - ref) / scale) < 1e-12
    np.testing.assert_array_equal(on.rhs_poly(u, p), on.rhs(u, p))


def test_piline_known_answer():
    """One π-line between two PQ buses: the currents are the line's admittance equations,
    i_dst = (Vs - Vd)/(R + iωL) - iωC2·Vd into the destination, and the PQ buses map them to
    du = S / conj(i)."""
    g = nd.Graph(2, np.array([0]), np.array([1]))
    on = O.OracleNetwork.from_batches(2, g.src, g.dst, [O.V_PQ], [0, 0], [(O.E_PILINE, O.C_FIDUCIAL)], [0])
    Vs, Vd = 1.0 + 0.2j, 0.9 - 0.1j
    L, R, C1, C2 = 1e-3, 0.05, 2e-5, 3e-5
    P = np.array([0.3, -0.4, 0.1, 0.2])                 # (P, Q) of bus 0, then of bus 1
    u = np.array([Vs.real, Vs.imag, Vd.real, Vd.imag])
    p = np.concatenate([P, [L, R, C1, C2]])
    w = 2 * np.pi * 50
    imain = (Vs - Vd) / (R + 1j * w * L)
    i_to_src = imain + 1j * w * C1 * Vs                   # -isrc
    i_to_dst = -(imain - 1j * w * C2 * Vd)                # -idst
    du = on.rhs(u, p)
    exp0 = (P[0] + 1j * P[1]) / np.conj(i_to_src)
    exp1 = (P[2] + 1j * P[3]) / np.conj(i_to_dst)
    np.testing.assert_allclose(du, [exp0.real, exp0.imag, exp1.real, exp1.imag], rtol=1e-13)


def test_mixed_output_dimensions_rejected():
    """All vertex models (and edge models) must have the same output dimension
    (src/construction.jl:98-106)."""
    g = nd.cycle_graph(4)
    with pytest.raises(ValueError):
        O.OracleNetwork.from_batches(4, g.src, g.dst, [O.V_PQ, O.V_DIFFUSION], [0, 1, 0, 1],
                                     [(O.E_PILINE, O.C_FIDUCIAL)], [0] * 4)
    with pytest.raises(nd.ArgumentError):
        nd.Network(g, [nd.pqnode(), nd.diffusion_vertex(), nd.pqnode(), nd.diffusion_vertex()], nd.piline())


def test_inhomogeneous_pq_batches():
    """powergrid_inhomogeneous_pq (benchmark/benchmark_cases.jl:82-102): every PQ bus closes
    over its own P, Q and is a batch of its own; the constants ride with the batches."""
    g = nd.watts_strogatz(60, 4, 0.5, seed=4)
    rng = np.random.default_rng(4)
    gen_at = rng.permutation(g.nv)[:30]
    vb, vbi, consts = [], np.empty(g.nv, dtype=np.int32), []
    gen_batch = None
    for v in range(g.nv):                               # batches in order of first appearance
        if v in gen_at:
            if gen_batch is None:
                gen_batch = len(vb)
                vb.append(O.V_GENERATOR)
                consts.append((0.0, 0.0))
            vbi[v] = gen_batch
        else:
            vbi[v] = len(vb)
            vb.append(O.V_PQ_CONST)
            consts.append((-rng.random(), -rng.random()))
    eb, ebi = [(O.E_PILINE, O.C_FIDUCIAL)], np.zeros(g.ne, dtype=np.int32)
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, vbi, eb, ebi, vertex_constants=consts)
    assert len(vb) == 31 and on.pdim == 30 * 11 + g.ne * 4
    u, p = rng.normal(size=on.dim), rng.uniform(0.5, 1.5, size=on.pdim)
    ref = O.rhs_numpy_batched(g.nv, g.src, g.dst, vb, vbi, eb, ebi, u, p, vertex_constants=consts)
    assert np.max(np.abs(on.rhs(u, p) - ref) / (1 + np.abs(ref))) < 1e-12


@pytest.mark.parametrize("name", ["batched_gpu_test", "powergrid_ws300"])
def test_batched_golden_fixtures_reproduce(name):
    """The oracle reproduces its committed fixtures bit for bit (tests/golden/gen_golden.py)."""
    d = np.load(Path(__file__).resolve().parent / "golden" / f"{name}.npz")
    on = O.OracleNetwork.from_batches(int(d["nv"]), d["src"], d["dst"], d["vb"].tolist(), d["vbi"],
                                      [tuple(x) for x in d["eb"].tolist()], d["ebi"])
    np.testing.assert_array_equal(on.rhs(d["u"], d["p"]), d["du"])
