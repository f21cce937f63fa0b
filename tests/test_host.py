"""Host-side logic of the GB300 Network mirror: layout sizes, component checks, graph
generators.  No GPU needed."""
import operator

import numpy as np
import pytest

import nd_gb300 as nd


def test_layout_sizes_match_reference_layout():
    g = nd.barabasi_albert(100, 2, seed=1)
    nw = nd.Network(g, nd.kuramoto_second(), nd.static_line())
    assert nw.dim == 200
    assert nw.pdim == 3 * 100 + g.ne
    assert nw.edge_param_index(0) == 300
    nw1 = nd.Network(g, nd.diffusion_vertex(), nd.diffusion_edge_unit())
    assert nw1.dim == 100 and nw1.pdim == 0


def test_pflat_defaults_and_overrides():
    g = nd.cycle_graph(4)
    nw = nd.Network(g, nd.kuramoto_second(), nd.static_line())
    p = nw.pflat(vertex={"Pm": np.array([1.0, -1.0, 1.0, -1.0])}, edge={"K": 6.0})
    np.testing.assert_array_equal(p[:12].reshape(4, 3), [[1, .1, 1], [1, .1, -1], [1, .1, 1], [1, .1, -1]])
    np.testing.assert_array_equal(p[12:], 6.0)
    with pytest.raises(nd.ArgumentError):
        nd.Network(g, nd.kuramoto_first(), nd.kuramoto_edge()).pflat()  # ω and K have no default


def test_unsupported_component_raises_no_fallback():
    g = nd.cycle_graph(4)
    user_vertex = nd.VertexModel("my_vertex", dim=1, pdim=0, f=lambda *a: None)
    with pytest.raises(nd.UnsupportedComponentError):
        nd.Network(g, user_vertex, nd.diffusion_edge())
    with pytest.raises(nd.UnsupportedComponentError):
        nd.Symmetric(nd.diffusion_odeedge())  # the wrappers take a static single-sided g


def test_external_inputs_and_loopback_edges_are_rejected_by_name():
    """A network with external inputs (src/external_inputs.jl:51-80) or loopback edges
    (src/post_utils.jl:213-248) raises ArgumentError naming the feature, before any
    component lookup, also when the component would otherwise be a library one."""
    import dataclasses
    g = nd.cycle_graph(4)
    v_ext = dataclasses.replace(nd.kuramoto_first(), extin=[("VIndex", 2, "θ")])
    with pytest.raises(nd.ArgumentError, match="external inputs"):
        nd.Network(g, v_ext, nd.kuramoto_edge())
    user_ext = nd.VertexModel("fvext", dim=1, pdim=0, f=lambda *a: None, extin=[("VIndex", 2, "a")])
    with pytest.raises(nd.ArgumentError, match="external inputs") as err:
        nd.Network(g, user_ext, nd.diffusion_edge())
    assert not isinstance(err.value, nd.UnsupportedComponentError)
    e_ext = dataclasses.replace(nd.diffusion_edge(), extin=[("EIndex", 2, "a")])
    with pytest.raises(nd.ArgumentError, match="external inputs"):
        nd.Network(g, nd.diffusion_vertex(), e_ext)
    loop = dataclasses.replace(nd.diffusion_edge(), loopback=True)
    with pytest.raises(nd.ArgumentError, match="LoopbackConnection"):
        nd.Network(g, nd.diffusion_vertex(), [nd.diffusion_edge()] * (g.ne - 1) + [loop])


def test_heterogeneous_network_layout():
    """Batches in order of first appearance, laid out batch by batch; edge states after
    every vertex state (src/construction.jl:155-195, src/network_structure.jl:224-258)."""
    g = nd.complete_graph(4)
    vf = [nd.kuramoto_second(), nd.diffusion_vertex(), nd.kuramoto_second(), nd.diffusion_vertex()]
    ef = [nd.diffusion_odeedge(), nd.kuramoto_edge(), nd.kuramoto_edge(), nd.diffusion_edge_fid(),
          nd.diffusion_odeedge(), nd.diffusion_edge_fid()]
    nw = nd.Network(g, vf, ef)
    assert not nw.homogeneous and nw.vertexm is None and nw.edgem is None
    assert (nw.dim, nw.pdim) == (10, 12)
    assert nw.vertex_batch.tolist() == [0, 1, 0, 1] and nw.edge_batch.tolist() == [0, 1, 1, 2, 0, 2]
    assert [nw.vertex_state_index(v) for v in range(4)] == [0, 4, 2, 5]
    assert [nw.edge_state_index(e) for e in (0, 4)] == [6, 8]
    assert [nw.edge_param_index(e) for e in range(6)] == [6, 8, 9, 10, 7, 11]
    p = nw.pflat(vertex={"Pm": np.arange(4.0)}, edge={"K": 3.0})
    np.testing.assert_array_equal(p, [1, .1, 0, 1, .1, 2, 100, 100, 3, 3, 1, 1])
    same = nd.Network(g, [nd.kuramoto_first()] * 4, [nd.Directed(nd.kuramoto_edge())] * 6)
    assert same.homogeneous and same.edgem.coupling == "Directed"


def test_aggregator_only_plus():
    assert nd.GB300Aggregator(operator.add).f is operator.add
    with pytest.raises(nd.ArgumentError):
        nd.GB300Aggregator(operator.mul)
    a = nd.GB300Aggregator("+")
    assert isinstance(nd.get_aggr_constructor(a), nd.GB300Aggregator)
    assert nd.iscudacompatible(nd.GB300Execution()) and nd.iscudacompatible(a)


def _is_edges_order(g):
    assert np.all(g.src < g.dst)
    key = g.src * (g.nv + 1) + g.dst
    assert np.all(np.diff(key) > 0)


def test_generators_edge_order_and_sizes():
    ba = nd.barabasi_albert(2000, 4, seed=5)
    assert ba.ne == 4 * (2000 - 4)
    _is_edges_order(ba)
    ws = nd.watts_strogatz(1000, 10, 0.1, seed=1)
    assert ws.ne == 5000
    _is_edges_order(ws)
    assert ws.degree().min() >= 1
    rgg, xy = nd.random_geometric(500, 0.1, seed=3, return_positions=True)
    _is_edges_order(rgg)
    d = np.linalg.norm(xy[rgg.src] - xy[rgg.dst], axis=1)
    assert np.all(d < 0.1)
    # brute force: every pair closer than r is an edge
    diff = xy[:, None, :] - xy[None, :, :]
    close = (diff ** 2).sum(-1) < 0.01
    assert close[np.triu_indices(500, 1)].sum() == rgg.ne


def test_generators_are_deterministic():
    a = nd.barabasi_albert(5000, 3, seed=9)
    b = nd.barabasi_albert(5000, 3, seed=9)
    c = nd.barabasi_albert(5000, 3, seed=10)
    np.testing.assert_array_equal(a.src, b.src)
    np.testing.assert_array_equal(a.dst, b.dst)
    assert not np.array_equal(a.dst, c.dst)


def test_ba_is_power_law_with_hubs():
    g = nd.barabasi_albert(200_000, 4, seed=1)
    deg = g.degree()
    assert deg.min() == 4
    assert deg.max() > 300  # hubs well beyond the thread-per-vertex bucket


def test_power_grid_layout_and_closure_batches():
    """A power-grid network lays PQ buses (2 states) and generators (4 states) out batch by
    batch, with the π-line parameters after every vertex parameter; components closing over
    distinct values form one batch each."""
    g = nd.cycle_graph(6)
    vf = [nd.pqnode(), nd.generator(), nd.pqnode(), nd.generator(), nd.generator(), nd.pqnode()]
    nw = nd.Network(g, vf, nd.piline())
    assert [m.name for m in nw.vertex_batches] == ["pqnode", "generator"]
    assert [nw.vertex_state_index(v) for v in range(6)] == [0, 6, 2, 10, 14, 4]
    assert nw.dim == 3 * 2 + 3 * 4 and nw.pdim == 3 * 2 + 3 * 11 + 6 * 4
    assert [nw.edge_param_index(e) for e in range(6)] == [39 + 4 * e for e in range(6)]
    with pytest.raises(nd.ArgumentError):
        nw.pflat()  # P, Q and the machine data have no defaults
    many = [nd.EdgeModel(f"e{i}", pdim=0, kind=nd.capi.ND_E_DIFFUSION_UNIT, coupling=c)
            for i, c in enumerate(["AntiSymmetric", "Symmetric", "Directed"])]
    assert len(nd.Network(g, nd.diffusion_vertex(), [many[i % 3] for i in range(6)]).edge_batches) == 3
    # one batch per distinct closure value (pqnode_inhomogeneous), equal values share one
    big = nd.cycle_graph(40)
    buses = [nd.pqnode_inhomogeneous(-0.01 * (i % 30), -0.02) for i in range(40)]
    pg = nd.Network(big, buses, nd.piline())
    assert len(pg.vertex_batches) == 30 and pg.vertex_batch.tolist() == [i % 30 for i in range(40)]
    assert pg.pdim == 40 * 4 and pg.vertex_state_index(30) == 2


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_python_layout_matches_oracle_layout(seed):
    """The host-side layout of a batched network (Network.v_data / v_para / e_data / e_para)
    equals the oracle's restatement of register_vertices! / register_edges!
    (src/network_structure.jl:224-258) on random mixes of every kind and wrapper."""
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    g = nd.barabasi_albert(120, 3, seed=seed)
    vms = [nd.diffusion_vertex, nd.kuramoto_first, nd.kuramoto_second, nd.kuramoto_vertex_2d]
    ems = [nd.diffusion_edge, nd.diffusion_edge_unit, nd.kuramoto_edge, nd.diffusion_odeedge, nd.diffusion_dedge,
           nd.diffusion_edge_fid, lambda: nd.Symmetric(nd.kuramoto_edge()), lambda: nd.Directed(nd.diffusion_edge())]
    net = nd.Network(g, [vms[i]() for i in rng.integers(0, len(vms), g.nv)],
                     [ems[i]() for i in rng.integers(0, len(ems), g.ne)])
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, [m.kind for m in net.vertex_batches], net.vertex_batch,
                                      [(m.kind, nd.capi.COUPLINGS[m.coupling]) for m in net.edge_batches],
                                      net.edge_batch)
    assert (on.dim, on.pdim) == (net.dim, net.pdim)
    lib = on.lib
    assert [lib.nd_oracle_v_data(on.L, v) for v in range(g.nv)] == net.v_data.tolist()
    assert [lib.nd_oracle_v_para(on.L, v) for v in range(g.nv)] == net.v_para.tolist()
    assert [lib.nd_oracle_e_para(on.L, e) for e in range(g.ne)] == net.e_para.tolist()
    ode = [e for e in range(g.ne) if net.edge_batches[net.edge_batch[e]].dim == 2]
    assert [lib.nd_oracle_e_data(on.L, e) for e in ode] == net.e_data[ode].tolist()


def test_mass_matrix_like_construct_mass_matrix():
    """construct_mass_matrix (src/construction.jl:409-467): the identity (None) when no
    component has a mass matrix; otherwise each component's diagonal at its state range.
    The PQ bus is algebraic (mass matrix 0, benchmark/benchmark_models.jl:74)."""
    import dataclasses
    g = nd.watts_strogatz(12, 2, 0.3, seed=3)
    assert nd.Network(g, nd.kuramoto_second(), nd.static_line()).mass_matrix() is None
    vm = [nd.pqnode() if v % 3 == 0 else nd.generator() for v in range(g.nv)]
    net = nd.Network(g, vm, nd.piline())
    mm = net.mass_matrix()
    assert mm.shape == (net.dim,)
    for v in range(g.nv):
        s = net.vertex_state_index(v)
        want = [0.0, 0.0] if v % 3 == 0 else [1.0] * 4
        np.testing.assert_array_equal(mm[s:s + len(want)], want)
    # any library vertex can be made algebraic; it then forms a batch of its own
    alg = dataclasses.replace(nd.diffusion_vertex(), mass_matrix=0)
    vms = [alg if v in (2, 5) else nd.diffusion_vertex() for v in range(g.nv)]
    net = nd.Network(g, vms, nd.diffusion_edge())
    assert len(net.vertex_batches) == 2
    mm = net.mass_matrix()
    assert mm[net.vertex_state_index(2)] == 0 and mm[net.vertex_state_index(5)] == 0 and mm.sum() == g.nv - 2
    # per-state diagonals; a full matrix is rejected
    sw = dataclasses.replace(nd.kuramoto_second(), mass_matrix=[1.0, 0.5])
    net = nd.Network(g, sw, nd.static_line())
    np.testing.assert_array_equal(net.mass_matrix(), np.tile([1.0, 0.5], g.nv))
    bad = dataclasses.replace(nd.kuramoto_second(), mass_matrix=np.eye(2))
    with pytest.raises(nd.ArgumentError):
        nd.Network(g, bad, nd.static_line()).mass_matrix()


def test_execution_options_are_checked_and_kept():
    ex = nd.GB300Execution(sum_order="tree", layout="fused", kernel_timing=True)
    assert (ex.sum_order, ex.layout, ex.kernel_timing) == ("tree", "fused", True)
    assert repr(nd.GB300Execution()) == "GB300Execution()"
    assert repr(ex) == "GB300Execution(sum_order='tree', layout='fused', kernel_timing=True)"
    assert nd.GB300Execution() == nd.GB300Execution(sum_order="sequential")
    with pytest.raises(nd.ArgumentError):
        nd.GB300Execution(sum_order="pairwise")
    with pytest.raises(nd.ArgumentError):
        nd.GB300Execution(layout="blocked")
    nw = nd.Network(nd.cycle_graph(5), nd.diffusion_vertex(), nd.diffusion_edge(), execution=ex)
    assert nw.execution is ex


def test_ensemble_snapshot_files_round_trip(tmp_path):
    """EnsembleSolveResult.save_snapshot / load_snapshot: state and step control as .npy
    files, the snapshot time, and the refusal to save a solve without step control."""
    import torch
    from nd_gb300.ensemble import EnsembleSolveResult, load_snapshot
    u = torch.arange(6, dtype=torch.float64)
    control = torch.tensor([[2.0, 0.1, 1e-3], [2.0, 0.2, 2e-3]], dtype=torch.float64)
    res = EnsembleSolveResult(u, torch.zeros(2, dtype=torch.int32), torch.tensor([5, 7]), control)
    res.save_snapshot(tmp_path / "s")
    snap = load_snapshot(tmp_path / "s")
    np.testing.assert_array_equal(snap.u, u.numpy())
    np.testing.assert_array_equal(snap.control, control.numpy())
    assert snap.t == 2.0
    np.testing.assert_array_equal(np.load(tmp_path / "s" / "nsteps.npy"), [5, 7])
    with pytest.raises(nd.ArgumentError):
        EnsembleSolveResult(u, None, None).save_snapshot(tmp_path / "t")
