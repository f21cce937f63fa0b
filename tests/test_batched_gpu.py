"""Batched networks on the GPU (several vertex / edge batches, ODE edges, Symmetric /
Directed / Fiducial outputs) against the CPU oracle, through the C ABI.

Bars: without transcendental functions the FP64 RHS equals the oracle bit for bit in the
sequential orders (exact and hardware adds), rows of every length included; with sines
(CUDA's vs libm's, each within 1 ulp) every entry is within 1.6e-15 · (terms + 4) · scale.
FP32 follows the reference's GPU test: isapprox with rtol √eps(Float32), normwise.
"""
import numpy as np
import pytest

import nd_gb300 as nd
from nd_gb300 import _capi as capi
from nd_gb300.solve import solve_tsit5
from oracle import oracle as O

from ndtest import gpu_rhs

pytestmark = pytest.mark.gpu

VERTEX = {O.V_DIFFUSION: nd.diffusion_vertex, O.V_KURAMOTO: nd.kuramoto_first, O.V_SWING: nd.kuramoto_second,
          O.V_SWING_UNIT: nd.kuramoto_vertex_2d}
STATIC = {O.E_DIFFUSION: nd.diffusion_edge, O.E_DIFFUSION_UNIT: nd.diffusion_edge_unit, O.E_KURAMOTO: nd.kuramoto_edge}
WRAP = {O.C_ANTISYMMETRIC: nd.AntiSymmetric, O.C_SYMMETRIC: nd.Symmetric, O.C_DIRECTED: nd.Directed}


def edge_model(kind, coupling):
    if kind == O.E_DIFFUSION_ODE:
        return nd.diffusion_odeedge()
    if kind == O.E_DIFFUSION_ODE_FIXED:
        return nd.diffusion_dedge()
    if coupling == O.C_FIDUCIAL:
        return nd.diffusion_edge_fid()
    return WRAP[coupling](STATIC[kind]())


def build(g, vkinds, ebatches, vassign, eassign):
    """Network with the given vertex kinds / edge (kind, coupling) pairs assigned per
    component, and the oracle with the same batches."""
    vm = [VERTEX[vkinds[i]]() for i in vassign]
    em = [edge_model(*ebatches[i]) for i in eassign]
    nw = nd.Network(g, vm, em)
    vb = [m.kind for m in nw.vertex_batches]
    eb = [(m.kind, capi.COUPLINGS[m.coupling]) for m in nw.edge_batches]
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, nw.vertex_batch, eb, nw.edge_batch)
    assert (on.dim, on.pdim) == (nw.dim, nw.pdim)
    return nw, on


def adapt(nw, dtype):
    import torch
    return nd.adapt(nw, torch.float64 if dtype == np.float64 else torch.float32)


def check_sine_f64(got, ref, g, nw, u, p):
    """Each sine may differ by 1 ulp between CUDA and libm; the differences pass through
    the same sequence of additions.  Bound: 1.6e-15 · (terms of the entry + 4) · scale."""
    deg = np.bincount(np.concatenate([g.src, g.dst]), minlength=g.nv).astype(np.float64)
    terms = np.full(nw.dim, 4.0)
    terms[nw.v_data] += deg
    two = np.array([m.dim for m in nw.vertex_batches])[nw.vertex_batch] == 2
    terms[nw.v_data[two] + 1] += deg[two]
    scale = max(1.0, np.abs(u).max(), np.abs(p).max() if len(p) else 1.0, np.abs(ref).max())
    d = np.abs(got - ref)
    ok = d <= 1.6e-15 * terms * scale
    assert ok.all(), f"{(~ok).sum()} entries off; worst {d.max():.3e}"


def check_f32_isapprox(got, ref):
    # isapprox(a, b) of the reference's test: norm(a - b) <= sqrt(eps(Float32)) * max(norm(a), norm(b))
    assert np.linalg.norm(got - ref) <= np.sqrt(np.finfo(np.float32).eps) * max(np.linalg.norm(got),
                                                                                  np.linalg.norm(ref))


def test_reference_gpu_test_network(cuda):
    """test/GPU_test.jl:12-70: complete_graph(4) with swing / diffusion vertices and ODE,
    Kuramoto and two-sided Fiducial edges, x0 and p uniform in [0, 1); Float32 and Float64
    handles against the sequential CPU result, and the precision mismatch error."""
    import torch
    g = nd.complete_graph(4)
    vf = [nd.kuramoto_second(), nd.diffusion_vertex(), nd.kuramoto_second(), nd.diffusion_vertex()]
    ef = [nd.diffusion_odeedge(), nd.kuramoto_edge(), nd.kuramoto_edge(), nd.diffusion_edge_fid(),
          nd.diffusion_odeedge(), nd.diffusion_edge_fid()]
    nw = nd.Network(g, vf, ef)
    vb = [m.kind for m in nw.vertex_batches]
    eb = [(m.kind, capi.COUPLINGS[m.coupling]) for m in nw.edge_batches]
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, nw.vertex_batch, eb, nw.edge_batch)
    rng = np.random.default_rng(1)
    x0 = rng.random(nw.dim)
    p = rng.random(nw.pdim)
    dx = on.rhs(x0, p)
    nw1, nw2 = adapt(nw, np.float32), adapt(nw, np.float64)
    info = nw2.info()
    assert (info.n_vertex_batches, info.n_edge_batches, info.dim, info.pdim) == (2, 3, 10, 12)
    d1 = gpu_rhs(nw1, x0, p, cuda, np.float32)
    check_f32_isapprox(d1.astype(np.float64), dx)
    d2 = gpu_rhs(nw2, x0, p, cuda, np.float64)
    check_sine_f64(d2, dx, g, nw, x0, p)
    with pytest.raises(nd.ArgumentError):      # wrong type for the cache (GPU_test.jl:63, 70)
        gpu_rhs(nw2, x0, p, cuda, np.float32)
    with pytest.raises(nd.ArgumentError):
        gpu_rhs(nw1, x0, p, cuda, np.float64)
    # the JVP of a batched network (assembled Jacobian times v) against central differences
    u = torch.from_numpy(x0).to(cuda)
    v = rng.normal(size=nw.dim)
    jv = torch.empty_like(u)
    nd.jvp(nw2, jv, u, torch.from_numpy(p).to(cuda), torch.from_numpy(v).to(cuda))
    h = 1e-6
    fd = (on.rhs(x0 + h * v, p) - on.rhs(x0 - h * v, p)) / (2 * h)
    np.testing.assert_allclose(jv.cpu().numpy(), fd, rtol=1e-6, atol=1e-7)


VKINDS = [O.V_SWING, O.V_DIFFUSION, O.V_KURAMOTO, O.V_SWING_UNIT]
ALL_EDGES = [(O.E_DIFFUSION, O.C_ANTISYMMETRIC), (O.E_DIFFUSION_UNIT, O.C_SYMMETRIC), (O.E_KURAMOTO, O.C_DIRECTED),
             (O.E_DIFFUSION_ODE, O.C_FIDUCIAL), (O.E_DIFFUSION, O.C_FIDUCIAL), (O.E_KURAMOTO, O.C_ANTISYMMETRIC),
             (O.E_DIFFUSION_ODE_FIXED, O.C_FIDUCIAL), (O.E_DIFFUSION_UNIT, O.C_DIRECTED),
             (O.E_KURAMOTO, O.C_SYMMETRIC)]
NO_SINE = [(O.E_DIFFUSION, O.C_ANTISYMMETRIC), (O.E_DIFFUSION_UNIT, O.C_SYMMETRIC), (O.E_DIFFUSION, O.C_DIRECTED),
           (O.E_DIFFUSION, O.C_FIDUCIAL), (O.E_DIFFUSION_UNIT, O.C_ANTISYMMETRIC)]


@pytest.mark.parametrize("nv,m,seed", [(300, 3, 0), (5000, 4, 1), (40_000, 2, 2)])
def test_random_batched_parity(cuda, nv, m, seed):
    """All vertex kinds and all (edge kind, coupling) pairs mixed at random on BA graphs,
    whose hubs exceed the one-thread row length (warp rows)."""
    g = nd.barabasi_albert(nv, m, seed=seed)
    rng = np.random.default_rng(seed)
    nw, on = build(g, VKINDS, ALL_EDGES, vassign=rng.integers(0, 4, g.nv),
                   eassign=rng.integers(0, len(ALL_EDGES), g.ne))
    assert len(nw.vertex_batches) == 4 and len(nw.edge_batches) == len(ALL_EDGES)
    u = rng.normal(size=nw.dim)
    p = rng.uniform(0.5, 1.5, size=nw.pdim)
    ref = on.rhs(u, p)
    nw64, nw32 = adapt(nw, np.float64), adapt(nw, np.float32)
    # FP32 rows of 65+ terms take a warp each; FP64 rows only beyond 2048 terms
    assert (nw32.info().n_hubs > 0) == (nv >= 5000) and nw64.info().n_hubs == 0
    check_sine_f64(gpu_rhs(nw64, u, p, cuda, np.float64), ref, g, nw, u, p)
    got32 = gpu_rhs(nw32, u, p, cuda, np.float32).astype(np.float64)
    check_f32_isapprox(got32, ref)
    np.testing.assert_allclose(got32, ref, rtol=2e-4, atol=2e-4 * (1 + np.abs(ref).max()))


def star_with_ring(n):
    """Vertex 0 linked to all others (a row of n - 1 terms), the others on a ring."""
    src = np.concatenate([np.zeros(n - 1, dtype=np.int64), np.arange(1, n - 1)])
    dst = np.concatenate([np.arange(1, n), np.arange(2, n)])
    return nd.Graph(n, src, dst)


@pytest.mark.parametrize("graph", ["ba20k", "dense_ws1500", "star6000"])
@pytest.mark.parametrize("order", ["sequential", "sequential_hw"])
def test_batched_without_sine_bitwise(cuda, order, graph):
    """Power-law hubs, a dense graph (rows of ~1400 terms), and a hub of 5999 terms that
    takes the warp-row path and spans several shared-memory tiles of its exact scan."""
    g = {"ba20k": lambda: nd.barabasi_albert(20_000, 3, seed=7),
         "dense_ws1500": lambda: nd.watts_strogatz(1500, 1400, 0.1, seed=7),
         "star6000": lambda: star_with_ring(6000)}[graph]()
    rng = np.random.default_rng(7)
    nw, on = build(g, VKINDS, NO_SINE, vassign=rng.integers(0, 4, g.nv), eassign=rng.integers(0, len(NO_SINE), g.ne))
    u = rng.normal(size=nw.dim)
    p = rng.uniform(0.5, 1.5, size=nw.pdim)
    nw64 = adapt(nw, np.float64)
    assert nw64.info().n_hubs == (1 if graph == "star6000" else 0)
    nw64.set_sum_order(order)
    np.testing.assert_array_equal(gpu_rhs(nw64, u, p, cuda, np.float64), on.rhs(u, p))


def test_batched_tree_order_close(cuda):
    g = star_with_ring(6000)
    rng = np.random.default_rng(8)
    nw, on = build(g, VKINDS, NO_SINE, vassign=rng.integers(0, 4, g.nv), eassign=rng.integers(0, len(NO_SINE), g.ne))
    u = rng.normal(size=nw.dim)
    p = rng.uniform(0.5, 1.5, size=nw.pdim)
    nw64 = adapt(nw, np.float64)
    nw64.set_sum_order("tree")
    got, ref = gpu_rhs(nw64, u, p, cuda, np.float64), on.rhs(u, p)
    check_sine_f64(got, ref, g, nw, u, p)


@pytest.mark.parametrize("case", ["diffusion_static_edge", "diffusion_ode_edge", "kuramoto_homogeneous",
                                  "kuramoto_heterogeneous"])
def test_reference_benchmark_cases(cuda, case):
    """The reference's benchmark networks (benchmark/benchmark_cases.jl:20-66) at their
    smallest size, with a seeded graph of the same kind."""
    N = 100
    rng = np.random.default_rng(11)
    if case.startswith("diffusion"):
        g = nd.watts_strogatz(N, N // 2, 0.0, seed=1)
        em = nd.diffusion_edge_unit() if case == "diffusion_static_edge" else nd.diffusion_dedge()
        nw = nd.Network(g, nd.diffusion_vertex(), em)
    else:
        g = nd.watts_strogatz(N, 4, 0.8, seed=1)
        if case == "kuramoto_homogeneous":
            vm = nd.kuramoto_vertex_2d()
        else:
            kinds = rng.permutation(np.repeat([0, 1], N // 2))
            vm = [nd.kuramoto_vertex_1d() if k == 0 else nd.kuramoto_vertex_2d() for k in kinds]
        nw = nd.Network(g, vm, nd.static_kuramoto_edge())
    vb = [m.kind for m in nw.vertex_batches]
    eb = [(m.kind, capi.COUPLINGS[m.coupling]) for m in nw.edge_batches]
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, nw.vertex_batch, eb, nw.edge_batch)
    u = rng.normal(size=nw.dim)
    p = rng.uniform(0.5, 1.5, size=nw.pdim)
    ref = on.rhs(u, p)
    got = gpu_rhs(adapt(nw, np.float64), u, p, cuda, np.float64)
    if case == "diffusion_static_edge":
        np.testing.assert_array_equal(got, ref)
    else:
        check_sine_f64(got, ref, g, nw, u, p)


@pytest.mark.parametrize("case,N", __import__("bench").CASES)
def test_reference_benchmark_cases_at_timed_size(cuda, case, N):
    """The six reference benchmark networks exactly as `bench.py --cases` times them (largest
    N, same graphs and inputs), FP64 and FP32 against the oracle: bitwise where no
    transcendental function enters, within the sine / cos bounds elsewhere, FP32 by the
    reference's isapprox."""
    import bench
    g, vm, em = bench._case_networks(N, case)
    net = nd.Network(g, vm, em)
    u, p = bench.case_inputs(case, net, g)
    vb = [m.kind for m in net.vertex_batches]
    eb = [(m.kind, capi.COUPLINGS[m.coupling]) for m in net.edge_batches]
    consts = [m.constants or (0.0, 0.0) for m in net.vertex_batches]
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, net.vertex_batch, eb, net.edge_batch,
                                      vertex_constants=consts)
    ref = on.rhs_poly(u, p)
    got = gpu_rhs(adapt(net, np.float64), u, p, cuda, np.float64)
    if case == "diffusion_static_edge":
        np.testing.assert_array_equal(got, ref)
    elif case.startswith("powergrid"):
        assert np.max(np.abs(got - ref) / (1 + np.abs(ref))) < 1e-12
    else:
        check_sine_f64(got, ref, g, net, u, p)
    got32 = gpu_rhs(adapt(net, np.float32), u, p, cuda, np.float32).astype(np.float64)
    check_f32_isapprox(got32, ref)


def test_kernel_counts_of_batched_rhs(cuda):
    g = nd.barabasi_albert(2000, 3, seed=3)
    rng = np.random.default_rng(3)
    nw, _ = build(g, VKINDS, ALL_EDGES, vassign=rng.integers(0, 4, g.nv), eassign=rng.integers(0, len(ALL_EDGES), g.ne))
    nw64 = adapt(nw, np.float64)
    nw64.set_kernel_timing(True)
    u = rng.normal(size=nw.dim)
    p = rng.uniform(0.5, 1.5, size=nw.pdim)
    for _ in range(3):
        gpu_rhs(nw64, u, p, cuda, np.float64)
    kt = nw64.kernel_times()
    assert kt["batched_edges"][0] == 3 and kt["batched_rows"][0] == 3
    assert kt["edge_phase"][0] == kt["row_phase"][0] == kt["fused"][0] == kt["heavy_rows"][0] == 0
    assert kt["batched_edges"][1] > 0 and kt["batched_rows"][1] > 0


def test_tsit5_with_ode_edges_matches_oracle(cuda):
    """Tsit5 on the GPU through a batched network (Kuramoto and diffusion vertices, ODE
    and static edges) follows the oracle's Tsit5 step for step."""
    g = nd.watts_strogatz(200, 6, 0.2, seed=4)
    rng = np.random.default_rng(4)
    nw, on = build(g, [O.V_KURAMOTO, O.V_DIFFUSION],
                   [(O.E_DIFFUSION_ODE, O.C_FIDUCIAL), (O.E_KURAMOTO, O.C_ANTISYMMETRIC)],
                   vassign=rng.integers(0, 2, g.nv), eassign=rng.integers(0, 2, g.ne))
    u0 = rng.normal(size=nw.dim)
    p = nw.pflat(vertex={"ω": rng.normal(size=g.nv)}, edge={"τ": 0.5, "K": 2.0})
    u, st = solve_tsit5(adapt(nw, np.float64), u0, p, (0.0, 2.0), reltol=1e-8, abstol=1e-10)
    ref, rst = on.tsit5(u0, p, 0.0, 2.0, reltol=1e-8, abstol=1e-10)
    assert st.status == 0 and rst.status == 0
    assert abs(st.naccept - rst.naccept) <= 1 and abs(st.nreject - rst.nreject) <= 1
    np.testing.assert_allclose(u.cpu().numpy(), ref, rtol=1e-7, atol=1e-7)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_device_sine_is_odd(cuda, dtype):
    """The ODE edge evaluates sin(vs - vd) once and uses its negation for sin(vd - vs): the
    same bits only if the device sine is exactly odd (vd - vs is exactly -(vs - vd) in
    IEEE arithmetic).  Checked on the device over 2^22 arguments of every magnitude."""
    import torch
    dt = getattr(torch, dtype)
    g = torch.Generator(device=cuda).manual_seed(0)
    mag = torch.pow(10.0, torch.empty(1 << 22, device=cuda, dtype=torch.float64).uniform_(-12, 6, generator=g))
    x = (mag * torch.empty_like(mag).uniform_(1, 2, generator=g)).to(dt)
    assert torch.equal(torch.sin(-x), -torch.sin(x))


def test_batched_errors(cuda):
    import torch
    g = nd.cycle_graph(6)
    with pytest.raises(nd.UnsupportedComponentError):
        nd.Directed(nd.diffusion_edge_fid())
    many = [nd.kuramoto_first()] * 6
    nw = adapt(nd.Network(g, many, [nd.diffusion_odeedge()] * 6), np.float64)
    assert nw.info().n_edge_batches == 1 and nw.dim == 6 + 12
    du = torch.empty(nw.dim - 1, dtype=torch.float64, device=cuda)
    u = torch.zeros(nw.dim - 1, dtype=torch.float64, device=cuda)
    p = torch.ones(nw.pdim, dtype=torch.float64, device=cuda)
    with pytest.raises(nd.ArgumentError):
        nw(du, u, p)


def powergrid_network(nv, seed, pq_only=False):
    g = nd.watts_strogatz(nv, 4, 0.5, seed=seed)
    rng = np.random.default_rng(seed)
    kinds = np.zeros(nv, dtype=int) if pq_only else rng.integers(0, 2, nv)
    vm = [nd.pqnode() if k == 0 else nd.generator() for k in kinds]
    net = nd.Network(g, vm, nd.piline())
    vb = [m.kind for m in net.vertex_batches]
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, net.vertex_batch, [(O.E_PILINE, O.C_FIDUCIAL)],
                                      net.edge_batch)
    return g, net, on


@pytest.mark.parametrize("nv", [300, 20_000])
def test_powergrid_parity(cuda, nv):
    """PQ buses, generators and π-lines (benchmark/benchmark_cases.jl:68-79): complex
    outputs on the GPU against the oracle.  Without generators there is no transcendental
    function and the FP64 result is bitwise; generators differ through cos / sin."""
    for pq_only in (True, False):
        g, net, on = powergrid_network(nv, 3, pq_only)
        rng = np.random.default_rng(4)
        u, p = rng.normal(size=net.dim), rng.uniform(0.5, 1.5, size=net.pdim)
        ref = on.rhs(u, p)
        got = gpu_rhs(adapt(net, np.float64), u, p, cuda, np.float64)
        if pq_only:
            np.testing.assert_array_equal(got, ref)
        else:
            assert np.max(np.abs(got - ref) / (1 + np.abs(ref))) < 1e-12
        got32 = gpu_rhs(adapt(net, np.float32), u, p, cuda, np.float32).astype(np.float64)
        check_f32_isapprox(got32, ref)


def test_inhomogeneous_pq_parity(cuda):
    """powergrid_inhomogeneous_pq (benchmark/benchmark_cases.jl:82-102): half the buses are
    PQ buses closing over their own P, Q (one batch each, ~1500 batches), half generators."""
    nv = 3000
    g = nd.watts_strogatz(nv, 4, 0.5, seed=6)
    rng = np.random.default_rng(6)
    gen = rng.permutation(np.repeat([False, True], nv // 2))
    vm = [nd.generator() if x else nd.pqnode_inhomogeneous(-rng.random(), -rng.random()) for x in gen]
    net = nd.Network(g, vm, nd.piline())
    assert len(net.vertex_batches) == nv // 2 + 1
    vb = [m.kind for m in net.vertex_batches]
    consts = [m.constants or (0.0, 0.0) for m in net.vertex_batches]
    on = O.OracleNetwork.from_batches(g.nv, g.src, g.dst, vb, net.vertex_batch, [(O.E_PILINE, O.C_FIDUCIAL)],
                                      net.edge_batch, vertex_constants=consts)
    assert (on.dim, on.pdim) == (net.dim, net.pdim)
    u, p = rng.normal(size=net.dim), rng.uniform(0.5, 1.5, size=net.pdim)
    ref = on.rhs(u, p)
    got = gpu_rhs(adapt(net, np.float64), u, p, cuda, np.float64)
    assert np.max(np.abs(got - ref) / (1 + np.abs(ref))) < 1e-12
    check_f32_isapprox(gpu_rhs(adapt(net, np.float32), u, p, cuda, np.float32).astype(np.float64), ref)
