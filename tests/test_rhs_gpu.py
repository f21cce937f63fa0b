"""Parity of the GB300 RHS (through the C ABI) with the CPU oracle.

Bars: FP64 diffusion is bitwise equal to SequentialExecution + SequentialAggregator
(same operations, same order, no FMA).  FP64 Kuramoto / swing differ only through the
sine (CUDA's vs libm's, each within 1 ulp): every entry must satisfy
|Δ| <= 1e-13 · |du| or, where the sum cancels, |Δ| <= 1e-13 · Σ|terms|.
FP32 is compared with the FP64 oracle: |Δ| <= 4e-6 · (Σ|terms| + |du|).
"""
import zlib

import numpy as np
import pytest

import nd_gb300 as nd
from oracle import oracle as O

from ndtest import exact_rows, gpu_rhs, random_inputs

pytestmark = pytest.mark.gpu

GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"

MODELS = {
    (O.V_DIFFUSION, O.E_DIFFUSION): (nd.diffusion_vertex, nd.diffusion_edge),
    (O.V_DIFFUSION, O.E_DIFFUSION_UNIT): (nd.diffusion_vertex, nd.diffusion_edge_unit),
    (O.V_KURAMOTO, O.E_KURAMOTO): (nd.kuramoto_first, nd.kuramoto_edge),
    (O.V_KURAMOTO, O.E_DIFFUSION): (nd.kuramoto_first, nd.diffusion_edge),
    (O.V_SWING, O.E_KURAMOTO): (nd.kuramoto_second, nd.static_line),
    (O.V_SWING, O.E_DIFFUSION): (nd.kuramoto_second, nd.diffusion_edge),
    (O.V_DIFFUSION, O.E_KURAMOTO): (nd.diffusion_vertex, nd.kuramoto_edge),
}

GRAPHS = {
    "ws1000": lambda: nd.watts_strogatz(1000, 10, 0.1, seed=1),
    "ba20k_m3": lambda: nd.barabasi_albert(20_000, 3, seed=2),
    "ba100k_m2": lambda: nd.barabasi_albert(100_000, 2, seed=3),
}


def make(g, vk, ek, dtype):
    import torch
    vm, em = MODELS[(vk, ek)]
    return nd.adapt(nd.Network(g, vm(), em()), torch.float64 if dtype == np.float64 else torch.float32)


def check_f64(got, ref, terms, exact):
    if exact:
        np.testing.assert_array_equal(got, ref)
        return
    d = np.abs(got - ref)
    ok = (d <= 1e-13 * np.abs(ref)) | (d <= 1e-13 * terms)
    assert ok.all(), f"{(~ok).sum()} entries off; worst {d[~ok].max():.3e}"


@pytest.mark.parametrize("gname", list(GRAPHS))
@pytest.mark.parametrize("vk,ek", list(MODELS))
def test_f64_parity(cuda, gname, vk, ek):
    g = GRAPHS[gname]()
    nw = make(g, vk, ek, np.float64)
    on = O.OracleNetwork.from_graph(g, vk, ek)
    rng = np.random.default_rng(zlib.crc32(f"{gname}-{vk}-{ek}".encode()))
    u, p = random_inputs(on, vk, rng)
    ref = on.rhs(u, p)
    got = gpu_rhs(nw, u, p, cuda, np.float64)
    exact = ek != O.E_KURAMOTO
    check_f64(got, ref, on.abs_terms(u, p), exact)


@pytest.mark.parametrize("gname", ["ws1000", "ba100k_m2"])
@pytest.mark.parametrize("vk,ek", [(O.V_DIFFUSION, O.E_DIFFUSION), (O.V_KURAMOTO, O.E_KURAMOTO),
                                   (O.V_SWING, O.E_KURAMOTO)])
def test_f32_against_f64_oracle(cuda, gname, vk, ek):
    g = GRAPHS[gname]()
    nw = make(g, vk, ek, np.float32)
    on = O.OracleNetwork.from_graph(g, vk, ek)
    u, p = random_inputs(on, vk, np.random.default_rng(5))
    u32, p32 = u.astype(np.float32), p.astype(np.float32)
    ref = on.rhs(u32.astype(np.float64), p32.astype(np.float64))
    got = gpu_rhs(nw, u32, p32, cuda, np.float32).astype(np.float64)
    terms = on.abs_terms(u32.astype(np.float64), p32.astype(np.float64))
    bound = 4e-6 * (terms + np.abs(ref))
    assert np.all(np.abs(got - ref) <= bound), np.max(np.abs(got - ref) / bound)


@pytest.mark.parametrize("layout", ["auto", "fused"])
def test_f32_heavy_rows_against_f64_oracle(cuda, layout):
    """FP32 with rows above the heavy-row degree (compensated block sums), on both layouts."""
    g = nd.simple_graph(6001, [(0, i) for i in range(1, 6001)] + [(i, i + 1) for i in range(1, 6000, 7)])
    for vk, ek in [(O.V_DIFFUSION, O.E_DIFFUSION), (O.V_SWING, O.E_KURAMOTO)]:
        nw = make(g, vk, ek, np.float32)
        nw.set_layout(layout)
        on = O.OracleNetwork.from_graph(g, vk, ek)
        u, p = random_inputs(on, vk, np.random.default_rng(9))
        u32, p32 = u.astype(np.float32), p.astype(np.float32)
        ref = on.rhs(u32.astype(np.float64), p32.astype(np.float64))
        got = gpu_rhs(nw, u32, p32, cuda, np.float32).astype(np.float64)
        terms = on.abs_terms(u32.astype(np.float64), p32.astype(np.float64))
        assert np.all(np.abs(got - ref) <= 4e-6 * (terms + np.abs(ref)))


def test_tree_order_is_deterministic_and_close(cuda):
    g = nd.barabasi_albert(50_000, 4, seed=11)
    nw = make(g, O.V_DIFFUSION, O.E_DIFFUSION, np.float64)
    nw.set_sum_order("tree")
    on = O.OracleNetwork.from_graph(g, O.V_DIFFUSION, O.E_DIFFUSION)
    u, p = random_inputs(on, O.V_DIFFUSION, np.random.default_rng(1))
    ref = on.rhs(u, p)
    runs = [gpu_rhs(nw, u, p, cuda, np.float64) for _ in range(5)]
    for r in runs[1:]:
        np.testing.assert_array_equal(r, runs[0])
    d = np.abs(runs[0] - ref)
    assert np.all(d <= 1e-13 * on.abs_terms(u, p))
    assert nw.info().sum_order == 1


def test_sequential_is_deterministic(cuda):
    g = nd.barabasi_albert(50_000, 4, seed=12)
    nw = make(g, O.V_KURAMOTO, O.E_KURAMOTO, np.float64)
    on = O.OracleNetwork.from_graph(g, O.V_KURAMOTO, O.E_KURAMOTO)
    u, p = random_inputs(on, O.V_KURAMOTO, np.random.default_rng(2))
    first = gpu_rhs(nw, u, p, cuda, np.float64)
    for _ in range(9):
        np.testing.assert_array_equal(gpu_rhs(nw, u, p, cuda, np.float64), first)


def test_golden_fixtures_on_gpu(cuda):
    d = np.load(GOLDEN / "diffusion_ba10_5.npz")
    g = nd.Graph(int(d["nv"]), d["src"], d["dst"])
    nw = make(g, O.V_DIFFUSION, O.E_DIFFUSION_UNIT, np.float64)
    for x, du in zip(d["x"], d["du"]):
        np.testing.assert_array_equal(gpu_rhs(nw, x, None, cuda, np.float64), du)
    d = np.load(GOLDEN / "kuramoto_ws1000.npz")
    g = nd.Graph(int(d["nv"]), d["src"], d["dst"])
    nw = make(g, O.V_KURAMOTO, O.E_KURAMOTO, np.float64)
    got = gpu_rhs(nw, d["u"], d["p"], cuda, np.float64)
    on = O.OracleNetwork.from_graph(g, O.V_KURAMOTO, O.E_KURAMOTO)
    check_f64(got, d["du"], on.abs_terms(d["u"], d["p"]), exact=False)
    d = np.load(GOLDEN / "swing_ba200.npz")
    g = nd.Graph(int(d["nv"]), d["src"], d["dst"])
    nw = make(g, O.V_SWING, O.E_KURAMOTO, np.float64)
    on = O.OracleNetwork.from_graph(g, O.V_SWING, O.E_KURAMOTO)
    check_f64(gpu_rhs(nw, d["u"], d["p"], cuda, np.float64), d["du"], on.abs_terms(d["u"], d["p"]), exact=False)


@pytest.mark.parametrize("kind", ["isolated", "no_edges", "star", "pair", "two_hubs"])
def test_edge_case_graphs(cuda, kind):
    if kind == "isolated":
        g = nd.simple_graph(50, [(0, 1), (1, 2), (10, 20)])
    elif kind == "no_edges":
        g = nd.simple_graph(7, [])
    elif kind == "star":
        g = nd.simple_graph(5001, [(0, i) for i in range(1, 5001)])
    elif kind == "pair":
        g = nd.simple_graph(2, [(0, 1)])
    else:
        g = nd.simple_graph(3000, [(0, i) for i in range(2, 3000)] + [(1, i) for i in range(2, 3000, 2)])
    for vk, ek in [(O.V_DIFFUSION, O.E_DIFFUSION), (O.V_SWING, O.E_KURAMOTO)]:
        nw = make(g, vk, ek, np.float64)
        on = O.OracleNetwork.from_graph(g, vk, ek)
        u, p = random_inputs(on, vk, np.random.default_rng(3))
        check_f64(gpu_rhs(nw, u, p, cuda, np.float64), on.rhs(u, p), on.abs_terms(u, p), exact=ek != O.E_KURAMOTO)


def test_wrong_precision_and_sizes_raise(cuda):
    """GPU_test.jl:63,70 (wrong eltype → ArgumentError) and coreloop.jl:2-7 (sizes)."""
    import torch
    g = nd.barabasi_albert(100, 2, seed=1)
    nw64 = make(g, O.V_KURAMOTO, O.E_KURAMOTO, np.float64)
    nw32 = make(g, O.V_KURAMOTO, O.E_KURAMOTO, np.float32)
    u32 = torch.zeros(nw64.dim, dtype=torch.float32, device=cuda)
    p32 = torch.zeros(nw64.pdim, dtype=torch.float32, device=cuda)
    du32 = torch.zeros_like(u32)
    with pytest.raises(nd.ArgumentError):
        nw64(du32, u32, p32, 0.0)
    u64, p64, du64 = u32.double(), p32.double(), du32.double()
    with pytest.raises(nd.ArgumentError):
        nw32(du64, u64, p64, 0.0)
    nw64(du64, u64, p64, 0.0)
    nw32(du32, u32, p32, 0.0)
    with pytest.raises(nd.ArgumentError):
        nw64(du64[:-1], u64[:-1], p64, 0.0)
    with pytest.raises(nd.ArgumentError):
        nw64(du64, u64, p64[:-1], 0.0)
    with pytest.raises(nd.ArgumentError):
        nw64(du64, u64, None, 0.0)
    with pytest.raises(nd.ArgumentError):
        nw64(du64.cpu(), u64, p64, 0.0)


def test_full_size_ba10m_against_oracle(cuda):
    """The headline workload, BA(1e7, m=4) diffusion with the benchmark's seeded inputs: the
    whole FP64 du equals the sequential oracle (SequentialExecution + SequentialAggregator)
    bit for bit, f(2u) == 2 f(u) bitwise, and the whole FP32 du is within
    4e-6 (Σ|terms| + |du|) of the FP64 oracle on the rounded inputs."""
    import torch
    g = nd.barabasi_albert(10_000_000, 4, seed=1)
    rng = np.random.default_rng(1)
    u = rng.normal(size=g.nv)
    p = rng.uniform(0.0, 1.0, size=g.ne)
    on = O.OracleNetwork.from_graph(g, O.V_DIFFUSION, O.E_DIFFUSION)
    nw = make(g, O.V_DIFFUSION, O.E_DIFFUSION, np.float64)
    du = gpu_rhs(nw, u, p, cuda, np.float64)
    np.testing.assert_array_equal(du, on.rhs(u, p))
    du2 = gpu_rhs(nw, 2.0 * u, p, cuda, np.float64)
    np.testing.assert_array_equal(du2, 2.0 * du)
    del nw
    torch.cuda.empty_cache()
    nw32 = make(g, O.V_DIFFUSION, O.E_DIFFUSION, np.float32)
    u32, p32 = u.astype(np.float32), p.astype(np.float32)
    got = gpu_rhs(nw32, u32, p32, cuda, np.float32).astype(np.float64)
    ref = on.rhs_poly(u32.astype(np.float64), p32.astype(np.float64))
    terms = on.abs_terms(u32.astype(np.float64), p32.astype(np.float64))
    d = np.abs(got - ref)
    ok = d <= 4e-6 * (terms + np.abs(ref))
    assert ok.all(), f"{(~ok).sum()} entries off; worst {d[~ok].max():.3e}"
    del nw32
    torch.cuda.empty_cache()


@pytest.mark.parametrize("vk,ek", [(O.V_DIFFUSION, O.E_DIFFUSION), (O.V_SWING, O.E_KURAMOTO)])
def test_exact_integer_sums_equal_hardware_sums(cuda, vk, ek):
    """The integer-exact adds / hub scan and hardware DADD chains give identical bits
    (both are the sequential order); heavy rows (degree > 2048) included."""
    g = nd.barabasi_albert(1_000_000, 4, seed=21)
    assert g.degree().max() > 2048
    nw = make(g, vk, ek, np.float64)
    on = O.OracleNetwork.from_graph(g, vk, ek)
    u, p = random_inputs(on, vk, np.random.default_rng(4))
    exact = gpu_rhs(nw, u, p, cuda, np.float64)
    nw.set_sum_order("sequential_hw")
    hw = gpu_rhs(nw, u, p, cuda, np.float64)
    np.testing.assert_array_equal(exact, hw)
    if ek != O.E_KURAMOTO:
        np.testing.assert_array_equal(exact, on.rhs(u, p))


@pytest.mark.parametrize("vk,ek", list(MODELS))
def test_two_phase_equals_fused_layout(cuda, vk, ek):
    """The edge-centric two-phase kernels and the fused kernel give identical bits, in every
    summation order (heavy rows included)."""
    g = nd.barabasi_albert(1_000_000, 4, seed=31)
    assert g.degree().max() > 2048
    nw = make(g, vk, ek, np.float64)
    on = O.OracleNetwork.from_graph(g, vk, ek)
    u, p = random_inputs(on, vk, np.random.default_rng(8))
    for order in ("sequential", "sequential_hw", "tree"):
        nw.set_sum_order(order)
        nw.set_layout("auto")
        a = gpu_rhs(nw, u, p, cuda, np.float64)
        nw.set_layout("fused")
        b = gpu_rhs(nw, u, p, cuda, np.float64)
        np.testing.assert_array_equal(a, b)
    nw.set_layout("auto")
    nw.set_sum_order("sequential")
    check_f64(gpu_rhs(nw, u, p, cuda, np.float64), on.rhs(u, p), on.abs_terms(u, p), exact=ek != O.E_KURAMOTO)


def test_kernel_counts_and_timing(cuda):
    """Each RHS launches edge phase + row phase (+ heavy rows on the side stream); the
    timer brackets each of them and leaves the results unchanged."""
    g = nd.barabasi_albert(1_000_000, 4, seed=31)
    assert g.degree().max() > 2048
    nw = make(g, O.V_DIFFUSION, O.E_DIFFUSION, np.float64)
    on = O.OracleNetwork.from_graph(g, O.V_DIFFUSION, O.E_DIFFUSION)
    u, p = random_inputs(on, O.V_DIFFUSION, np.random.default_rng(2))
    nw.kernel_times()
    ref = gpu_rhs(nw, u, p, cuda, np.float64)
    counts = nw.kernel_times()
    assert counts["edge_phase"][0] == 1 and counts["row_phase"][0] == 1 and counts["heavy_rows"][0] == 1
    assert counts["fused"][0] == 0 and all(ms == 0.0 for _, ms in counts.values())
    nw.set_kernel_timing(True)
    for _ in range(3):
        out = gpu_rhs(nw, u, p, cuda, np.float64)
        np.testing.assert_array_equal(out, ref)
    times = nw.kernel_times()
    for k in ("edge_phase", "row_phase", "heavy_rows"):
        assert times[k][0] == 3 and times[k][1] > 0.0
    nw.set_layout("fused")
    gpu_rhs(nw, u, p, cuda, np.float64)
    times = nw.kernel_times()
    assert times["fused"][0] == 1 and times["edge_phase"][0] == 0 and times["heavy_rows"][0] == 1
    nw.set_kernel_timing(False)


def test_non_canonical_edge_list_uses_fused_path(cuda):
    """Edges in arbitrary order and orientation (a directed edge list) are summed in the
    order the reference's output buffer has for them."""
    rng = np.random.default_rng(17)
    g0 = nd.barabasi_albert(20_000, 3, seed=5)
    perm = rng.permutation(g0.ne)
    flip = rng.random(g0.ne) < 0.5
    src = np.where(flip, g0.dst, g0.src)[perm]
    dst = np.where(flip, g0.src, g0.dst)[perm]
    g = nd.Graph(g0.nv, np.ascontiguousarray(src), np.ascontiguousarray(dst))
    for vk, ek in [(O.V_DIFFUSION, O.E_DIFFUSION), (O.V_SWING, O.E_KURAMOTO)]:
        nw = make(g, vk, ek, np.float64)
        on = O.OracleNetwork.from_graph(g, vk, ek)
        u, p = random_inputs(on, vk, rng)
        check_f64(gpu_rhs(nw, u, p, cuda, np.float64), on.rhs(u, p), on.abs_terms(u, p), exact=ek != O.E_KURAMOTO)


def test_edge_phase_sources_of_sparse_and_dense_chunks(cuda):
    """Edge chunks of very different shape: one 2048-edge chunk whose sources lie 12
    vertices apart (spanning ~18,000 vertices, one edge each) and dense chunks of 2-4 edges
    per source with empty source blocks in between.  Both give the oracle's bits."""
    rng = np.random.default_rng(23)
    nv = 40_000
    pairs = set()
    for i in range(1500):  # sources 0, 12, 24, ...: one chunk spans ~18,000 vertices
        pairs.add((12 * i, 39_000 + (i % 1000)))
    for s in range(20_000, 24_000):  # dense region: 2-4 edges per source, some sources empty
        if s % 7 == 0:
            continue
        for d in rng.choice(np.arange(s + 1, nv), size=rng.integers(2, 5), replace=False):
            pairs.add((s, int(d)))
    arr = np.array(sorted(pairs), dtype=np.int64)
    g = nd.Graph(nv, np.ascontiguousarray(arr[:, 0]), np.ascontiguousarray(arr[:, 1]))
    nw = make(g, O.V_DIFFUSION, O.E_DIFFUSION, np.float64)
    on = O.OracleNetwork.from_graph(g, O.V_DIFFUSION, O.E_DIFFUSION)
    u, p = random_inputs(on, O.V_DIFFUSION, rng)
    np.testing.assert_array_equal(gpu_rhs(nw, u, p, cuda, np.float64), on.rhs(u, p))


def test_execution_options_reach_the_handle(cuda):
    """GB300Execution(sum_order=..., layout=..., kernel_timing=...) configures the handle
    that adapt creates: the fused layout gives the two-phase bits, the tree order is
    reported by nd_get_info, and the kernels are timed."""
    import torch
    g = nd.barabasi_albert(1_000_000, 4, seed=12)
    assert g.degree().max() > 2048
    on = O.OracleNetwork.from_graph(g, O.V_DIFFUSION, O.E_DIFFUSION)
    u, p = random_inputs(on, O.V_DIFFUSION, np.random.default_rng(4))
    plain = nd.adapt(nd.Network(g, nd.diffusion_vertex(), nd.diffusion_edge()), torch.float64)
    ex = nd.GB300Execution(layout="fused", kernel_timing=True)
    fused = nd.adapt(nd.Network(g, nd.diffusion_vertex(), nd.diffusion_edge(), execution=ex), torch.float64)
    ref = gpu_rhs(plain, u, p, cuda, np.float64)
    np.testing.assert_array_equal(ref, on.rhs(u, p))
    np.testing.assert_array_equal(gpu_rhs(fused, u, p, cuda, np.float64), ref)
    t = fused.kernel_times()
    assert t["fused"][0] == 1 and t["fused"][1] > 0.0 and t["edge_phase"][0] == 0
    tree = nd.adapt(nd.Network(g, nd.diffusion_vertex(), nd.diffusion_edge(),
                               execution=nd.GB300Execution(sum_order="tree")), torch.float64)
    assert tree.info().sum_order == nd.capi.ND_ORDER_TREE and plain.info().sum_order == nd.capi.ND_ORDER_SEQUENTIAL
    got = gpu_rhs(tree, u, p, cuda, np.float64)
    # a hub of n terms summed in two orders differs by at most about n·eps·Σ|terms| (n < 4500)
    assert np.all(np.abs(got - ref) <= 1e-12 * on.abs_terms(u, p))


@pytest.mark.parametrize("vk,ek", [(O.V_SWING, O.E_KURAMOTO), (O.V_KURAMOTO, O.E_DIFFUSION)])
def test_dense_network_rows(cuda, vk, ek):
    """A dense graph (rows of ~900 terms carry every incidence) takes the dense-network row
    kernels: FP64 gives the fused layout's bits and the oracle within the sine bound, FP32
    (a warp per row) stays within the FP32 bound."""
    g = nd.watts_strogatz(1800, 900, 0.1, seed=21)
    assert g.degree().min() > 32
    on = O.OracleNetwork.from_graph(g, vk, ek)
    u, p = random_inputs(on, vk, np.random.default_rng(21))
    nw = make(g, vk, ek, np.float64)
    got = gpu_rhs(nw, u, p, cuda, np.float64)
    nw.set_layout("fused")
    np.testing.assert_array_equal(gpu_rhs(nw, u, p, cuda, np.float64), got)
    check_f64(got, on.rhs(u, p), on.abs_terms(u, p), exact=ek != O.E_KURAMOTO)
    nw32 = make(g, vk, ek, np.float32)
    u32, p32 = u.astype(np.float32), p.astype(np.float32)
    got32 = gpu_rhs(nw32, u32, p32, cuda, np.float32).astype(np.float64)
    ref = on.rhs(u32.astype(np.float64), p32.astype(np.float64))
    terms = on.abs_terms(u32.astype(np.float64), p32.astype(np.float64))
    assert np.all(np.abs(got32 - ref) <= 4e-6 * (terms + np.abs(ref)))
