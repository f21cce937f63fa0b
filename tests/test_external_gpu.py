"""External-input and loopback gathers on the GPU (nd_collect_externals, nd_apply_loopback)
against the oracle's restatement, bit for bit: the reference's ExtMap test
(test/external_inputs_test.jl:11-33: 10,000 shuffled StateBufIdx / OutBufIdx entries,
Float64 and Float32 device buffers equal to the CPU gather), repeated sources, an empty
loopback map and the host-side argument checks."""
import numpy as np
import pytest

import nd_gb300 as nd
from nd_gb300 import external as X
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_collect_externals_shuffled_map(cuda, dtype):
    import torch
    td = getattr(torch, dtype)
    rng = np.random.default_rng(0)
    N = 10_000
    u, o = rng.random(N).astype(dtype), rng.random(N).astype(dtype)
    entries = [X.StateBufIdx(i) if rng.random() < 0.5 else X.OutBufIdx(i) for i in range(N)]
    entries = [entries[i] for i in rng.permutation(N)]
    m = X.ExtMap(entries)
    ext = torch.full((N,), float("nan"), dtype=td, device="cuda")
    X.collect_externals(m, ext, torch.from_numpy(u).cuda(), torch.from_numpy(o).cuda())
    want = O.collect_externals([isinstance(e, X.StateBufIdx) for e in entries], [e.idx for e in entries], u, o)
    np.testing.assert_array_equal(ext.cpu().numpy(), want)


def test_collect_externals_repeated_and_all_one_kind(cuda):
    import torch
    rng = np.random.default_rng(1)
    u, o = rng.normal(size=50), rng.normal(size=7)
    for entries in ([X.StateBufIdx(int(i)) for i in rng.integers(0, 50, 300)],
                    [X.OutBufIdx(int(i)) for i in rng.integers(0, 7, 300)],
                    [X.OutBufIdx(3)]):
        m = X.ExtMap(entries)
        ext = torch.empty(len(entries), dtype=torch.float64, device="cuda")
        X.collect_externals(m, ext, torch.from_numpy(u).cuda(), torch.from_numpy(o).cuda())
        want = O.collect_externals([isinstance(e, X.StateBufIdx) for e in entries], [e.idx for e in entries], u, o)
        np.testing.assert_array_equal(ext.cpu().numpy(), want)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_apply_loopback_matches_oracle(cuda, dtype):
    import torch
    td = getattr(torch, dtype)
    rng = np.random.default_rng(2)
    g = nd.barabasi_albert(2000, 3, seed=9)
    lb = rng.random(g.ne) < 0.25
    # each vertex is the source of at most one loopback edge, so no aggregation slot is
    # written twice (the reference's injector/satellite pairs have the same property)
    seen = set()
    for e in range(g.ne):
        if lb[e] and int(g.src[e]) in seen:
            lb[e] = False
        elif lb[e]:
            seen.add(int(g.src[e]))
    v_out = [range(2 * v, 2 * v + 2) for v in range(g.nv)]
    v_aggr = [range(3 * v, 3 * v + 2) for v in range(g.nv)]
    m = X.gen_loopback_map(g.src, g.dst, lb, v_out, v_aggr)
    obuf = rng.normal(size=2 * g.nv).astype(dtype)
    agg0 = rng.normal(size=3 * g.nv).astype(dtype)
    agg = torch.from_numpy(agg0).cuda()
    X.apply_loopback(agg, torch.from_numpy(obuf).cuda(), m)
    want = O.apply_loopback(agg0, obuf, m.out_idx.cpu().numpy(), m.agg_idx.cpu().numpy())
    np.testing.assert_array_equal(agg.cpu().numpy(), want)
    assert (agg.cpu().numpy() != agg0).sum() > 0


def test_empty_loopback_map_and_argument_checks(cuda):
    import torch
    m = X.gen_loopback_map([0, 1], [1, 2], [False, False], [[0], [1], [2]], [[0], [1], [2]])
    agg = torch.arange(3.0, dtype=torch.float64, device="cuda")
    X.apply_loopback(agg, torch.zeros(3, dtype=torch.float64, device="cuda"), m)
    assert agg.tolist() == [0.0, 1.0, 2.0]
    em = X.ExtMap([X.StateBufIdx(5)])
    f64 = lambda n: torch.zeros(n, dtype=torch.float64, device="cuda")
    with pytest.raises(nd.ArgumentError):
        X.collect_externals(em, f64(1), f64(5), f64(5))            # index 5 outside u
    with pytest.raises(nd.ArgumentError):
        X.collect_externals(em, f64(2), f64(6), f64(6))            # extbuf length
    with pytest.raises(nd.ArgumentError):
        X.collect_externals(em, f64(1).float(), f64(6), f64(6))    # dtype mix
    with pytest.raises(nd.ArgumentError):
        X.collect_externals(em, torch.zeros(1, dtype=torch.int64, device="cuda"), f64(6), f64(6))
    lm = X.gen_loopback_map([0], [1], [True], [[0], [9]], [[0], [1]])
    with pytest.raises(nd.ArgumentError):
        X.apply_loopback(f64(3), f64(3), lm)                        # out index 9 outside obuf
    # the C ABI rejects what the host did not check
    lib = nd.capi.load()
    assert lib.nd_collect_externals(7, 1, None, None, None, None, None, None) == nd.capi.ND_ERR_DTYPE
    assert lib.nd_collect_externals(nd.capi.ND_F64, -1, None, None, None, None, None, None) == nd.capi.ND_ERR_ARG
    assert lib.nd_collect_externals(nd.capi.ND_F64, 0, None, None, None, None, None, None) == nd.capi.ND_OK
    assert lib.nd_apply_loopback(nd.capi.ND_F64, 3, None, None, None, None, None) == nd.capi.ND_ERR_ARG
