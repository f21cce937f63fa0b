"""External inputs and loopback edges, host side: the oracle's restatement of the two
core-loop copies on worked examples, and the host map builders with their argument
checks (no GPU)."""
import numpy as np
import pytest

import nd_gb300 as nd
from nd_gb300 import external as X
from oracle import oracle as O


def test_oracle_collect_externals_worked_example():
    u = np.array([10.0, 11.0, 12.0])
    o = np.array([20.0, 21.0])
    # ExtMap [StateBufIdx(3), OutBufIdx(1), StateBufIdx(1), OutBufIdx(2)] in 1-based Julia
    ext = O.collect_externals([1, 0, 1, 0], [2, 0, 0, 1], u, o)
    np.testing.assert_array_equal(ext, [12.0, 20.0, 10.0, 21.0])


def test_oracle_loopback_map_and_copy():
    # edges 0->1 (loopback), 1->2, 2->0 (loopback); vertex v has outputs [2v, 2v+1] and
    # aggregation slots [3v, 3v+1] (a third slot not fed back)
    src, dst = [0, 1, 2], [1, 2, 0]
    v_out = [[2 * v, 2 * v + 1] for v in range(3)]
    v_aggr = [[3 * v, 3 * v + 1] for v in range(3)]
    out_idx, agg_idx = O.gen_loopback_map(src, dst, [True, False, True], v_out, v_aggr)
    np.testing.assert_array_equal(out_idx, [2, 3, 0, 1])
    np.testing.assert_array_equal(agg_idx, [0, 1, 6, 7])
    agg = O.apply_loopback(np.zeros(9), np.arange(6.0) + 1, out_idx, agg_idx)
    np.testing.assert_array_equal(agg, [3, 4, 0, 0, 0, 0, 1, 2, 0])


def test_host_loopback_map_matches_oracle():
    rng = np.random.default_rng(0)
    g = nd.barabasi_albert(40, 2, seed=3)
    lb = rng.random(g.ne) < 0.3
    v_out = [range(2 * v, 2 * v + 2) for v in range(g.nv)]
    v_aggr = [range(5 * v + 1, 5 * v + 3) for v in range(g.nv)]
    m = X.gen_loopback_map(g.src, g.dst, lb, v_out, v_aggr, device="cpu")
    ro, ra = O.gen_loopback_map(g.src, g.dst, lb, v_out, v_aggr)
    np.testing.assert_array_equal(m.out_idx.numpy(), ro)
    np.testing.assert_array_equal(m.agg_idx.numpy(), ra)
    with pytest.raises(nd.ArgumentError):
        X.gen_loopback_map([0], [1], [True], [[0], [1, 2]], [[0], [1]], device="cpu")


def test_extmap_arguments():
    with pytest.raises(nd.ArgumentError, match="no external inputs"):
        X.ExtMap([], device="cpu")
    with pytest.raises(nd.ArgumentError):
        X.ExtMap([X.StateBufIdx(1), 3], device="cpu")
    with pytest.raises(nd.ArgumentError):
        X.ExtMap([X.OutBufIdx(-1)], device="cpu")
    m = X.ExtMap([X.StateBufIdx(4), X.OutBufIdx(2), X.StateBufIdx(0)], device="cpu")
    assert len(m) == 3 and m.max_state == 4 and m.max_out == 2
    assert m.from_state.tolist() == [1, 0, 1] and m.idx.tolist() == [4, 2, 0]
