"""The MPNN oracle's gradient against central finite differences (CPU, float64)."""
import numpy as np
import pytest

from oracle import mpnn_oracle as MO


def _tiny_case(seed=0, nv=9, L=2, B=2):
    rng = np.random.default_rng(seed)
    # a ring with two chords and one isolated vertex
    src = np.array([0, 1, 2, 3, 4, 5, 6, 0, 2])
    dst = np.array([1, 2, 3, 4, 5, 6, 0, 4, 6])
    P = rng.uniform(-1, 1, (B, nv))
    K = rng.uniform(5, 10, (B, src.size))
    T = rng.normal(size=(B, nv))
    params = MO.random_params(L, rng, scale=0.2)
    return params, L, nv, src, dst, P, K, T


@pytest.mark.parametrize("hops", [1, 3])
def test_gradient_matches_finite_differences(hops):
    params, L, nv, src, dst, P, K, T = _tiny_case()
    loss, g = MO.loss_grad(params, L, nv, src, dst, P, K, T, hops=hops)
    assert np.isclose(loss, MO.loss_only(params, L, nv, src, dst, P, K, T, hops=hops), rtol=1e-14)
    rng = np.random.default_rng(1)
    o = MO.offsets(L)
    # every parameter group, a few coordinates each
    picks = [0, 1, o["b_in"], o["b_in"] + 5, o["W_s0"] + 3, o["W_m0"] + 70, o["b0"] + 2, o["W_s1"] + 4000,
             o["W_m1"] + 17, o["b1"] + 63, o["w_out"], o["w_out"] + 40, o["b_out"]]
    picks += list(rng.integers(0, o["n"], 12))
    eps = 1e-6
    for j in picks:
        pp, pm = params.copy(), params.copy()
        pp[j] += eps
        pm[j] -= eps
        fd = (MO.loss_only(pp, L, nv, src, dst, P, K, T, hops=hops) -
              MO.loss_only(pm, L, nv, src, dst, P, K, T, hops=hops)) / (2 * eps)
        assert abs(fd - g[j]) <= 1e-7 + 1e-5 * abs(fd), (j, fd, g[j])


def test_prediction_is_centred_and_shift_free():
    params, L, nv, src, dst, P, K, T = _tiny_case(3)
    th = MO.forward(params, L, nv, src, dst, P, K)
    np.testing.assert_allclose(th.mean(axis=1), 0.0, atol=1e-14)
    # the loss ignores a uniform shift of the target (phases are defined up to one)
    l0, _ = MO.loss_grad(params, L, nv, src, dst, P, K, T)
    l1, _ = MO.loss_grad(params, L, nv, src, dst, P, K, T + 3.0)
    assert np.isclose(l0, l1, rtol=1e-12)


def test_adam_first_step_moves_by_lr():
    p = np.zeros(4)
    g = np.array([1.0, -2.0, 0.5, 0.0])
    p1, m, v = MO.adam(p, g, np.zeros(4), np.zeros(4), 1, lr=0.01)
    np.testing.assert_allclose(p1[:3], -0.01 * np.sign(g[:3]), rtol=1e-6)
    assert p1[3] == 0.0
