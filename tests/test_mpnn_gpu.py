"""The MPNN's CUDA forward, backward and Adam kernels against the float64 oracle, and
what the trained network gains as a Newton warm start."""
import numpy as np
import pytest

import nd_gb300 as nd
from nd_gb300 import warmstart as W
from oracle import mpnn_oracle as MO

pytestmark = pytest.mark.gpu


def _case(nv=200, L=4, B=3, seed=0):
    g = nd.barabasi_albert(nv, 2, seed=40 + seed)
    P, K = W.swing_instances(g, B, seed)
    rng = np.random.default_rng(seed)
    T = rng.normal(scale=0.3, size=(B, nv))
    params = MO.random_params(L, rng, scale=0.15).astype(np.float32)
    return g, P, K, T, params


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def test_forward_matches_oracle(cuda):
    g, P, K, T, params = _case()
    m = nd.MPNN(g, layers=4)
    assert m.nparams == MO.offsets(4)["n"]
    m.set_params(params)
    th = m.forward(P, K).cpu().numpy()
    ref = MO.forward(params.astype(np.float64), 4, g.nv, g.src, g.dst, P.astype(np.float32), K.astype(np.float32))
    np.testing.assert_allclose(th, ref, atol=2e-5 * np.abs(ref).max() + 1e-6)
    np.testing.assert_allclose(th.mean(axis=1), 0.0, atol=1e-5)


@pytest.mark.parametrize("layers,hops", [(1, 1), (4, 1), (2, 3)])
def test_gradients_match_oracle(cuda, layers, hops):
    """Every parameter group's gradient within 1e-4 (normwise, FP32 vs float64)."""
    g, P, K, T, params = _case(L=layers, seed=1)
    m = nd.MPNN(g, layers=layers, hops=hops)
    m.set_params(params)
    loss = float(m.loss_grad(P, K, T).item())
    grads = m.get_grads().cpu().numpy().astype(np.float64)
    l_ref, g_ref = MO.loss_grad(params.astype(np.float64), layers, g.nv, g.src, g.dst, P.astype(np.float32),
                                K.astype(np.float32), T.astype(np.float32), hops=hops)
    assert abs(loss - l_ref) <= 1e-5 * l_ref
    o = MO.offsets(layers)
    groups = [("W_in", 0, 128), ("b_in", 128, 192)]
    for l in range(layers):
        groups += [(f"W_s{l}", o[f"W_s{l}"], o[f"W_s{l}"] + 4096), (f"W_m{l}", o[f"W_m{l}"], o[f"W_m{l}"] + 4096),
                   (f"b{l}", o[f"b{l}"], o[f"b{l}"] + 64)]
    groups += [("w_out", o["w_out"], o["w_out"] + 64), ("b_out", o["b_out"], o["b_out"] + 1)]
    for name, lo, hi in groups:
        if np.linalg.norm(g_ref[lo:hi]) < 1e-12:
            np.testing.assert_allclose(grads[lo:hi], 0.0, atol=1e-7)
            continue
        assert _rel(grads[lo:hi], g_ref[lo:hi]) < 1e-4, name


def test_adam_step_matches_oracle(cuda):
    g, P, K, T, params = _case(seed=2)
    m = nd.MPNN(g, layers=4)
    m.set_params(params)
    p = params.astype(np.float64)
    mm, vv = np.zeros_like(p), np.zeros_like(p)
    for t in (1, 2, 3):
        m.loss_grad(P, K, T)
        grad = m.get_grads().cpu().numpy().astype(np.float64)
        m.adam_step(lr=1e-3)
        p, mm, vv = MO.adam(p, grad, mm, vv, t, lr=1e-3)
        got = m.get_params().cpu().numpy()
        np.testing.assert_allclose(got, p, rtol=0, atol=2e-6)


def test_training_is_deterministic_and_weights_round_trip(cuda, tmp_path):
    g = nd.barabasi_albert(150, 2, seed=7)
    P, K = W.swing_instances(g, 96, 7)
    T = np.random.default_rng(7).normal(scale=0.3, size=P.shape)
    runs = []
    for _ in range(2):
        m = nd.MPNN(g, layers=2, seed=11)
        hist = m.fit(P, K, T, epochs=2, batch=32, lr=1e-3)
        runs.append((hist, m.get_params().cpu().numpy()))
    assert runs[0][0] == runs[1][0]
    np.testing.assert_array_equal(runs[0][1], runs[1][1])
    path = tmp_path / "w.bin"
    m.save(path)
    m2 = nd.MPNN(g, layers=2, seed=99)
    m2.load(path)
    np.testing.assert_array_equal(m2.get_params().cpu().numpy(), runs[1][1])
    with pytest.raises(nd.ArgumentError):
        nd.MPNN(g, layers=3).load(path)


def test_bad_arguments_raise(cuda):
    g = nd.barabasi_albert(50, 2, seed=1)
    with pytest.raises(nd.ArgumentError):
        nd.MPNN(g, hidden=32)
    m = nd.MPNN(g)
    P, K = W.swing_instances(g, 2, 0)
    with pytest.raises(nd.ArgumentError):
        m.forward(P[:, :10], K)


def test_warm_start_gain(cuda):
    """What the trained network gains over the plain cold start θ = 0 on held-out
    instances of this small training run (BA(300, 2), 1536 instances, 40 epochs; measured
    on a GB300: prediction error 0.05 rad, Newton iterations 3.0 -> 3.0, CG iterations
    185 -> 168): a much closer initial guess, every warm-started Newton solve converging to
    1e-10 without the cold-start fallback, no more Newton iterations and at least 5 % fewer
    conjugate-gradient iterations.  The full benchmark (BA(2000, 2), 20,000 instances,
    80 epochs) reaches 3.00 -> 2.04 Newton iterations; one Newton iteration would need a
    prediction within ~1e-5 rad, which a 4-hop network cannot give."""
    g = nd.barabasi_albert(300, 2, seed=5)
    P, K = W.swing_instances(g, 1536 + 128, 5)
    train = W.fixpoints(g, P[:1536], K[:1536], tol=1e-10)
    assert (train.status == 0).all()
    m = nd.MPNN(g, layers=4, seed=1)
    hist = m.fit(P[:1536], K[:1536], train.theta, epochs=40, batch=32, lr=2e-3, lr_final=1e-4)
    assert hist[-1] < 0.1 * hist[0]
    res = W.warm_vs_cold(m, g, P[1536:], K[1536:], tol=1e-10)
    assert res["cold"]["converged"] == 128 and res["warm"]["converged"] == 128
    assert res["warm"]["fallbacks"] == 0
    cold_th = W.fixpoints(g, P[1536:], K[1536:]).theta
    zero_err = np.abs(cold_th - cold_th.mean(axis=1, keepdims=True)).max(axis=1).mean()
    assert res["prediction_max_abs_err"]["mean"] < 0.5 * zero_err
    assert res["warm"]["newton_iters_mean"] <= res["cold"]["newton_iters_mean"]
    assert res["cg_iter_ratio"] >= 1.05
