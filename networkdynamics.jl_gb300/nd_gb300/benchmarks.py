"""Secondary GPU benchmarks of the package (the headline RHS benchmark is bench.py).

    python -m nd_gb300.benchmarks rhs       [--nv 10000000 --dtype f64 --calls 8]
    python -m nd_gb300.benchmarks warmstart [--train 20000 --test 2000 --nv 2000]
    python -m nd_gb300.benchmarks ensemble  [--instances 4096]
    python -m nd_gb300.benchmarks swing     [--nv 100000]
    python -m nd_gb300.benchmarks jacobian  [--nv 1000000]
    python -m nd_gb300.benchmarks fixpoint  [--nv 1000000]

Each prints one JSON object.  All inputs are seeded synthetic instances of the stated
shapes; no dataset is read.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np


def _sync():
    import torch
    torch.cuda.synchronize()


_T0 = time.perf_counter()


def _log(msg):
    print(f"[{time.perf_counter() - _T0:8.1f} s] {msg}", file=sys.stderr, flush=True)


def rhs(nv=10_000_000, m=4, dtype="f64", calls=8, seed=1):
    """A few calls of the diffusion RHS on Barabasi-Albert(nv, m) with the headline
    benchmark's seeded inputs (u ~ N(0, 1), w ~ U(0, 1)): the short program that per-kernel
    profiler captures run.  Reports the mean wall time of the calls and a checksum of du."""
    import torch
    import nd_gb300 as nd
    td = {"f64": torch.float64, "f32": torch.float32}[dtype]
    g = nd.barabasi_albert(nv, m, seed=seed)
    rng = np.random.default_rng(seed)
    u_h, w_h = rng.normal(size=g.nv), rng.uniform(0.0, 1.0, size=g.ne)
    nw = nd.adapt(nd.Network(g, nd.diffusion_vertex(), nd.diffusion_edge()), td)
    u = torch.from_numpy(u_h).to("cuda", td)
    p = torch.from_numpy(w_h).to("cuda", td)
    du = torch.empty_like(u)
    nw(du, u, p, 0.0)
    _sync()
    t0 = time.perf_counter()
    for _ in range(calls):
        nw(du, u, p, 0.0)
    _sync()
    return {"workload": f"diffusion on Barabasi-Albert N={g.nv}, m={m}, {dtype.upper()} RHS", "ne": g.ne,
            "calls": calls, "ms_per_call_wall": 1e3 * (time.perf_counter() - t0) / calls,
            "checksum": float(du.double().sum().item())}


def dense(nv=3000, dtype="f64", calls=8):
    """A few calls of the reference's dense diffusion benchmark network, diffusion_static_edge
    (benchmark/benchmark_cases.jl): WS(nv, nv/2, 0) with unit diffusion edges, N(0, 1) states
    -- rows of nv/2 terms, summed by the dense-network row kernels.  The short program that
    per-kernel profiler captures run; reports the mean wall time of the calls."""
    import torch
    import nd_gb300 as nd
    td = {"f64": torch.float64, "f32": torch.float32}[dtype]
    g = nd.watts_strogatz(nv, nv // 2, 0.0, seed=1)
    nw = nd.adapt(nd.Network(g, nd.diffusion_vertex(), nd.diffusion_edge_unit()), td)
    u = torch.from_numpy(np.random.default_rng(2).normal(size=nw.dim)).to("cuda", td)
    du = torch.empty_like(u)
    nw(du, u, None, 0.0)
    _sync()
    t0 = time.perf_counter()
    for _ in range(calls):
        nw(du, u, None, 0.0)
    _sync()
    return {"workload": f"diffusion_static_edge, WS({nv}, {nv // 2}, 0), {dtype.upper()} RHS", "ne": g.ne,
            "calls": calls, "ms_per_call_wall": 1e3 * (time.perf_counter() - t0) / calls,
            "checksum": float(du.double().sum().item())}


def warmstart(n_train=20000, n_test=2000, nv=2000, m=2, layers=4, epochs=80, batch=64, lr=2e-3, lr_final=5e-5,
              seed=0, tol=1e-10):
    """Swing steady states on BA(nv, m): solve n_train + n_test instances from the cold
    start, train the MPNN on the first n_train, compare cold and warm starts on the rest."""
    import nd_gb300 as nd
    from nd_gb300 import warmstart as W
    g = nd.barabasi_albert(nv, m, seed=seed + 1)
    P, K = W.swing_instances(g, n_train + n_test, seed + 2)
    t0 = time.perf_counter()
    train = W.fixpoints(g, P[:n_train], K[:n_train], tol=tol)
    t_gen = time.perf_counter() - t0
    _log(f"training data: {n_train} steady states in {t_gen:.1f} s")
    ok = train.status == 0
    model = nd.MPNN(g, layers=layers, seed=seed + 3)
    _sync()
    t0 = time.perf_counter()
    hist = model.fit(P[:n_train][ok], K[:n_train][ok], train.theta[ok], epochs=epochs, batch=batch, lr=lr,
                     lr_final=lr_final, seed=seed + 4)
    _sync()
    t_train = time.perf_counter() - t0
    _log(f"trained {epochs} epochs in {t_train:.1f} s, loss {hist[0]:.3e} -> {hist[-1]:.3e}")
    res = W.warm_vs_cold(model, g, P[n_train:], K[n_train:], tol=tol)
    res.update({
        "workload": f"swing steady states on Barabasi-Albert N={nv}, m={m}; P, K resampled per instance",
        "train_instances": int(ok.sum()), "data_generation_seconds": t_gen,
        "data_generation_newton_iters_mean": float(train.iters.mean()),
        "train_seconds": t_train, "epochs": epochs, "batch": batch, "loss_first_epoch": hist[0],
        "loss_last_epoch": hist[-1], "model": f"MPNN {layers} layers x 64 hidden, FP32",
        "tolerance": tol,
    })
    return res


def ensemble(n=4096, nv_lo=50, nv_hi=5000, t_end=50.0, reltol=1e-6, abstol=1e-6, seed=0, baseline_sample=16):
    """Basin-stability ensemble: n swing instances on random geometric graphs (mean degree
    ~6), each from its steady state plus one perturbed vertex, integrated to t_end by the
    batched Tsit5 with an FP64 and an FP32 RHS; the per-instance FP64 GPU solve of
    solve_tsit5 is timed on a sample of the instances as the plain baseline.

    Sparse geometric graphs have bottleneck lines that often cannot carry the drawn
    injections, and such an instance has no steady state.  Its parameters are drawn again
    (twice), then its injections are halved until the Newton solve converges; the counts
    are reported."""
    import torch

    import nd_gb300 as nd
    from nd_gb300 import warmstart as W
    from nd_gb300.ensemble import Ensemble
    from nd_gb300.solve import solve_tsit5
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nv_lo, nv_hi + 1, n)
    graphs = [nd.random_geometric(int(k), float(np.sqrt(6.0 / (np.pi * k))), seed=seed + 10 + i)
              for i, k in enumerate(sizes)]
    _log(f"{n} graphs, {int(sizes.sum())} vertices")
    draw = np.zeros(n, dtype=np.int64)   # parameter draw of each instance
    scale = np.ones(n)                    # factor on its injections

    def params(i):
        P, K = W.swing_instances(graphs[i], 1, seed + 100000 + 7919 * int(draw[i]) + i)
        return W.swing_flat_params(graphs[i], scale[i] * P, K)

    ps = [params(i) for i in range(n)]
    e64 = Ensemble(graphs, nd.kuramoto_second(), nd.static_line(), torch.float64)
    _log("ensemble built")
    for attempt in range(12):
        p64 = torch.from_numpy(np.concatenate(ps)).cuda()
        fx = e64.fixpoint(torch.zeros(e64.dim, dtype=torch.float64, device="cuda"), p64, tol=1e-10,
                          max_newton=12, max_cg=4000)
        status_fx = fx.status.cpu().numpy()
        bad = np.nonzero(status_fx != 0)[0]
        _log(f"fixpoints: {n - bad.size} of {n} converged (round {attempt})")
        if bad.size == 0:
            break
        for i in bad:
            if draw[i] < 2:
                draw[i] += 1
            else:
                scale[i] *= 0.5
            ps[i] = params(i)
    u0 = fx.u.clone()
    # one perturbed vertex per instance: Δθ ~ U(-π, π), Δω ~ U(-10, 10)
    uh = u0.cpu().numpy()
    for i, g in enumerate(graphs):
        v = int(rng.integers(0, g.nv))
        s = int(e64.u_offset[i]) + 2 * v
        uh[s] += rng.uniform(-np.pi, np.pi)
        uh[s + 1] += rng.uniform(-10.0, 10.0)
    u0 = torch.from_numpy(uh).cuda()
    out = {"workload": f"{n} swing instances on random geometric graphs, N ~ U[{nv_lo}, {nv_hi}], mean degree ~6; "
                       f"steady state + one perturbed vertex; Tsit5 to T={t_end}, reltol {reltol}, abstol {abstol}",
           "vertices": int(sizes.sum()), "edges": int(sum(g.ne for g in graphs)),
           "fixpoints_converged": int((status_fx == 0).sum()),
           "instances_redrawn": int((draw > 0).sum()), "instances_with_scaled_injections": int((scale < 1).sum()),
           "injection_scale_min": float(scale.min())}
    finals = {}
    # f64: the FP64 RHS; f32: FP32 RHS on FP32-rounded parameters; f32x2: double-float RHS
    # on the FP32 pipe with FP64 parameters.  Two more FP64 solves measure the floor that
    # separates precision from sensitivity: parameters perturbed by one relative ulp
    # (f64_1ulp), and rounded to FP32 (f64_f32params).
    one_ulp = p64 * (1.0 + 2.0 ** -52)
    runs = (("f64", torch.float64, p64), ("f32", torch.float32, p64.float()), ("f32x2", "f32x2", p64),
            ("f64_1ulp", torch.float64, one_ulp), ("f64_f32params", torch.float64, p64.float().double()))
    for name, dt, p in runs:
        ens = e64 if dt == torch.float64 else Ensemble(graphs, nd.kuramoto_second(), nd.static_line(), dt)
        threads = ens.autotune(u0, p, 0.0, 0.5, reltol, abstol)
        _log(f"{name}: autotuned {threads} threads per instance")
        ens.solve_tsit5(u0, p, (0.0, 0.5), reltol, abstol)  # warm-up (graph capture)
        _sync()
        t0 = time.perf_counter()
        r = ens.solve_tsit5(u0, p, (0.0, t_end), reltol, abstol)
        _sync()
        el = time.perf_counter() - t0
        _log(f"{name}: solved in {el:.2f} s")
        finals[name] = r.u.cpu().numpy()
        st = r.status.cpu().numpy()
        out[name] = {"seconds": el, "solves_per_s": n / el, "threads_per_instance": threads,
                     "steps_mean": float(r.nsteps.double().mean().item()), "ok": int((st == 0).sum())}
    # synchronised / desynchronised verdict per instance: max |ω| at T below 0.1
    verdict = {}
    for name in finals:
        w = np.abs(finals[name][1::2])
        per = np.maximum.reduceat(w, (e64.u_offset[:-1] // 2).astype(np.int64))
        verdict[name] = per < 0.1
    out["sync_fraction_f64"] = float(verdict["f64"].mean())
    sync = verdict["f64"]

    def err_stats(name):
        err = np.abs(finals[name] - finals["f64"])
        per_inst = np.maximum.reduceat(err, e64.u_offset[:-1].astype(np.int64))
        q = lambda m, x: float(np.percentile(per_inst[m], x)) if m.any() else None  # noqa: E731
        return {"max": float(err.max()), "median_instance": float(np.median(per_inst)),
                "instances_within_1e-6": int((per_inst <= 1e-6).sum()),
                "synchronised_median": q(sync, 50), "synchronised_p95": q(sync, 95),
                "synchronised_max": float(per_inst[sync].max()) if sync.any() else None,
                "synchronised_within_1e-6": int((per_inst[sync] <= 1e-6).sum()),
                "desynchronised_median": q(~sync, 50),
                "sync_verdict_agreement": float((verdict[name] == verdict["f64"]).mean())}

    for name in finals:
        if name != "f64":
            out[f"{name}_final_state_err_vs_f64"] = err_stats(name)
    out["sync_verdict_agreement_f32_vs_f64"] = out["f32_final_state_err_vs_f64"]["sync_verdict_agreement"]
    # the plain per-instance FP64 GPU solve on a sample of the instances
    idx = rng.choice(n, size=min(baseline_sample, n), replace=False)
    t_plain = 0.0
    d64, d32 = [], []  # final-state differences of the batched solves from the plain one
    for i in idx:
        g = graphs[i]
        net = nd.adapt(nd.Network(g, nd.kuramoto_second(), nd.static_line()), torch.float64)
        ui = u0[e64.u_slice(i)].clone()
        pi = p64[e64.p_slice(i)].clone()
        solve_tsit5(net, ui, pi, (0.0, 0.5), reltol, abstol)  # warm-up
        _sync()
        t0 = time.perf_counter()
        uT, _ = solve_tsit5(net, ui, pi, (0.0, t_end), reltol, abstol)
        _sync()
        t_plain += time.perf_counter() - t0
        ref = uT.cpu().numpy()
        sl = e64.u_slice(i)
        d64.append(float(np.abs(finals["f64"][sl] - ref).max()))
        d32.append(float(np.abs(finals["f32x2"][sl] - ref).max()))
    plain = len(idx) / t_plain
    _log(f"plain per-instance FP64: {len(idx)} solves in {t_plain:.2f} s")
    out["plain_f64_per_instance"] = {
        "solves_per_s": plain, "sample": int(len(idx)),
        "note": "solve_tsit5 of one Network at a time, sampled instances",
        "final_state_diff_batched_f64_vs_plain": {"median": float(np.median(d64)), "max": float(np.max(d64))},
        "final_state_diff_batched_f32x2_vs_plain": {"median": float(np.median(d32)), "max": float(np.max(d32))}}
    out["f32_batched_vs_plain_f64"] = out["f32"]["solves_per_s"] / plain
    out["f32x2_batched_vs_plain_f64"] = out["f32x2"]["solves_per_s"] / plain
    out["f64_batched_vs_plain_f64"] = out["f64"]["solves_per_s"] / plain
    return out


def swing(nv=100000, m=2, t_end=20.0, steps=200, seed=0):
    """Swing network on BA(nv, m): FP64 / FP32 RHS evaluations per second and a Tsit5 solve
    to t_end (reltol 1e-6) from a random state."""
    import torch

    import nd_gb300 as nd
    from nd_gb300 import warmstart as W
    from nd_gb300.solve import solve_tsit5
    g = nd.barabasi_albert(nv, m, seed=seed + 1)
    P, K = W.swing_instances(g, 1, seed + 2)
    p = W.swing_flat_params(g, P, K)
    rng = np.random.default_rng(seed + 3)
    u = np.empty(2 * nv)
    u[0::2] = rng.uniform(-np.pi, np.pi, nv)
    u[1::2] = rng.normal(size=nv)
    net = nd.Network(g, nd.kuramoto_second(), nd.static_line())
    out = {"workload": f"swing on Barabasi-Albert N={nv}, m={m}; K ~ U(5,10), P = ±U(0.5,1.5) zero-sum, M=1, D=0.1"}
    for name, dt in (("f64", torch.float64), ("f32", torch.float32)):
        nw = nd.adapt(net, dt)
        ut = torch.from_numpy(u).to("cuda", dt)
        pt = torch.from_numpy(p).to("cuda", dt)
        du = torch.empty_like(ut)
        for _ in range(3):
            nw(du, ut, pt)
        _sync()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(steps):
            nw(du, ut, pt)
        b.record()
        b.synchronize()
        ms = a.elapsed_time(b) / steps
        out[name] = {"rhs_ms": ms, "rhs_per_s": 1e3 / ms, "edges_per_s": g.ne * 1e3 / ms}
    nw = nd.adapt(net, torch.float64)
    ut = torch.from_numpy(u).cuda()
    pt = torch.from_numpy(p).cuda()
    _sync()
    t0 = time.perf_counter()
    uT, st = solve_tsit5(nw, ut, pt, (0.0, t_end), 1e-6, 1e-8)
    _sync()
    out["tsit5_f64"] = {"seconds": time.perf_counter() - t0, "naccept": st.naccept, "nreject": st.nreject,
                        "t_end": t_end}
    return out


def jacobian(nv=1_000_000, m=2, seed=0, steps=100):
    """Swing network on BA(nv, m): build time of the Jacobian pattern (host, once per
    network), device time of the analytic values, and of one JVP for comparison."""
    import torch

    import nd_gb300 as nd
    from nd_gb300 import warmstart as W
    g = nd.barabasi_albert(nv, m, seed=seed + 1)
    P, K = W.swing_instances(g, 1, seed + 2)
    p = torch.from_numpy(W.swing_flat_params(g, P, K)).cuda()
    net = nd.Network(g, nd.kuramoto_second(), nd.static_line())
    nw = nd.adapt(net, torch.float64)
    rng = np.random.default_rng(seed + 3)
    u = torch.from_numpy(rng.normal(size=net.dim)).cuda()
    t0 = time.perf_counter()
    rowptr, colidx = nd.jacobian_pattern(nw)
    t_pattern = time.perf_counter() - t0
    values = torch.empty(len(colidx), dtype=torch.float64, device="cuda")
    lib = nw._lib
    import ctypes as C
    from nd_gb300 import _capi as capi
    stream = torch.cuda.current_stream()

    def values_call():
        capi.check(lib.nd_jacobian(nw.handle, capi.ND_F64, values.data_ptr(), u.data_ptr(), p.data_ptr(), 0.0,
                                   C.c_void_p(stream.cuda_stream)))

    jv = torch.empty_like(u)
    out = {"workload": f"swing on Barabasi-Albert N={nv}, m={m}", "dim": net.dim, "nnz": int(len(colidx)),
           "pattern_build_s": t_pattern}
    for name, fn in (("values", values_call), ("jvp", lambda: nd.jvp(nw, jv, u, p, u))):
        for _ in range(3):
            fn()
        _sync()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(steps):
            fn()
        b.record()
        b.synchronize()
        out[f"{name}_us"] = 1e3 * a.elapsed_time(b) / steps
    # bytes of one values call: memset + write of the values, the pattern and structure reads
    out["values_bytes"] = int(8 * 2 * len(colidx) + 4 * len(colidx) + 4 * (net.dim + 1) + 16 * g.ne)
    return out


def fixpoint(nv=1_000_000, m=2, seed=0):
    """First-order Kuramoto on BA(nv, m) with zero-sum frequencies ω ~ U(-0.2, 0.2) and
    K ~ U(4, 6): the general Newton-GMRES steady-state solve from θ = 0 (host wall time,
    Newton iterations, final residual)."""
    import torch

    import nd_gb300 as nd
    g = nd.barabasi_albert(nv, m, seed=seed + 1)
    rng = np.random.default_rng(seed + 2)
    om = rng.uniform(-0.2, 0.2, g.nv)
    om -= om.mean()
    K = rng.uniform(4, 6, g.ne)
    nw = nd.adapt(nd.Network(g, nd.kuramoto_first(), nd.kuramoto_edge()), torch.float64)
    p = np.concatenate([om, K])
    nd.find_fixpoint(nw, p, tol=1e-10)  # builds the Jacobian pattern
    _sync()
    t0 = time.perf_counter()
    u = nd.find_fixpoint(nw, p, tol=1e-10)
    _sync()
    el = time.perf_counter() - t0
    st = nd.find_fixpoint.last_stats
    return {"workload": f"Kuramoto (first order) on Barabasi-Albert N={nv}, m={m}, from theta = 0",
            "dim": nw.dim, "seconds": el, "newton_iters": st["newton_iters"], "resid": st["resid"],
            "theta_spread": float(u.max().item() - u.min().item())}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("which", choices=["rhs", "dense", "warmstart", "ensemble", "swing", "jacobian", "fixpoint"])
    ap.add_argument("--dtype", choices=["f64", "f32"], default="f64")
    ap.add_argument("--calls", type=int, default=8)
    ap.add_argument("--train", type=int, default=20000)
    ap.add_argument("--test", type=int, default=2000)
    ap.add_argument("--nv", type=int, default=None)
    ap.add_argument("--epochs", type=int, default=80)
    ap.add_argument("--instances", type=int, default=4096)
    ap.add_argument("--sample", type=int, default=16)
    ap.add_argument("--t-end", type=float, default=50.0)
    a = ap.parse_args()
    if a.which == "rhs":
        r = rhs(a.nv or 10_000_000, dtype=a.dtype, calls=a.calls)
    elif a.which == "dense":
        r = dense(a.nv or 3000, dtype=a.dtype, calls=a.calls)
    elif a.which == "warmstart":
        r = warmstart(a.train, a.test, a.nv or 2000, epochs=a.epochs)
    elif a.which == "ensemble":
        r = ensemble(a.instances, baseline_sample=a.sample, t_end=a.t_end)
    elif a.which == "jacobian":
        r = jacobian(a.nv or 1_000_000)
    elif a.which == "fixpoint":
        r = fixpoint(a.nv or 1_000_000)
    else:
        r = swing(a.nv or 100000)
    print(json.dumps(r), flush=True)


if __name__ == "__main__":
    main()
