"""The integer-exact binary64 adder (networkdynamics.jl_gb300/csrc/nd_exact.cuh) against
the CPU's IEEE-754 addition, bit for bit.  The CPU test compiles the header for the host;
the GPU tests run the device build and the warp exact scan through the diagnostic C ABI."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "networkdynamics.jl_gb300" / "csrc"
NATIVE = Path(__file__).resolve().parent / "native"


@pytest.fixture(scope="module")
def host_lib():
    out = NATIVE / "_build" / "libexact_host.so"
    out.parent.mkdir(exist_ok=True)
    src = NATIVE / "exact_add_host.cpp"
    hdr = CSRC / "nd_exact.cuh"
    if not out.exists() or out.stat().st_mtime < max(src.stat().st_mtime, hdr.stat().st_mtime):
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", f"-I{CSRC}", str(src),
                        "-o", str(out)], check=True)
    lib = C.CDLL(str(out))
    lib.nd_exact_add_host.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
    return lib


def adversarial_pairs(n, seed=0):
    rng = np.random.default_rng(seed)
    cases = [(rng.normal(size=n), rng.normal(size=n)),
             (rng.normal(size=n), -rng.normal(size=n) * rng.choice([1, 1e-3, 1e-10, 1e3], size=n))]
    x = rng.normal(size=n)
    cases.append((x, -x * (1 + rng.integers(-3, 3, size=n) * 2.0 ** -52)))          # cancellation
    hi = np.uint64(63)
    b1 = rng.integers(0, 2 ** 63, size=n, dtype=np.uint64) | (rng.integers(0, 2, size=n, dtype=np.uint64) << hi)
    b2 = rng.integers(0, 2 ** 63, size=n, dtype=np.uint64) | (rng.integers(0, 2, size=n, dtype=np.uint64) << hi)
    cases.append((b1.view(np.float64), b2.view(np.float64)))                          # any bit pattern
    sub = rng.integers(0, 2 ** 53, size=n, dtype=np.uint64).view(np.float64)         # subnormal / tiny
    neg = (rng.integers(0, 2 ** 53, size=n, dtype=np.uint64) | (np.uint64(1) << hi)).view(np.float64)
    cases.append((sub, neg))
    a = rng.normal(size=n)
    cases.append((a, np.spacing(a) / 2 * rng.choice([1, -1, 3, -3, 5], size=n)))     # ties
    z = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 1.7976931348623157e308,
                  -1.7976931348623157e308, 2.2250738585072014e-308])
    A, B = np.meshgrid(z, z)
    cases.append((A.ravel(), B.ravel()))
    return cases


def assert_bitwise(ref, got):
    same = (ref.view(np.uint64) == got.view(np.uint64)) | (np.isnan(ref) & np.isnan(got))
    if not same.all():
        i = np.nonzero(~same)[0][:5]
        raise AssertionError(f"{(~same).sum()} mismatches, e.g. {[(ref[j], got[j]) for j in i]}")


def test_host_exact_add_matches_ieee(host_lib):
    for a, b in adversarial_pairs(400_000):
        a = np.ascontiguousarray(a)
        b = np.ascontiguousarray(b)
        out = np.empty_like(a)
        host_lib.nd_exact_add_host(a.ctypes.data, b.ctypes.data, out.ctypes.data, a.size)
        with np.errstate(all="ignore"):
            assert_bitwise(a + b, out)


@pytest.mark.gpu
def test_device_exact_add_matches_ieee(cuda):
    import torch

    from nd_gb300 import _capi as capi
    lib = capi.load()
    for a, b in adversarial_pairs(1_000_000, seed=1):
        ta = torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
        tb = torch.from_numpy(np.ascontiguousarray(b)).to(cuda)
        out = torch.empty_like(ta)
        capi.check(lib.nd_selftest_exact_add(ta.data_ptr(), tb.data_ptr(), out.data_ptr(), ta.numel(), None))
        with np.errstate(all="ignore"):
            assert_bitwise(a + b, out.cpu().numpy())


def sequential(s0, terms):
    s = s0
    for t in terms:
        s = s + t
    return s


@pytest.mark.gpu
def test_device_exact_scan_equals_sequential_sum(cuda):
    import torch

    from nd_gb300 import _capi as capi
    lib = capi.load()
    rng = np.random.default_rng(7)
    segs, s0 = [], []
    # diffusion-like hub rows: terms w (u_n - u_v) with a drifting partial sum
    for _ in range(40):
        d = int(rng.integers(1, 7000))
        uv = rng.normal()
        segs.append(rng.uniform(0, 1, d) * (rng.normal(size=d) - uv))
        s0.append(0.0)
    # adversarial: mixed magnitudes, exact cancellations, ties to the running sum's ulp
    for _ in range(40):
        d = int(rng.integers(1, 700))
        t = rng.normal(size=d) * 10.0 ** rng.integers(-12, 12, size=d)
        t[rng.random(d) < 0.1] = 0.0
        segs.append(t)
        s0.append(float(rng.choice([0.0, -0.0, 1.0, -3.5, 1e-300, 1e300])))
    for _ in range(20):
        d = int(rng.integers(32, 300))
        base = float(2.0 ** rng.integers(-5, 5))
        t = np.spacing(base) * rng.integers(-8, 8, size=d) / 2    # many exact half-ulp ties
        t[0] = base
        segs.append(t)
        s0.append(0.0)
    segs.append(np.array([1.0, -1.0, 2.0 ** -60, 5e-324, -5e-324]))
    s0.append(0.0)
    seg = np.zeros(len(segs) + 1, dtype=np.int64)
    seg[1:] = np.cumsum([len(s) for s in segs])
    terms = np.concatenate(segs)
    dt = torch.from_numpy(terms).to(cuda)
    dseg = torch.from_numpy(seg).to(cuda)
    ds0 = torch.tensor(s0, dtype=torch.float64, device=cuda)
    out = torch.empty(len(segs), dtype=torch.float64, device=cuda)
    capi.check(lib.nd_selftest_exact_scan(dt.data_ptr(), dseg.data_ptr(), ds0.data_ptr(), out.data_ptr(), len(segs),
                                          None))
    got = out.cpu().numpy()
    ref = np.array([sequential(s, t) for s, t in zip(s0, segs)])
    assert_bitwise(ref, got)
