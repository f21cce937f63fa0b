"""The allocation-free RHS entry point (nd_rhs_static_scratch) against the regular one.

nd_rhs_static_scratch serves callers that cannot allocate device memory while they run
the RHS (a process whose device memory belongs to a caching allocator such as CUDA.jl's
or PyTorch's pool, or one that budgets its device memory up front).  It takes the
topology as device arrays and keeps its edge values in a fixed file-scope device array.
Here it must reproduce nd_rhs on the same network, on two calls in a row (the second call
reuses the scratch the first one left), and leave the device's free memory unchanged.
This file runs last so a failure here never hides the other tests.
"""
import ctypes as C

import numpy as np
import pytest

import nd_gb300 as nd
from nd_gb300 import _capi as capi
from oracle import oracle as O

from ndtest import random_inputs

MAX_F64_EDGES = (64 << 20) // 8


def csr_arrays(g):
    """src_ptr, dst_ptr, dst_eid of a canonical edge list (numpy, host)."""
    src_ptr = np.zeros(g.nv + 1, dtype=np.uint32)
    np.add.at(src_ptr, g.src + 1, 1)
    src_ptr = np.cumsum(src_ptr).astype(np.uint32)
    order = np.argsort(g.dst, kind="stable")  # edge ids grouped by destination, ascending within
    dst_ptr = np.zeros(g.nv + 1, dtype=np.uint32)
    np.add.at(dst_ptr, g.dst + 1, 1)
    dst_ptr = np.cumsum(dst_ptr).astype(np.uint32)
    return src_ptr, dst_ptr, order.astype(np.int32)


def static_rhs(lib, vk, ek, g, dev_arrays, du, u, p, dtype_code):
    src, dst, sp, dp, de = dev_arrays
    return lib.nd_rhs_static_scratch(dtype_code, vk, ek, g.nv, g.ne, src.data_ptr(), dst.data_ptr(), sp.data_ptr(),
                                     dp.data_ptr(), de.data_ptr(), du.data_ptr(), u.data_ptr(),
                                     p.data_ptr() if p is not None else None, None)


@pytest.mark.gpu
@pytest.mark.parametrize("vk,ek,make_vm,make_em", [
    (O.V_DIFFUSION, O.E_DIFFUSION, nd.diffusion_vertex, nd.diffusion_edge),
    (O.V_KURAMOTO, O.E_KURAMOTO, nd.kuramoto_first, nd.kuramoto_edge),
    (O.V_SWING, O.E_KURAMOTO, nd.kuramoto_second, nd.static_line),
])
def test_static_scratch_rhs_matches_nd_rhs(cuda, vk, ek, make_vm, make_em):
    import torch
    lib = capi.load()
    g = nd.barabasi_albert(200_000, 4, seed=41)
    src_ptr, dst_ptr, dst_eid = csr_arrays(g)
    dev_arrays = [torch.from_numpy(np.ascontiguousarray(x)).to(cuda) for x in
                  (g.src.astype(np.int32), g.dst.astype(np.int32), src_ptr.view(np.int32), dst_ptr.view(np.int32),
                   dst_eid)]
    nw = nd.adapt(nd.Network(g, make_vm(), make_em()), torch.float64)
    on = O.OracleNetwork.from_graph(g, vk, ek)
    rng = np.random.default_rng(12)
    for call in range(2):  # two calls in a row: the second reuses the scratch left by the first
        u_h, p_h = random_inputs(on, vk, rng)
        u = torch.from_numpy(u_h).to(cuda)
        p = torch.from_numpy(p_h).to(cuda)
        ref = torch.empty_like(u)
        nw(ref, u, p, 0.0)
        got = torch.full_like(u, float("nan"))
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        capi.check(static_rhs(lib, vk, ek, g, dev_arrays, got, u, p, capi.ND_F64))
        torch.cuda.synchronize()
        if call == 1:  # after the first call (module and scratch loaded) nothing is allocated
            assert torch.cuda.mem_get_info()[0] == free_before
        # same operations in the same order as nd_rhs: identical bits
        np.testing.assert_array_equal(got.cpu().numpy(), ref.cpu().numpy())
        if call == 0:  # and against the oracle directly (the sine models: CUDA's sin vs libm's)
            want = on.rhs(u_h, p_h)
            if ek == O.E_DIFFUSION:
                np.testing.assert_array_equal(got.cpu().numpy(), want)
            else:
                dd = np.abs(got.cpu().numpy() - want)
                assert np.all((dd <= 1e-13 * np.abs(want)) | (dd <= 1e-13 * on.abs_terms(u_h, p_h)))
    # FP32: the bits of nd_rhs on every row of fewer than 128 terms (both add them in order,
    # compensating rows longer than 32); within the FP32 tolerance of the parity tests on the
    # longer rows, which nd_rhs sums a warp per row
    nw32 = nd.adapt(nd.Network(g, make_vm(), make_em()), torch.float32)
    u32 = u.float()
    p32 = p.float()
    ref32 = torch.empty_like(u32)
    nw32(ref32, u32, p32, 0.0)
    got32 = torch.empty_like(u32)
    capi.check(static_rhs(lib, vk, ek, g, dev_arrays, got32, u32, p32, capi.ND_F32))
    r32, g32 = ref32.cpu().numpy(), got32.cpu().numpy()
    short = np.repeat(g.degree() < 128, nw.dim // g.nv)
    assert short.sum() > 0.99 * len(short) and (~short).any()
    np.testing.assert_array_equal(g32[short], r32[short])
    terms = on.abs_terms(u32.double().cpu().numpy(), p32.double().cpu().numpy())
    d = np.abs(g32.astype(np.float64) - r32.astype(np.float64))
    assert np.all(d <= 4e-6 * (terms + np.abs(r32.astype(np.float64))))


@pytest.mark.gpu
def test_static_scratch_rejects_oversized_networks(cuda):
    lib = capi.load()
    code = lib.nd_rhs_static_scratch(capi.ND_F64, capi.ND_V_DIFFUSION, capi.ND_E_DIFFUSION, 10, MAX_F64_EDGES + 1,
                                     None, None, None, None, None, None, None, None, None)
    assert code == capi.ND_ERR_ARG
    assert "exceed the static scratch" in capi.last_error()


@pytest.mark.gpu
def test_static_scratch_with_a_non_canonical_order(cuda):
    """With device checks off (the default), arrays that are not the canonical sort are not
    detected (they live on the device); the result is still the network's RHS, summed in
    the arrays' order: equal to nd_rhs within the rounding of a reordered FP64 sum, not bit
    for bit."""
    import torch
    lib = capi.load()
    g = nd.barabasi_albert(50_000, 4, seed=43)
    src_ptr, dst_ptr, dst_eid = csr_arrays(g)
    rng = np.random.default_rng(2)
    for v in range(g.nv):  # reverse each vertex's destination-side order
        a, b = int(dst_ptr[v]), int(dst_ptr[v + 1])
        dst_eid[a:b] = dst_eid[a:b][::-1]
    dev_arrays = [torch.from_numpy(np.ascontiguousarray(x)).to(cuda) for x in
                  (g.src.astype(np.int32), g.dst.astype(np.int32), src_ptr.view(np.int32), dst_ptr.view(np.int32),
                   dst_eid)]
    on = O.OracleNetwork.from_graph(g, O.V_DIFFUSION, O.E_DIFFUSION)
    u_h, p_h = random_inputs(on, O.V_DIFFUSION, rng)
    u = torch.from_numpy(u_h).to(cuda)
    p = torch.from_numpy(p_h).to(cuda)
    ref = torch.empty_like(u)
    nd.adapt(nd.Network(g, nd.diffusion_vertex(), nd.diffusion_edge()), torch.float64)(ref, u, p, 0.0)
    got = torch.empty_like(u)
    capi.check(static_rhs(lib, O.V_DIFFUSION, O.E_DIFFUSION, g, dev_arrays, got, u, p, capi.ND_F64))
    d = np.abs(got.cpu().numpy() - ref.cpu().numpy())
    assert np.all(d <= 1e-13 * on.abs_terms(u_h, p_h))


@pytest.mark.gpu
def test_device_checks_report_non_canonical_arrays(cuda):
    """nd_set_device_checks(1): a canonical list gives the bits of the unchecked call; the
    reversed destination lists above, and an edge whose endpoints are swapped (src > dst),
    come back as ND_ERR_DEVICE_CHECK naming the finding and its position, and the next
    call on the same context succeeds.  Every input here is in range: the checks' range
    tests (an out-of-range index is skipped and reported) are not exercised on the GPU."""
    import torch
    lib = capi.load()
    assert lib.nd_set_device_checks(2) == capi.ND_ERR_ARG
    g = nd.barabasi_albert(20_000, 3, seed=44)
    on = O.OracleNetwork.from_graph(g, O.V_DIFFUSION, O.E_DIFFUSION)
    u_h, p_h = random_inputs(on, O.V_DIFFUSION, np.random.default_rng(3))
    u = torch.from_numpy(u_h).to(cuda)
    p = torch.from_numpy(p_h).to(cuda)

    def arrays(src, dst, dst_eid=None):
        gg = nd.Graph(g.nv, src, dst) if dst_eid is None else g
        sp, dp, de = csr_arrays(gg)
        if dst_eid is not None:
            de = dst_eid
        return [torch.from_numpy(np.ascontiguousarray(x)).to(cuda) for x in
                (src.astype(np.int32), dst.astype(np.int32), sp.view(np.int32), dp.view(np.int32), de)]

    def run(dev_arrays):
        out = torch.empty_like(u)
        return static_rhs(lib, O.V_DIFFUSION, O.E_DIFFUSION, g, dev_arrays, out, u, p, capi.ND_F64), out

    canonical = arrays(g.src, g.dst)
    code, plain = run(canonical)
    assert code == capi.ND_OK
    _, dp, de = csr_arrays(g)
    for v in range(g.nv):
        a, b = int(dp[v]), int(dp[v + 1])
        de[a:b] = de[a:b][::-1]
    src_sw, dst_sw = g.src.copy(), g.dst.copy()
    k = int(np.nonzero(np.diff(g.src) > 0)[0][100]) + 1  # first edge of a source block
    src_sw[k], dst_sw[k] = g.dst[k], g.src[k]
    lib.nd_set_device_checks(1)
    try:
        code, got = run(canonical)
        assert code == capi.ND_OK
        np.testing.assert_array_equal(got.cpu().numpy(), plain.cpu().numpy())
        code, _ = run(arrays(g.src, g.dst, de))
        assert code == capi.ND_ERR_DEVICE_CHECK
        assert "dst_eid not ascending" in capi.last_error()
        code, _ = run(arrays(src_sw, dst_sw))
        assert code == capi.ND_ERR_DEVICE_CHECK
        msg = capi.last_error()
        assert "device check" in msg and ("not canonical" in msg or "source block" in msg), msg
        code, got = run(canonical)
        assert code == capi.ND_OK
        np.testing.assert_array_equal(got.cpu().numpy(), plain.cpu().numpy())
    finally:
        lib.nd_set_device_checks(0)
    with pytest.raises(nd.ArgumentError):
        capi.check(capi.ND_ERR_DEVICE_CHECK)
