"""Analytic JVP against central finite differences of the GPU RHS (the pattern of the
reference's test/AD_test.jl:54-60) and against a numpy restatement of the derivative."""
import numpy as np
import pytest

import nd_gb300 as nd
from oracle import oracle as O

from ndtest import random_inputs

pytestmark = pytest.mark.gpu

CASES = [(O.V_DIFFUSION, O.E_DIFFUSION, nd.diffusion_vertex, nd.diffusion_edge),
         (O.V_DIFFUSION, O.E_DIFFUSION_UNIT, nd.diffusion_vertex, nd.diffusion_edge_unit),
         (O.V_KURAMOTO, O.E_KURAMOTO, nd.kuramoto_first, nd.kuramoto_edge),
         (O.V_SWING, O.E_KURAMOTO, nd.kuramoto_second, nd.static_line)]


def jvp_numpy(g, vk, ek, u, p, v):
    dv = O.VDIM[vk]
    th, vt = u[::dv], v[::dv]
    pe = p[g.nv * O.VPDIM[vk]:]
    if ek == O.E_DIFFUSION:
        c = pe
    elif ek == O.E_DIFFUSION_UNIT:
        c = np.ones(g.ne)
    else:
        c = pe * np.cos(th[g.src] - th[g.dst])
    y = c * (vt[g.src] - vt[g.dst])
    acc = np.zeros(g.nv)
    np.add.at(acc, g.dst, y)
    np.add.at(acc, g.src, -y)
    if vk == O.V_SWING:
        P = p[:3 * g.nv].reshape(-1, 3)
        out = np.empty(2 * g.nv)
        out[0::2] = v[1::2]
        out[1::2] = (acc - P[:, 1] * v[1::2]) / P[:, 0]
        return out
    return acc


@pytest.mark.parametrize("vk,ek,vm,em", CASES)
def test_jvp_matches_finite_differences(cuda, vk, ek, vm, em):
    import torch
    g = nd.barabasi_albert(5000, 3, seed=6)
    nw = nd.adapt(nd.Network(g, vm(), em()), torch.float64)
    on = O.OracleNetwork.from_graph(g, vk, ek)
    rng = np.random.default_rng(10)
    u, p = random_inputs(on, vk, rng)
    v = rng.normal(size=nw.dim)
    tu, tp, tv = (torch.from_numpy(x).to(cuda) for x in (u, p, v))
    jv = torch.empty_like(tu)
    nd.jvp(nw, jv, tu, tp, tv)
    got = jv.cpu().numpy()
    np.testing.assert_allclose(got, jvp_numpy(g, vk, ek, u, p, v), rtol=1e-12, atol=1e-12)
    eps = 1e-6
    fp, fm = torch.empty_like(tu), torch.empty_like(tu)
    nw(fp, tu + eps * tv, tp, 0.0)
    nw(fm, tu - eps * tv, tp, 0.0)
    fd = ((fp - fm) / (2 * eps)).cpu().numpy()
    np.testing.assert_allclose(got, fd, rtol=1e-6, atol=1e-6)
