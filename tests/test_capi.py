"""The C ABI library loads, exports every declared symbol, and rejects bad descriptors
before any device work (no GPU needed for these)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import nd_gb300 as nd
from nd_gb300 import _capi as capi

HEADER_DIR = Path(__file__).resolve().parent.parent / "include"


def declared_symbols():
    names = set()
    for h in HEADER_DIR.glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(nd_[a-z_0-9]+)\s*\(", text, flags=re.M))
    return names


def test_library_exports_every_declared_symbol():
    lib = capi.load()
    names = declared_symbols()
    assert "nd_rhs" in names and "nd_create" in names
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, f"symbols declared in include/*.h but not exported: {missing}"
    assert set(capi.SIGNATURES) >= names, "ctypes signature table misses declared symbols"


def test_version_and_error_string():
    lib = capi.load()
    assert lib.nd_version() == 10000
    assert isinstance(capi.last_error(), str)


def _desc(g, vk, ek, coupling=capi.ND_ANTISYMMETRIC, flags=0):
    src = np.ascontiguousarray(g.src)
    dst = np.ascontiguousarray(g.dst)
    P = C.POINTER(C.c_int64)
    d = capi.nd_network_desc(g.nv, g.ne, src.ctypes.data_as(P), dst.ctypes.data_as(P), vk, ek, coupling, flags)
    return d, (src, dst)


@pytest.mark.parametrize("vk,ek,code", [
    (0, capi.ND_E_DIFFUSION, capi.ND_ERR_UNSUPPORTED_COMPONENT),
    (capi.ND_V_SWING, 9, capi.ND_ERR_UNSUPPORTED_COMPONENT),
    (7, 7, capi.ND_ERR_UNSUPPORTED_COMPONENT),
])
def test_create_rejects_unknown_components(vk, ek, code):
    lib = capi.load()
    g = nd.cycle_graph(5)
    d, _keep = _desc(g, vk, ek)
    h = C.c_void_p()
    assert lib.nd_create(C.byref(d), capi.ND_F64, C.byref(h)) == code
    assert "library" in capi.last_error()
    assert not h.value


def test_create_rejects_bad_dtype_and_coupling():
    lib = capi.load()
    g = nd.cycle_graph(5)
    d, _keep = _desc(g, capi.ND_V_DIFFUSION, capi.ND_E_DIFFUSION)
    h = C.c_void_p()
    assert lib.nd_create(C.byref(d), 3, C.byref(h)) == capi.ND_ERR_DTYPE
    for ek, coupling in ((capi.ND_E_DIFFUSION, 9), (capi.ND_E_KURAMOTO, capi.ND_FIDUCIAL),
                         (capi.ND_E_DIFFUSION_ODE, capi.ND_ANTISYMMETRIC), (7, capi.ND_FIDUCIAL),
                         (capi.ND_E_PILINE, capi.ND_ANTISYMMETRIC)):
        d2, _keep2 = _desc(g, capi.ND_V_DIFFUSION, ek, coupling=coupling)
        assert lib.nd_create(C.byref(d2), capi.ND_F64, C.byref(h)) == capi.ND_ERR_UNSUPPORTED_COMPONENT
        assert not h.value
    assert lib.nd_create(None, capi.ND_F64, C.byref(h)) == capi.ND_ERR_ARG


def test_null_handle_calls_fail_cleanly():
    lib = capi.load()
    assert lib.nd_rhs(None, capi.ND_F64, None, 0, None, 0, None, 0, 0.0, None) == capi.ND_ERR_ARG
    assert lib.nd_destroy(None) == capi.ND_OK
    info = capi.nd_info()
    assert lib.nd_get_info(None, C.byref(info)) == capi.ND_ERR_ARG


def _bdesc(g, vbatches, vbatch, ebatches, ebatch, consts=None):
    P = C.POINTER(C.c_int64)
    P32 = C.POINTER(C.c_int32)
    src = np.ascontiguousarray(g.src, dtype=np.int64)
    dst = np.ascontiguousarray(g.dst, dtype=np.int64)
    vb = (capi.nd_batch * max(len(vbatches), 1))(*vbatches)
    eb = (capi.nd_batch * max(len(ebatches), 1))(*ebatches)
    vbi = np.ascontiguousarray(vbatch, dtype=np.int32)
    ebi = np.ascontiguousarray(ebatch, dtype=np.int32)
    cst = None if consts is None else np.ascontiguousarray(consts, dtype=np.float64)
    d = capi.nd_batched_network_desc(g.nv, g.ne, src.ctypes.data_as(P), dst.ctypes.data_as(P), len(vbatches),
                                     len(ebatches), vb, eb, vbi.ctypes.data_as(P32), ebi.ctypes.data_as(P32), 0, 0,
                                     cst.ctypes.data_as(C.POINTER(C.c_double)) if cst is not None else None)
    return d, (src, dst, vb, eb, vbi, ebi, cst)


def test_create_batched_rejects_bad_descriptions():
    """Every check of a batched description runs on the host, before any device resource:
    the reference's construction errors (src/construction.jl:98-106) and the library's."""
    lib = capi.load()
    g = nd.cycle_graph(4)
    ok_e = [(capi.ND_E_PILINE, capi.ND_FIDUCIAL)]
    cases = [
        # mixed output dimensions: PQ bus (complex) and diffusion vertex
        (([(capi.ND_V_PQ, 0), (capi.ND_V_DIFFUSION, 0)], [0, 1, 0, 1], ok_e, [0] * 4), capi.ND_ERR_ARG, "output"),
        (([(99, 0)], [0] * 4, [(capi.ND_E_DIFFUSION, capi.ND_ANTISYMMETRIC)], [0] * 4),
         capi.ND_ERR_UNSUPPORTED_COMPONENT, "library"),
        (([(capi.ND_V_PQ_CONST, 0)], [0] * 4, ok_e, [0] * 4), capi.ND_ERR_ARG, "vertex_constants"),
        (([(capi.ND_V_PQ, 0)], [0, 0, 3, 0], ok_e, [0] * 4), capi.ND_ERR_ARG, "batch"),
        (([(capi.ND_V_PQ, 0)], [0] * 4, [(capi.ND_E_PILINE, capi.ND_ANTISYMMETRIC)], [0] * 4),
         capi.ND_ERR_UNSUPPORTED_COMPONENT, "two-sided"),
        (([], [0] * 4, ok_e, [0] * 4), capi.ND_ERR_ARG, "n_vertex_batches"),
        (([(capi.ND_V_DIFFUSION, 0)], [0] * 4, [(capi.ND_E_DIFFUSION, capi.ND_ANTISYMMETRIC)], [0, 0, 1, 0]),
         capi.ND_ERR_ARG, "batch"),
    ]
    for args, code, word in cases:
        d, _keep = _bdesc(g, *args)
        h = C.c_void_p()
        assert lib.nd_create_batched(C.byref(d), capi.ND_F64, C.byref(h)) == code, args
        assert word in capi.last_error() and not h.value
    d, _keep = _bdesc(g, [(capi.ND_V_DIFFUSION, 0)], [0] * 4, [(capi.ND_E_DIFFUSION, capi.ND_ANTISYMMETRIC)], [0] * 4)
    assert lib.nd_create_batched(C.byref(d), 7, C.byref(C.c_void_p())) == capi.ND_ERR_DTYPE
    assert lib.nd_create_batched(None, capi.ND_F64, C.byref(C.c_void_p())) == capi.ND_ERR_ARG
