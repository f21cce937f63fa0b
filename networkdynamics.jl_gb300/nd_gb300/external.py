"""External inputs and loopback edges on the GPU: the two device copies of the reference's
core loop, for a host that runs its own components between them.

* ``StateBufIdx`` / ``OutBufIdx`` / ``ExtMap`` / ``collect_externals`` mirror the ExtMap
  gather of src/external_inputs.jl:1-80: entry k of the external-input buffer is a state
  u[i] or an output o[i].
* ``gen_loopback_map`` / ``apply_loopback`` mirror src/post_utils.jl:213-248: for every
  loopback edge the destination vertex's outputs are copied into the source vertex's
  aggregated inputs.

Indices are 0-based (the reference's are 1-based Julia indices).  The copies run in
libnd_b200.so (nd_collect_externals, nd_apply_loopback); value buffers are CUDA tensors of
one dtype (float32 or float64).  ``Network`` itself rejects components with external
inputs or loopback edges: no library component reads the one or feeds the other.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Sequence, Union

import numpy as np

from . import _capi as capi
from ._capi import ArgumentError


@dataclass(frozen=True)
class StateBufIdx:
    """External input read from the state vector u (src/external_inputs.jl:1-3)."""
    idx: int


@dataclass(frozen=True)
class OutBufIdx:
    """External input read from the output buffer o (src/external_inputs.jl:4-6)."""
    idx: int


def _code(dtype) -> int:
    import torch
    if dtype == torch.float64:
        return capi.ND_F64
    if dtype == torch.float32:
        return capi.ND_F32
    raise ArgumentError(capi.ND_ERR_DTYPE, f"external inputs: dtype {dtype} is not float32 or float64")


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class ExtMap:
    """The external-input map (src/external_inputs.jl:7-35) held on the device: one entry
    per slot of the external-input buffer, each a ``StateBufIdx`` or an ``OutBufIdx``."""

    def __init__(self, entries: Sequence[Union[StateBufIdx, OutBufIdx]], device="cuda"):
        import torch
        if len(entries) == 0:
            raise ArgumentError(capi.ND_ERR_ARG, "There are no external inputs.")
        bad = next((e for e in entries if not isinstance(e, (StateBufIdx, OutBufIdx))), None)
        if bad is not None:
            raise ArgumentError(capi.ND_ERR_ARG, f"ExtMap entry {bad!r} is neither StateBufIdx nor OutBufIdx")
        idx = np.fromiter((e.idx for e in entries), dtype=np.int64, count=len(entries))
        if (idx < 0).any():
            raise ArgumentError(capi.ND_ERR_ARG, "ExtMap: negative index")
        self.entries = list(entries)
        self.max_state = max((e.idx for e in entries if isinstance(e, StateBufIdx)), default=-1)
        self.max_out = max((e.idx for e in entries if isinstance(e, OutBufIdx)), default=-1)
        self.idx = torch.from_numpy(idx).to(device)
        self.from_state = torch.tensor([isinstance(e, StateBufIdx) for e in entries], dtype=torch.uint8,
                                       device=device)

    def __len__(self):
        return len(self.entries)


def collect_externals(extmap: ExtMap, extbuf, u, o, stream=None):
    """extbuf[k] = u[i] or o[i] for every entry k of the map (collect_externals!,
    src/external_inputs.jl:51-80).  Sizes are checked on the host before the launch."""
    code = _code(extbuf.dtype)
    for name, t in (("u", u), ("o", o)):
        if t.dtype != extbuf.dtype:
            raise ArgumentError(capi.ND_ERR_DTYPE, f"collect_externals: {name} is {t.dtype}, extbuf {extbuf.dtype}")
    if extbuf.numel() != len(extmap):
        raise ArgumentError(capi.ND_ERR_ARG, f"collect_externals: extbuf has {extbuf.numel()} entries, "
                                             f"the map {len(extmap)}")
    if extmap.max_state >= u.numel() or extmap.max_out >= o.numel():
        raise ArgumentError(capi.ND_ERR_ARG, "collect_externals: map index outside u or o")
    for t in (extbuf, u, o):
        if not t.is_cuda or not t.is_contiguous():
            raise ArgumentError(capi.ND_ERR_ARG, "collect_externals: buffers must be contiguous CUDA tensors")
    lib = capi.load()
    capi.check(lib.nd_collect_externals(code, len(extmap), extmap.idx.data_ptr(), extmap.from_state.data_ptr(),
                                        extbuf.data_ptr(), u.data_ptr(), o.data_ptr(), _stream(stream)))
    return extbuf


@dataclass
class LoopbackMap:
    """(outindex, aggindex) of gen_loopback_map, as device int64 tensors."""
    out_idx: object
    agg_idx: object

    def __len__(self):
        return int(self.out_idx.numel())


def gen_loopback_map(src, dst, loopback, v_out, v_aggr, device="cuda") -> LoopbackMap:
    """For every loopback edge in edge order, the destination vertex's output indices and
    the source vertex's aggregation indices (gen_loopback_map, src/post_utils.jl:213-224).
    v_out[v] and v_aggr[v] are the index ranges of vertex v in the output and aggregation
    buffers; a loopback edge needs them of equal length."""
    import torch
    out_idx, agg_idx = [], []
    for e in range(len(src)):
        if not loopback[e]:
            continue
        o, a = list(v_out[int(dst[e])]), list(v_aggr[int(src[e])])
        if len(o) != len(a):
            raise ArgumentError(capi.ND_ERR_ARG, f"loopback edge {e}: destination has {len(o)} outputs, "
                                                 f"source aggregates {len(a)} inputs")
        out_idx.extend(o)
        agg_idx.extend(a)
    return LoopbackMap(torch.tensor(out_idx, dtype=torch.int64, device=device),
                       torch.tensor(agg_idx, dtype=torch.int64, device=device))


def apply_loopback(aggbuf, obuf, lbmap: LoopbackMap, stream=None):
    """aggbuf[agg] = obuf[out] for every entry of the map (apply_loopback!,
    src/post_utils.jl:230-248)."""
    code = _code(aggbuf.dtype)
    if obuf.dtype != aggbuf.dtype:
        raise ArgumentError(capi.ND_ERR_DTYPE, f"apply_loopback: obuf is {obuf.dtype}, aggbuf {aggbuf.dtype}")
    n = len(lbmap)
    if n and (int(lbmap.out_idx.max()) >= obuf.numel() or int(lbmap.agg_idx.max()) >= aggbuf.numel()
              or int(lbmap.out_idx.min()) < 0 or int(lbmap.agg_idx.min()) < 0):
        raise ArgumentError(capi.ND_ERR_ARG, "apply_loopback: map index outside obuf or aggbuf")
    for t in (aggbuf, obuf):
        if not t.is_cuda or not t.is_contiguous():
            raise ArgumentError(capi.ND_ERR_ARG, "apply_loopback: buffers must be contiguous CUDA tensors")
    lib = capi.load()
    capi.check(lib.nd_apply_loopback(code, n, lbmap.out_idx.data_ptr(), lbmap.agg_idx.data_ptr(),
                                     aggbuf.data_ptr(), obuf.data_ptr(), _stream(stream)))
    return aggbuf
