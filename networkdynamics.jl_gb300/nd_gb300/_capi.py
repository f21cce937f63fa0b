"""ctypes binding of libnd_b200.so (declarations in include/nd_gb300.h).

The library is loaded from the package's ``lib/`` folder.  When it is missing the import
of any GPU entry point raises: there is no CPU fallback for the GB300 path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from ._build import CUDA_LIB, GRAPHGEN_LIB

ND_OK = 0
ND_ERR_ARG = -1
ND_ERR_UNSUPPORTED_COMPONENT = -2
ND_ERR_DTYPE = -3
ND_ERR_CUDA = -4
ND_ERR_MAXITERS = -5
ND_ERR_UNSUPPORTED = -6
ND_ERR_NOMEM = -7
ND_ERR_NOT_CONVERGED = -8
ND_ERR_DEVICE_CHECK = -9

ND_F32 = 1
ND_F64 = 2
ND_F32X2 = 3  # ensembles: FP64 buffers, double-float RHS arithmetic on the FP32 pipe

ND_V_DIFFUSION = 1
ND_V_KURAMOTO = 2
ND_V_SWING = 3
ND_V_SWING_UNIT = 4
ND_V_PQ = 5
ND_V_GENERATOR = 6
ND_V_PQ_CONST = 7

ND_E_DIFFUSION = 1
ND_E_DIFFUSION_UNIT = 2
ND_E_KURAMOTO = 3
ND_E_DIFFUSION_ODE = 4
ND_E_DIFFUSION_ODE_FIXED = 5
ND_E_PILINE = 6

ND_ANTISYMMETRIC = 1
ND_SYMMETRIC = 2
ND_DIRECTED = 3
ND_FIDUCIAL = 4
COUPLINGS = {"AntiSymmetric": ND_ANTISYMMETRIC, "Symmetric": ND_SYMMETRIC, "Directed": ND_DIRECTED,
             "Fiducial": ND_FIDUCIAL}

ND_MAX_BATCHES = 1 << 20
ND_ENSEMBLE_DEFAULT_MAX_STEPS = 100000  # per-instance step budget of nd_ensemble_solve_tsit5 for max_steps <= 0
ND_BATCH_CONSTANTS = 2

ND_ORDER_SEQUENTIAL = 0
ND_ORDER_TREE = 1
ND_ORDER_SEQUENTIAL_HW = 2

KERNEL_KINDS = ("edge_phase", "row_phase", "heavy_rows", "fused", "batched_edges", "batched_rows")


class NDError(RuntimeError):
    """A failing libnd_b200 call; ``code`` is the nd_status value."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class ArgumentError(NDError, ValueError):
    """Counterpart of Julia's ArgumentError raised by the reference for the same inputs."""


class UnsupportedComponentError(ArgumentError):
    pass


class NotConvergedError(NDError):
    """Counterpart of the reference's NetworkInitError."""


class nd_network_desc(C.Structure):
    _fields_ = [("nv", C.c_int64), ("ne", C.c_int64),
                ("src", C.POINTER(C.c_int64)), ("dst", C.POINTER(C.c_int64)),
                ("vertex_kind", C.c_int32), ("edge_kind", C.c_int32),
                ("coupling", C.c_int32), ("flags", C.c_int32)]


class nd_info(C.Structure):
    _fields_ = [("dim", C.c_int64), ("pdim", C.c_int64), ("nv", C.c_int64), ("ne", C.c_int64),
                ("n_incidences", C.c_int64), ("dtype", C.c_int32), ("vertex_kind", C.c_int32),
                ("edge_kind", C.c_int32), ("max_degree", C.c_int32), ("n_hubs", C.c_int32),
                ("sum_order", C.c_int32), ("n_vertex_batches", C.c_int32), ("n_edge_batches", C.c_int32)]


class nd_batch(C.Structure):
    _fields_ = [("kind", C.c_int32), ("coupling", C.c_int32)]


class nd_batched_network_desc(C.Structure):
    _fields_ = [("nv", C.c_int64), ("ne", C.c_int64),
                ("src", C.POINTER(C.c_int64)), ("dst", C.POINTER(C.c_int64)),
                ("n_vertex_batches", C.c_int32), ("n_edge_batches", C.c_int32),
                ("vertex_batches", C.POINTER(nd_batch)), ("edge_batches", C.POINTER(nd_batch)),
                ("vertex_batch", C.POINTER(C.c_int32)), ("edge_batch", C.POINTER(C.c_int32)),
                ("flags", C.c_int32), ("reserved", C.c_int32), ("vertex_constants", C.POINTER(C.c_double))]


# Every symbol include/nd_gb300.h declares, with (restype, argtypes).
SIGNATURES = {
    "nd_version": (C.c_int, []),
    "nd_last_error": (C.c_char_p, []),
    "nd_create": (C.c_int, [C.POINTER(nd_network_desc), C.c_int, C.POINTER(C.c_void_p)]),
    "nd_create_batched": (C.c_int, [C.POINTER(nd_batched_network_desc), C.c_int, C.POINTER(C.c_void_p)]),
    "nd_destroy": (C.c_int, [C.c_void_p]),
    "nd_get_info": (C.c_int, [C.c_void_p, C.POINTER(nd_info)]),
    "nd_set_sum_order": (C.c_int, [C.c_void_p, C.c_int]),
    "nd_set_layout": (C.c_int, [C.c_void_p, C.c_int]),
    "nd_set_kernel_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "nd_kernel_times": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_double), C.c_int]),
    "nd_rhs": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                         C.c_void_p, C.c_int64, C.c_double, C.c_void_p]),
    "nd_rhs_static_scratch": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p]),
    # include/nd_gb300_selftest.h
    "nd_selftest_exact_add": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "nd_selftest_exact_scan": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
}

_lib = None
_graphgen = None


def library_path() -> Path:
    return CUDA_LIB


def load(path: Path | None = None):
    """Load libnd_b200.so (once) and attach the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else CUDA_LIB
    if not p.exists():
        raise ImportError(f"{p} is missing: build it first (__graft_entry__.build()); "
                          "the GB300 path has no CPU fallback")
    lib = C.CDLL(str(p), mode=C.RTLD_GLOBAL)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    msg = load().nd_last_error()
    return msg.decode() if msg else ""


def check(code: int) -> int:
    if code == ND_OK:
        return code
    msg = last_error()
    if code == ND_ERR_UNSUPPORTED_COMPONENT:
        raise UnsupportedComponentError(code, msg)
    if code in (ND_ERR_ARG, ND_ERR_DTYPE, ND_ERR_UNSUPPORTED, ND_ERR_DEVICE_CHECK):
        raise ArgumentError(code, msg)
    if code in (ND_ERR_NOT_CONVERGED, ND_ERR_MAXITERS):
        raise NotConvergedError(code, msg)
    raise NDError(code, msg)


def load_graphgen():
    global _graphgen
    if _graphgen is not None:
        return _graphgen
    if not GRAPHGEN_LIB.exists():
        raise ImportError(f"{GRAPHGEN_LIB} is missing: build it first (__graft_entry__.build())")
    lib = C.CDLL(str(GRAPHGEN_LIB))
    P = C.POINTER(C.c_int64)
    lib.nd_gen_watts_strogatz.restype = C.c_int64
    lib.nd_gen_watts_strogatz.argtypes = [C.c_int64, C.c_int64, C.c_double, C.c_uint64, P, P, C.c_int64]
    lib.nd_gen_barabasi_albert.restype = C.c_int64
    lib.nd_gen_barabasi_albert.argtypes = [C.c_int64, C.c_int64, C.c_uint64, P, P, C.c_int64]
    lib.nd_gen_random_geometric.restype = C.c_int64
    lib.nd_gen_random_geometric.argtypes = [C.c_int64, C.c_double, C.c_uint64, P, P, C.c_int64,
                                            C.POINTER(C.c_double)]
    _graphgen = lib
    return lib


class nd_solve_stats(C.Structure):
    _fields_ = [("naccept", C.c_int64), ("nreject", C.c_int64), ("nf", C.c_int64), ("t_final", C.c_double),
                ("dt_last", C.c_double), ("status", C.c_int32), ("reserved", C.c_int32)]


SIGNATURES["nd_solve_tsit5"] = (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                          C.c_double, C.c_int64, C.POINTER(nd_solve_stats), C.c_void_p])
SIGNATURES["nd_solve_rosenbrock23"] = (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                                 C.c_double, C.c_double, C.c_double, C.c_int64,
                                                 C.POINTER(nd_solve_stats), C.c_void_p])
SIGNATURES["nd_solve_rodas4"] = SIGNATURES["nd_solve_rosenbrock23"]


class nd_ensemble_desc(C.Structure):
    _fields_ = [("n_instances", C.c_int64), ("v_offset", C.POINTER(C.c_int64)), ("e_offset", C.POINTER(C.c_int64)),
                ("src", C.POINTER(C.c_int64)), ("dst", C.POINTER(C.c_int64)), ("vertex_kind", C.c_int32),
                ("edge_kind", C.c_int32), ("coupling", C.c_int32), ("flags", C.c_int32)]


_vp, _i64, _d = C.c_void_p, C.c_int64, C.c_double
SIGNATURES.update({
    "nd_jvp": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, _d, _vp]),
    "nd_jacobian_pattern": (C.c_int, [_vp, C.POINTER(C.c_int64), _vp, _vp]),
    "nd_jacobian": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _d, _vp]),
    "nd_find_fixpoint": (C.c_int, [_vp, _vp, _vp, _d, _d, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int32),
                                   C.POINTER(C.c_double), _vp]),
    "nd_ensemble_create": (C.c_int, [C.POINTER(nd_ensemble_desc), C.c_int, C.POINTER(C.c_void_p)]),
    "nd_ensemble_destroy": (C.c_int, [_vp]),
    "nd_ensemble_get_info": (C.c_int, [_vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "nd_ensemble_rhs": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp]),
    "nd_ensemble_solve_tsit5": (C.c_int, [_vp, _vp, _vp, _d, _d, _d, _d, _i64, C.c_int, _vp, _vp, _vp]),
    "nd_ensemble_solve_tsit5_ex": (C.c_int, [_vp, _vp, _vp, _d, _d, _d, _d, _i64, C.c_int, _vp, _vp, _vp, C.c_int,
                                             _vp]),
    "nd_ensemble_autotune": (C.c_int, [_vp, _vp, _vp, _d, _d, _d, _d, C.POINTER(C.c_int), _vp]),
    "nd_ensemble_set_threads": (C.c_int, [_vp, C.c_int]),
    "nd_ensemble_fixpoint": (C.c_int, [_vp, _vp, _vp, _d, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp]),
    "nd_mpnn_create": (C.c_int, [_i64, _i64, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_int, C.c_int,
                                 C.c_uint64, C.POINTER(C.c_void_p)]),
    "nd_mpnn_destroy": (C.c_int, [_vp]),
    "nd_mpnn_num_params": (C.c_int, [_vp, C.POINTER(C.c_int64)]),
    "nd_mpnn_get_params": (C.c_int, [_vp, _vp, _vp]),
    "nd_mpnn_set_params": (C.c_int, [_vp, _vp, _vp]),
    "nd_mpnn_get_grads": (C.c_int, [_vp, _vp, _vp]),
    "nd_mpnn_forward": (C.c_int, [_vp, _i64, _vp, _vp, _vp, _vp]),
    "nd_mpnn_loss_grad": (C.c_int, [_vp, _i64, _vp, _vp, _vp, _vp, _vp]),
    "nd_mpnn_adam": (C.c_int, [_vp, _d, _d, _d, _d, _vp]),
    "nd_mpnn_reset_optimizer": (C.c_int, [_vp, _vp]),
    "nd_mpnn_set_hops": (C.c_int, [_vp, C.c_int]),
    "nd_set_device_checks": (C.c_int, [C.c_int]),
    "nd_collect_externals": (C.c_int, [C.c_int, _i64, _vp, _vp, _vp, _vp, _vp, _vp]),
    "nd_apply_loopback": (C.c_int, [C.c_int, _i64, _vp, _vp, _vp, _vp, _vp]),
})
