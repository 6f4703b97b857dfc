"""ctypes binding of ``libgde.so`` (declared in ``include/gde.h``).

The library is built in-tree by ``gde._build``.  Loading fails loudly when
the shared object is missing: there is no CPU fallback for any solver.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import _build

_i64 = ctypes.c_int64
_i32 = ctypes.c_int32
_int = ctypes.c_int
_dbl = ctypes.c_double
_p = ctypes.c_void_p

GDE_OK, GDE_EINVAL, GDE_ENOMEM, GDE_EITERCAP, GDE_ECUDA, GDE_EHANG, GDE_ECAPACITY, GDE_ENOTFOUND = range(8)
PPR, KATZ, HK, IGN, UPPR = range(5)
LOCAL_GD, GLOBAL_GD, LOCAL_CHEBY, GLOBAL_CHEBY, HK_LOCAL, HK_GLOBAL, HK_TAYLOR = range(7)
FP64, FP32 = 0, 1
MEM_HOST, MEM_DEVICE = 0, 1


class Params(ctypes.Structure):
    _fields_ = [("kind", _int), ("method", _int), ("prec", _int), ("tile_w", _int),
                ("alpha", _dbl), ("tau", _dbl), ("l_max", _dbl), ("mu_min", _dbl), ("beta", _dbl), ("omega", _dbl),
                ("max_rounds", _int), ("small_max", _int), ("med_max", _int), ("chunk", _int), ("dense_div", _int),
                ("slots", _int), ("groups", _int),
                ("sparse_blocks", _int), ("sparse_cap", _int), ("sparse_eps", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("kernel_ms", _dbl), ("total_ms", _dbl), ("rounds", _i64), ("dense_rounds", _i64),
                ("union_vol", _dbl), ("col_vol", _dbl), ("union_nodes", ctypes.c_uint64),
                ("col_nodes", ctypes.c_uint64), ("tiles", _int), ("tile_w", _int),
                ("check_ms", _dbl), ("prep_ms", _dbl), ("scatter_ms", _dbl), ("edit_path", _int),
                ("edit_ms", _dbl), ("prec", _int),
                ("sparse_queries", _i64), ("sparse_overflows", _i64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


# Every symbol include/gde.h declares, with its ctypes signature.
SIGNATURES = {
    "gde_status_str": (ctypes.c_char_p, [_int]),
    "gde_version": (_int, []),
    "gde_probe_random_atomics": (_int, [_p, _i64, _int, ctypes.POINTER(ctypes.c_double)]),
    "gde_ctx_create": (_int, [_int, ctypes.POINTER(_p)]),
    "gde_ctx_destroy": (_int, [_p]),
    "gde_last_error": (ctypes.c_char_p, [_p]),
    "gde_ctx_sync": (_int, [_p]),
    "gde_graph_upload": (_int, [_p, _i64, _i64, _p, _p, _p, _p, ctypes.POINTER(_p)]),
    "gde_graph_free": (_int, [_p]),
    "gde_graph_info": (_int, [_p, _p, _p, _p]),
    "gde_solve": (_int, [_p, _p, ctypes.POINTER(Params), _i64, _p, _p, _p, _p, _int, _int, _i64, _p, _p, _p,
                         ctypes.POINTER(Stats)]),
    "gde_ctx_stream": (_p, [_p]),
    "gde_serve": (_int, [_p, _p, ctypes.POINTER(Params), _i64, _p, _p, _p, _p, _p, _int, _int, _i64, _p, _p, _p,
                         ctypes.POINTER(Stats)]),
    "gde_hk_estimate_n": (_i64, [_dbl, _dbl]),
    "gde_graph_repad": (_int, [_p, _p, _i64, _p, _p, _p]),
    "gde_graph_update": (_int, [_p, _p, _p, _p, _p, _p, _i64, _int, _p, ctypes.POINTER(Stats)]),
    "gde_feature_repair": (_int, [_p, _p, ctypes.POINTER(Params), _i64, _p, _p, _p, _i64, _i64, _p, _p, _p, _p]),
    "gde_feature_push": (_int, [_p, _p, ctypes.POINTER(Params), _i64, _p, _p, _i64, _dbl, _p, _i64, _p,
                                ctypes.POINTER(Stats)]),
    "gde_feature_update": (_int, [_p, _p, _p, _p, _p, _p, _i64, _int, ctypes.POINTER(Params), _i64, _p, _p, _p,
                                  _i64, _dbl, _p, ctypes.POINTER(Stats)]),
    "gde_plain_ppr_local": (_int, [_p, _p, _i32, _dbl, _dbl, _p, _p, _p, _p]),
    "gde_serve_mixed": (_int, [_p, _p, ctypes.POINTER(Params), _i64, _p, _p, _p, _p, _p, _dbl, _p, _int, _int, _i64,
                               _p, _p, _p, ctypes.POINTER(Stats)]),
    "gde_sor": (_int, [_p, _p, ctypes.POINTER(Params), _i64, _p, _p, _int, _p, _p, _int, _int, _i64, _p, _p,
                       ctypes.POINTER(Stats)]),
    "gde_graph_colors": (_int, [_p, _p, _p]),
    "gde_katz_spectral_bounds": (_int, [_p, _p, _dbl, _int, _dbl, _p, _p, _p, _p]),
    "gde_ctx_trace": (_int, [_p, _int]),
    "gde_ctx_trace_read": (_int, [_p, _p, _i64, _p, _p, _p]),
    "gde_ctx_set_wait_limit": (_int, [_p, _i64]),
    "gde_server_start": (_int, [_p, _p, ctypes.POINTER(Params), _i64, _dbl, _dbl, ctypes.POINTER(_p)]),
    "gde_server_submit": (_int, [_p, _int, _i32, _dbl, _dbl, _p, _int, ctypes.POINTER(_i64)]),
    "gde_server_poll": (_int, [_p, _i64, ctypes.POINTER(_int), ctypes.POINTER(_dbl), ctypes.POINTER(_i32),
                               ctypes.POINTER(_dbl)]),
    "gde_server_poll_many": (_int, [_p, _p, _i64, _p, _p, _p, _p]),
    "gde_server_info": (_int, [_p, ctypes.POINTER(_int), ctypes.POINTER(_i64), ctypes.POINTER(_dbl),
                               ctypes.POINTER(_i64)]),
    "gde_server_stop": (_int, [_p, _int, ctypes.POINTER(_i64)]),
    "gde_solve_noalloc": (_int, [_p, _p, ctypes.POINTER(Params), _i32, _dbl, _p, _p, _int, _p, _p]),
}

_lib = None
_lock = threading.Lock()


class GDEError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libgde.so (building it first when absent)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise OSError(f"{path} is missing: build it with gde._build.build()")
            _build.build()
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def check(ctx_ptr, status: int, what: str) -> None:
    if status != GDE_OK:
        L = load()
        msg = L.gde_last_error(ctx_ptr).decode() if ctx_ptr else L.gde_status_str(status).decode()
        raise GDEError(status, f"{what}: {msg}")
