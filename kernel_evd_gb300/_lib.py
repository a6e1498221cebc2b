"""ctypes binding of ``libkevd.so`` (the C ABI declared in include/kevd.h).

The library is built in-tree by ``python -m kernel_evd_gb300.build``.  There
is no fallback: if the shared library is missing every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("KEVD_LIB") or os.path.join(HERE, "lib", "libkevd.so")

KEVD_FP64 = 0
KEVD_MIXED = 1

STATUS = {
    0: "KEVD_OK", 1: "KEVD_ERR_ARG", 2: "KEVD_ERR_CUDA", 3: "KEVD_ERR_NONPOS_DTIL",
    4: "KEVD_ERR_POTRF", 5: "KEVD_ERR_NONPOS_QTIL", 6: "KEVD_ERR_SYEVD", 7: "KEVD_ERR_NOMEM",
    8: "KEVD_ERR_TIMEOUT",
}


class KevdError(RuntimeError):
    """A non-zero kevd status.  ``code`` is the enum value, ``name`` its name."""

    def __init__(self, code: int, msg: str):
        self.code = int(code)
        self.name = STATUS.get(self.code, "KEVD_ERR_UNKNOWN")
        super().__init__(f"{self.name}: {msg}")


class RpcholParams(C.Structure):
    _fields_ = [("k_max", C.c_int64), ("block", C.c_int32), ("max_rounds", C.c_int32),
                ("tol", C.c_double), ("err_target", C.c_double), ("seed", C.c_uint64),
                ("uniforms", C.POINTER(C.c_double)), ("precision", C.c_int32)]


class RpcholResult(C.Structure):
    _fields_ = [("rank", C.c_int64), ("rounds", C.c_int32), ("trace_error", C.c_double)]


class EvdInfo(C.Structure):
    _fields_ = [("trace_A", C.c_double), ("shift", C.c_double)]


class RpcholJob(C.Structure):
    _fields_ = [("X", C.c_void_p), ("N", C.c_int64), ("d", C.c_int32), ("block", C.c_int32),
                ("scale", C.c_double), ("F", C.c_void_p), ("ldF", C.c_int64), ("k_max", C.c_int64),
                ("max_rounds", C.c_int32), ("pad", C.c_int32), ("seed", C.c_uint64), ("piv", C.c_void_p),
                ("result", RpcholResult)]


class CalibJob(C.Structure):
    _fields_ = [("X", C.c_void_p), ("N", C.c_int64), ("d", C.c_int32), ("n_scales", C.c_int32),
                ("scales", C.c_void_p), ("sums", C.c_void_p)]


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("factor_workers", C.c_int32), ("max_query_batch", C.c_int64),
                ("hbm_budget_bytes", C.c_uint64), ("batch_window_us", C.c_double)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("model_id", C.c_int64), ("latency_s", C.c_double),
                ("queue_s", C.c_double), ("batch_rows", C.c_int64), ("trace_error", C.c_double),
                ("rank", C.c_int64), ("message", C.c_char * 192)]


class EvdDump(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_double)) for n in ("c1", "dtil", "cq", "qtil", "A", "B", "W", "Z")]


_P = C.c_void_p
_I64 = C.c_int64
_I32 = C.c_int32
_D = C.c_double

SIGNATURES = {
    "kevd_ctx_create": (C.c_int, [C.c_int, C.POINTER(_P)]),
    "kevd_ctx_destroy": (None, [_P]),
    "kevd_last_error": (C.c_char_p, [_P]),
    "kevd_status_name": (C.c_char_p, [C.c_int]),
    "kevd_abi_version": (C.c_int, []),
    "kevd_profile_enable": (C.c_int, [_P, C.c_int]),
    "kevd_profile_read": (C.c_int, [_P, C.c_int, C.c_char_p, C.c_int, C.POINTER(_D), C.POINTER(_I64)]),
    "kevd_launch_count": (_I64, [_P]),
    "kevd_peak_rate": (C.c_int, [_P, _I32, C.POINTER(_D), C.POINTER(_D), _P]),
    "kevd_hankel_rows": (C.c_int, [_P, _P, _I64, _I64, _I64, _P, _P]),
    "kevd_kernel_block": (C.c_int, [_P, _P, _I64, _I32, _D, _P, _I64, _I64, _P, _I64, _I32, _P, _I64, _P]),
    "kevd_calibrate": (C.c_int, [_P, _P, _I64, _I32, _P, _I32, _P, _P]),
    "kevd_calibrate_fp64": (C.c_int, [_P, _P, _I64, _I32, _P, _I32, _P, _P]),
    "kevd_calibrate_batched": (C.c_int, [_P, C.POINTER(CalibJob), _I32, _I32, _P]),
    "kevd_rpchol_batched": (C.c_int, [_P, C.POINTER(RpcholJob), _I32, _I32, _P]),
    "kevd_calibrate_noalloc": (C.c_int, [_P, _I64, _I32, _P, _I32, _P, _P]),
    "kevd_calibrate_select": (C.c_int, [_P, _P, _I32, _I64, _P, _P, _P, _P, _P]),
    "kevd_pair_median": (C.c_int, [_P, _P, _I64, _I32, _P, _P, _I64, _P, _P]),
    "kevd_rpchol": (C.c_int, [_P, _P, _I64, _I32, _D, C.POINTER(RpcholParams), _P, _I64, _P, _P, _P,
                              C.POINTER(RpcholResult), _P]),
    "kevd_linv_from_factor": (C.c_int, [_P, _P, _I32, _I64, _P, _I64, _P, _P]),
    "kevd_bistochastic_evd": (C.c_int, [_P, _P, _I32, _I64, _I64, _I64, _I32, _P, _P,
                                        C.POINTER(EvdInfo), C.POINTER(EvdDump), _P]),
    "kevd_weighted_gram": (C.c_int, [_P, _P, _I32, _I64, _I64, _I64, _P, _P, _P]),
    "kevd_weighted_gram2": (C.c_int, [_P, _P, _I32, _I64, _I64, _I64, _P, _P, _P, _P, _P]),
    "kevd_ks_generate": (C.c_int, [_P, _I32, _I32, _I32, _P, _P, _P, _I64, _P, _P, _P]),
    "kevd_factor_from_linv": (C.c_int, [_P, _P, _I64, _I32, _D, _P, _I64, _P, _I32, _P, _I64, _P]),
    "kevd_factor_from_pivots": (C.c_int, [_P, _P, _I64, _I32, _D, _P, _I64, _I32, _P, _I64, _P]),
    "kevd_nystrom_prepare": (C.c_int, [_P, _P, _I64, _I32, _D, _P, _I32, _I64, _P, _I64, _I32,
                                       C.POINTER(_P), _P]),
    "kevd_nystrom_eval": (C.c_int, [_P, _P, _P, _I64, _P, _P]),
    "kevd_model_destroy": (None, [_P]),
    "kevd_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(_P)]),
    "kevd_server_destroy": (None, [_P]),
    "kevd_factorization_footprint": (_I64, [_I64, C.c_int32, _I64, C.c_int32, C.c_int32]),
    "kevd_server_submit_factorization": (C.c_int, [_P, _P, _I64, C.c_int32, C.c_double, _I64, C.c_int32,
                                                   C.c_int32, C.c_uint64, C.c_int32, C.POINTER(_I64)]),
    "kevd_server_submit_query": (C.c_int, [_P, _I64, _P, _I64, _P, C.POINTER(_I64)]),
    "kevd_server_wait": (C.c_int, [_P, _I64, C.c_double, C.POINTER(RequestInfo)]),
    "kevd_server_release_model": (C.c_int, [_P, _I64]),
    "kevd_server_stats": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(_I64)]),
    "kevd_server_memory": (C.c_int, [_P, C.POINTER(_I64), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                     C.POINTER(C.c_int32)]),
}

_lib = None


def load() -> C.CDLL:
    """Load libkevd.so once; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m kernel_evd_gb300.build`")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, ctx=None):
    if status != 0:
        msg = ""
        if ctx is not None:
            raw = load().kevd_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise KevdError(status, msg)
