"""ctypes binding of the C ABI in include/ceos_gb300.h.

The shared library is built in-tree by ``ceos_gb300.build``. There is no CPU
fallback: if the library is missing or no CUDA device is visible, the calls
raise instead of silently computing something else.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libceos_gb300.so")

OK = 0
ERR_ARG = -1
ERR_NOT_BUILT = -2
ERR_PROBED_POINTS = -3
ERR_PROBED_VECTORS = -4
ERR_UPDATE_DEL = -5
ERR_UPDATE_TOPM = -6
ERR_CUDA = -7
ERR_NO_DEVICE = -8
ERR_UNSUPPORTED = -9
ERR_DEVICE_LIMIT = -10
ERR_TIMEOUT = -11
ERR_BUSY = -12

ALGO_DENSE, ALGO_COCEOS, ALGO_HASH = 0, 1, 2
PRECISION_FP32, PRECISION_SPLIT_BF16 = 0, 1

F32P = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
I32P = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
U8P = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
VP = C.c_void_p
IP = C.POINTER(C.c_int)
U64P = C.POINTER(C.c_uint64)


class ServerConfig(C.Structure):
    """struct ceos_server_config."""
    _fields_ = [("algo", C.c_int), ("n_slots", C.c_int), ("max_batch", C.c_int),
                ("max_neighbors", C.c_int), ("max_probed_vectors", C.c_int),
                ("mem_budget_bytes", C.c_longlong), ("use_graphs", C.c_int)]


class ServerStats(C.Structure):
    """struct ceos_server_stats."""
    _fields_ = [("requests", C.c_longlong), ("queries", C.c_longlong), ("batches", C.c_longlong),
                ("graph_launches", C.c_longlong), ("graphs_captured", C.c_longlong),
                ("updates", C.c_longlong), ("slots", C.c_int), ("slot_bytes", C.c_longlong),
                ("mean_batch_queries", C.c_double), ("p50_ms", C.c_double), ("p90_ms", C.c_double),
                ("p99_ms", C.c_double), ("max_ms", C.c_double), ("mean_ms", C.c_double),
                ("busy_s", C.c_double)]


# name -> (restype, argtypes); every entry point declared in include/ceos_gb300.h
SIGNATURES = {
    "ceos_abi_version": (C.c_int, []),
    "ceos_last_error": (C.c_char_p, []),
    "ceos_device_count": (C.c_int, []),
    "ceos_set_log_level": (None, [C.c_int]),
    "ceos_flush_l2": (C.c_int, [C.c_long]),
    "ceos_debug_stall_tensor_products": (C.c_int, [C.c_int]),
    "ceos_create": (C.c_int, [C.c_int, C.c_int, C.POINTER(VP)]),
    "ceos_destroy": (None, [VP]),
    "ceos_set_index_param": (C.c_int, [VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "ceos_get_index_param": (C.c_int, [VP, IP, IP, IP, IP, IP, IP]),
    "ceos_set_threads": (C.c_int, [VP, C.c_int]),
    "ceos_clear": (C.c_int, [VP]),
    "ceos_set_query_param": (C.c_int, [VP, C.c_int, C.c_int, C.c_int]),
    "ceos_get_query_param": (C.c_int, [VP, IP, IP, IP]),
    "ceos_set_centering": (C.c_int, [VP, C.c_int]),
    "ceos_get_centering": (C.c_int, [VP, IP]),
    "ceos_set_precision": (C.c_int, [VP, C.c_int]),
    "ceos_build": (C.c_int, [VP, F32P]),
    "ceos_search": (C.c_int, [VP, F32P, C.c_int, C.c_int, C.c_int, I32P, F32P]),
    "ceos_build_coceos_est": (C.c_int, [VP, F32P]),
    "ceos_search_coceos_est": (C.c_int, [VP, F32P, C.c_int, C.c_int, C.c_int, I32P, F32P]),
    "ceos_build_ceos_hash": (C.c_int, [VP, F32P]),
    "ceos_search_ceos_hash": (C.c_int, [VP, F32P, C.c_int, C.c_int, C.c_int, I32P, F32P]),
    "ceos_search_device": (C.c_int, [VP, C.c_int, VP, C.c_int, C.c_int, VP, VP, VP]),
    "ceos_search_coceos_est_device_noalloc": (C.c_int, [VP, VP, C.c_int, C.c_int, VP, VP, VP]),
    "ceos_get_buckets": (C.c_int, [VP, I32P, F32P]),
    "ceos_get_projections": (C.c_int, [VP, F32P]),
    "ceos_get_sign_bits": (C.c_int, [VP, U8P]),
    "ceos_last_timings": (C.c_int, [VP, F32P, C.c_int]),
    "ceos_timing_name": (C.c_char_p, [VP, C.c_int]),
    "ceos_stream_create": (C.c_int, [C.c_int, C.POINTER(VP)]),
    "ceos_stream_destroy": (None, [VP]),
    "ceos_stream_set_index_param": (C.c_int, [VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "ceos_stream_set_threads": (C.c_int, [VP, C.c_int]),
    "ceos_stream_set_precision": (C.c_int, [VP, C.c_int]),
    "ceos_stream_clear": (C.c_int, [VP]),
    "ceos_stream_set_query_param": (C.c_int, [VP, C.c_int, C.c_int, C.c_int]),
    "ceos_stream_get_query_param": (C.c_int, [VP, IP, IP, IP]),
    "ceos_stream_build": (C.c_int, [VP, F32P, C.c_int]),
    "ceos_stream_update": (C.c_int, [VP, VP, C.c_int, C.c_int]),
    "ceos_stream_estimate_search": (C.c_int, [VP, F32P, C.c_int, C.c_int, C.c_int, I32P, F32P]),
    "ceos_stream_hash_search": (C.c_int, [VP, F32P, C.c_int, C.c_int, C.c_int, I32P, F32P]),
    "ceos_stream_size": (C.c_int, [VP, IP]),
    "ceos_stream_get_buckets": (C.c_int, [VP, I32P, F32P]),
    "ceos_stream_set_reserve": (C.c_int, [VP, C.c_int]),
    "ceos_stream_get_reserve": (C.c_int, [VP, IP]),
    "ceos_stream_delete": (C.c_int, [VP, VP, C.c_int]),
    "ceos_bruteforce_fp64": (C.c_int, [F32P, C.c_long, C.c_int, F32P, C.c_int, C.c_int, I32P,
                                       np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")]),
    "ceos_get_shape": (C.c_int, [VP, IP, IP]),
    "ceos_get_precision": (C.c_int, [VP, IP]),
    "ceos_stream_get_index_param": (C.c_int, [VP, IP, IP, IP, IP, IP]),
    "ceos_stream_get_precision": (C.c_int, [VP, IP]),
    "ceos_build_from_file": (C.c_int, [VP, C.c_char_p, C.c_int]),
    "ceos_stream_build_from_file": (C.c_int, [VP, C.c_char_p, C.c_int]),
    "ceos_save": (C.c_int, [VP, C.c_char_p]),
    "ceos_load": (C.c_int, [C.c_char_p, C.POINTER(VP)]),
    "ceos_stream_save": (C.c_int, [VP, C.c_char_p]),
    "ceos_stream_load": (C.c_int, [C.c_char_p, C.POINTER(VP)]),
    "ceos_server_config_init": (C.c_int, [C.POINTER(ServerConfig)]),
    "ceos_server_create": (C.c_int, [VP, C.POINTER(ServerConfig), C.POINTER(VP)]),
    "ceos_server_create_stream": (C.c_int, [VP, C.POINTER(ServerConfig), C.POINTER(VP)]),
    "ceos_server_destroy": (None, [VP]),
    "ceos_server_submit": (C.c_int, [VP, VP, C.c_int, C.c_int, C.c_int, VP, VP, U64P]),
    "ceos_server_submit_update": (C.c_int, [VP, VP, C.c_int, C.c_int, U64P]),
    "ceos_server_submit_delete": (C.c_int, [VP, VP, C.c_int, U64P]),
    "ceos_server_wait": (C.c_int, [VP, C.c_uint64, C.c_int]),
    "ceos_server_get_stats": (C.c_int, [VP, C.POINTER(ServerStats)]),
    "ceos_server_reset_stats": (C.c_int, [VP]),
}

_lock = threading.Lock()
_lib = None


class CEOsError(RuntimeError):
    """A CUDA or device-limit failure inside the library."""


def lib():
    """Load the in-tree shared library (building it first if it is absent)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                from . import build as _build

                _build.build()
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            if L.ceos_abi_version() != 1:
                raise CEOsError("libceos_gb300.so ABI version mismatch")
            _lib = L
    return _lib


def last_error() -> str:
    return lib().ceos_last_error().decode(errors="replace")


def check(status: int) -> None:
    """Translate a C ABI status into the Python exception the reference's
    error paths correspond to (they print and exit(1))."""
    if status == OK:
        return
    msg = last_error()
    if status in (ERR_ARG, ERR_PROBED_POINTS, ERR_PROBED_VECTORS, ERR_UPDATE_DEL, ERR_UPDATE_TOPM,
                  ERR_UNSUPPORTED):
        raise ValueError(msg)
    if status in (ERR_NOT_BUILT, ERR_BUSY):
        raise RuntimeError(msg)
    if status == ERR_TIMEOUT:
        raise TimeoutError(msg)
    raise CEOsError(f"[{status}] {msg}")


def bruteforce_fp64(X, Q, k: int):
    """Exact FP64 top-k inner products on the GPU (ground truth for recall)."""
    X = np.ascontiguousarray(X, dtype=np.float32)
    Q = np.ascontiguousarray(Q, dtype=np.float32)
    ids = np.zeros((Q.shape[0], k), np.int32)
    scores = np.zeros((Q.shape[0], k), np.float64)
    check(lib().ceos_bruteforce_fp64(X, X.shape[0], X.shape[1], Q, Q.shape[0], k, ids, scores))
    return ids, scores
