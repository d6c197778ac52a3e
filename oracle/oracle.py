"""ctypes harness around the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``. The shipped library never imports
this module.

The classes mirror the reference's pybind11 module (python/python_wrapper.cpp
:13-74): ``CEOs(n_points, n_features)`` and ``streamCEOs(n_features)`` with
``setIndexParam``, the ``n_probed_vectors`` / ``n_probed_points`` / ``n_cand``
attributes and the build / search / update methods, so that a parity test can
run the same script against the oracle and against the GPU library.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
# The same source built like the reference's own release build (-O3 with the
# host's native instruction set, fused multiply-adds allowed): the timed CPU
# baseline. liboracle.so stays the bit-exact checker.
_TIMED_PATH = os.path.join(_HERE, "liboracle_timed.so")
_REF_FFHT = os.path.join(_HERE, "_ref", "libffht_ref.so")
_lock = threading.Lock()
_libs = {}

_F32P = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_F64P = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_I32P = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_U8P = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")

ST_MESSAGES = {
    -1: "invalid argument",
    -2: "index not built",
    -3: "Number of probed points must be smaller than number of indexed top-m points",
    -4: "Number of probed vectors must be smaller than n_proj * n_repeats",
    -5: "Number of removed points must be smaller than the current number of points",
    -6: "There is not enough indexed top-points for coCEOs after update",
}


def build(force: bool = False, timed: bool = False) -> str:
    """Compile liboracle.so (or, with timed, liboracle_timed.so) with the
    committed Makefile (g++, OpenMP)."""
    src = os.path.join(_HERE, "ceos_oracle.cpp")
    path = _TIMED_PATH if timed else _LIB_PATH
    if force or not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, os.path.basename(path)], check=True)
    return path


def reference_root() -> str:
    """Root of the reference project's sources (the directory holding src/):
    $CEOS_REFERENCE, else where this build environment mounts it."""
    return os.environ.get("CEOS_REFERENCE", "/root/reference")


def build_ref() -> str | None:
    """Compile the reference's FFHT and index classes (x86 only) into
    oracle/_ref when the reference sources are present; returns the FFHT
    library's path or None."""
    if os.path.exists(_REF_FFHT) and os.path.exists(os.path.join(_HERE, "_ref", "libceos_ref.so")):
        return _REF_FFHT
    root = reference_root()
    if not os.path.isdir(os.path.join(root, "src")) or os.uname().machine not in ("x86_64", "AMD64"):
        return _REF_FFHT if os.path.exists(_REF_FFHT) else None
    try:
        subprocess.run(["make", "-s", "-C", _HERE, "ref", f"CEOS_REFERENCE={root}"], check=True,
                       capture_output=True)
    except (subprocess.CalledProcessError, FileNotFoundError):
        return None
    return _REF_FFHT if os.path.exists(_REF_FFHT) else None


def lib(timed: bool = False):
    with _lock:
        if timed not in _libs:
            L = C.CDLL(build(timed=timed))
            vp = C.c_void_p
            L.orc_sign_bits.argtypes = [C.c_int, C.c_int, _U8P]
            L.orc_sign_bits_std.argtypes = [C.c_int, C.c_int, _U8P]
            L.orc_fwht.argtypes = [_F32P, C.c_int]
            L.orc_fwht.restype = None
            L.orc_fht_dim.argtypes = [C.c_int, C.c_int]
            L.orc_project.argtypes = [_F32P, C.c_long, C.c_int, C.c_int, C.c_int, C.c_int, _U8P, _F32P, C.c_int]
            L.orc_bruteforce.argtypes = [_F32P, C.c_long, C.c_int, _F32P, C.c_int, C.c_int, _I32P, _F64P, C.c_int]
            L.orc_ceos_create.argtypes = [C.c_int, C.c_int]
            L.orc_ceos_create.restype = vp
            L.orc_ceos_destroy.argtypes = [vp]
            L.orc_ceos_destroy.restype = None
            L.orc_ceos_set_param.argtypes = [vp] + [C.c_int] * 5
            L.orc_ceos_set_param.restype = None
            L.orc_ceos_set_query.argtypes = [vp, C.c_int, C.c_int, C.c_int]
            L.orc_ceos_set_query.restype = None
            L.orc_ceos_get_query.argtypes = [vp] + [C.POINTER(C.c_int)] * 3
            L.orc_ceos_get_query.restype = None
            L.orc_ceos_fht_dim.argtypes = [vp]
            L.orc_ceos_set_split.argtypes = [vp, C.c_int, C.c_int]
            L.orc_ceos_set_split.restype = None
            L.orc_stream_set_split.argtypes = [vp, C.c_int, C.c_int]
            L.orc_stream_set_split.restype = None
            L.orc_bf16_round.argtypes = [C.c_float]
            L.orc_bf16_round.restype = C.c_float
            L.orc_dot_bf16.argtypes = [_F32P, _F32P, C.c_int]
            L.orc_dot_bf16.restype = C.c_float
            L.orc_dot.argtypes = [_F32P, _F32P, C.c_int]
            L.orc_dot.restype = C.c_float
            for nm in ("dense", "coceos", "hash"):
                getattr(L, f"orc_ceos_build_{nm}").argtypes = [vp, _F32P]
                getattr(L, f"orc_ceos_search_{nm}").argtypes = [vp, _F32P, C.c_int, C.c_int, _I32P, _F32P]
            L.orc_ceos_get_buckets.argtypes = [vp, _I32P, _F32P]
            L.orc_ceos_get_projections.argtypes = [vp, _F32P]
            L.orc_stream_create.argtypes = [C.c_int]
            L.orc_stream_create.restype = vp
            L.orc_stream_destroy.argtypes = [vp]
            L.orc_stream_destroy.restype = None
            L.orc_stream_set_param.argtypes = [vp] + [C.c_int] * 5
            L.orc_stream_set_param.restype = None
            L.orc_stream_set_query.argtypes = [vp, C.c_int, C.c_int, C.c_int]
            L.orc_stream_set_query.restype = None
            L.orc_stream_get_query.argtypes = [vp] + [C.POINTER(C.c_int)] * 3
            L.orc_stream_get_query.restype = None
            L.orc_stream_size.argtypes = [vp]
            L.orc_stream_build.argtypes = [vp, _F32P, C.c_int]
            L.orc_stream_update.argtypes = [vp, _F32P, C.c_int, C.c_int]
            L.orc_stream_estimate_search.argtypes = [vp, _F32P, C.c_int, C.c_int, _I32P, _F32P]
            L.orc_stream_hash_search.argtypes = [vp, _F32P, C.c_int, C.c_int, _I32P, _F32P]
            L.orc_stream_get_buckets.argtypes = [vp, _I32P, _F32P]
            L.orc_ceos_set_centering.argtypes = [vp, C.c_int]
            L.orc_ceos_set_centering.restype = None
            L.orc_stream_set_exact.argtypes = [vp, C.c_int]
            L.orc_stream_set_exact.restype = None
            L.orc_stream_delete.argtypes = [vp, _I32P, C.c_int]
            _libs[timed] = L
    return _libs[timed]


def _check(st: int) -> None:
    if st != 0:
        raise ValueError(ST_MESSAGES.get(st, f"oracle status {st}"))


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def fht_dim(n_proj: int, n_features: int) -> int:
    return int(lib().orc_fht_dim(n_proj, n_features))


def sign_bits(n_bits: int, seed: int) -> np.ndarray:
    out = np.zeros(n_bits, np.uint8)
    _check(lib().orc_sign_bits(n_bits, seed, out))
    return out


def sign_bits_std(n_bits: int, seed: int) -> np.ndarray:
    out = np.zeros(n_bits, np.uint8)
    _check(lib().orc_sign_bits_std(n_bits, seed, out))
    return out


def fwht(v) -> np.ndarray:
    v = _f32(v).copy()
    n = v.shape[-1]
    L = n.bit_length() - 1
    flat = v.reshape(-1, n)
    for row in flat:
        r = np.ascontiguousarray(row)
        lib().orc_fwht(r, L)
        row[:] = r
    return flat.reshape(v.shape)


def project(X, n_proj: int, n_repeats: int, seed: int, n_threads: int = 0) -> np.ndarray:
    """Row-major n x (n_proj * n_repeats) projections with the reference's
    sign tables for ``seed``."""
    X = _f32(X)
    n, d = X.shape
    F = fht_dim(n_proj, d)
    bits = sign_bits(F * 3 * n_repeats, seed)
    P = np.zeros((n, n_proj * n_repeats), np.float32)
    _check(lib().orc_project(X, n, d, F, n_proj, n_repeats, bits, P, n_threads))
    return P


def bruteforce(X, Q, k: int, n_threads: int = 0):
    """Exact top-k maximum inner product in float64: (ids int32, scores f64)."""
    X, Q = _f32(X), _f32(Q)
    nq = Q.shape[0]
    ids = np.zeros((nq, k), np.int32)
    sc = np.zeros((nq, k), np.float64)
    _check(lib().orc_bruteforce(X, X.shape[0], X.shape[1], Q, nq, k, ids, sc, n_threads))
    return ids, sc


def bf16_round(x) -> np.ndarray:
    x = _f32(x)
    return np.array([lib().orc_bf16_round(float(v)) for v in x.ravel()], np.float32).reshape(x.shape)


def dot(q, x) -> float:
    q, x = _f32(q), _f32(x)
    return float(lib().orc_dot(q, x, q.shape[0]))


def dot_bf16(q, x) -> float:
    q, x = _f32(q), _f32(x)
    return float(lib().orc_dot_bf16(q, x, q.shape[0]))


def ref_ffht(v) -> np.ndarray | None:
    """The reference's fht_float run on each row of v (None when the
    reference FFHT could not be built on this machine)."""
    path = build_ref()
    if path is None:
        return None
    L = C.CDLL(path)
    L.fht_float.argtypes = [_F32P, C.c_int]
    v = _f32(v).copy()
    n = v.shape[-1]
    flat = v.reshape(-1, n)
    for i in range(flat.shape[0]):
        r = np.ascontiguousarray(flat[i])
        L.fht_float(r, n.bit_length() - 1)
        flat[i] = r
    return flat.reshape(v.shape)


class _Attrs:
    _get_q = None
    _set_q = None

    def _q(self):
        s, p, c = C.c_int(), C.c_int(), C.c_int()
        self._get_q(self._h, C.byref(s), C.byref(p), C.byref(c))
        return s.value, p.value, c.value

    @property
    def n_probed_vectors(self):
        return self._q()[0]

    @n_probed_vectors.setter
    def n_probed_vectors(self, v):
        s, p, c = self._q()
        self._set_q(self._h, int(v), p, c)

    @property
    def n_probed_points(self):
        return self._q()[1]

    @n_probed_points.setter
    def n_probed_points(self, v):
        s, p, c = self._q()
        self._set_q(self._h, s, int(v), c)

    @property
    def n_cand(self):
        return self._q()[2]

    @n_cand.setter
    def n_cand(self, v):
        s, p, c = self._q()
        self._set_q(self._h, s, p, int(v))


class CEOs(_Attrs):
    """Oracle twin of the reference's ``CEOs.CEOs`` (src/CEOs.h:18-114).
    timed=True runs the natively optimised build of the same source."""

    def __init__(self, n_points: int, n_features: int, timed: bool = False):
        L = lib(timed)
        self._L = L
        self._h = L.orc_ceos_create(int(n_points), int(n_features))
        self._get_q = L.orc_ceos_get_query
        self._set_q = L.orc_ceos_set_query
        self.n_points, self.n_features = int(n_points), int(n_features)
        self._centering = False
        self._D = 256
        self._R = 1
        self._m = 100

    @property
    def centering(self):
        return self._centering

    @centering.setter
    def centering(self, v):
        self._centering = bool(v)
        self._L.orc_ceos_set_centering(self._h, 1 if v else 0)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.orc_ceos_destroy(h)
            self._h = None

    def setIndexParam(self, n_proj, n_repeats=1, top_m=10, n_threads=-1, random_seed=-1):
        self._D, self._R, self._m = int(n_proj), int(n_repeats), int(top_m)
        self._L.orc_ceos_set_param(self._h, self._D, self._R, self._m, int(n_threads), int(random_seed))

    def set_threads(self, n_threads):
        pass

    @property
    def precision(self):
        return getattr(self, "_precision", "fp32")

    @precision.setter
    def precision(self, v):
        self._precision = v
        self._L.orc_ceos_set_split(self._h, 1 if v == "split_bf16" else 0, 4)

    def _search(self, fn, Q, k):
        Q = _f32(Q)
        nq = Q.shape[0]
        ids = np.zeros((nq, k), np.int32)
        d = np.zeros((nq, k), np.float32)
        _check(fn(self._h, Q, nq, int(k), ids, d))
        return ids, d

    def build(self, dataset):
        _check(self._L.orc_ceos_build_dense(self._h, _f32(dataset)))

    def search(self, queries, n_neighbors, verbose=False):
        return self._search(self._L.orc_ceos_search_dense, queries, n_neighbors)

    def build_coCEOs_Est(self, dataset):
        _check(self._L.orc_ceos_build_coceos(self._h, _f32(dataset)))

    def search_coCEOs_Est(self, queries, n_neighbors, verbose=False):
        return self._search(self._L.orc_ceos_search_coceos, queries, n_neighbors)

    def build_CEOs_Hash(self, dataset):
        _check(self._L.orc_ceos_build_hash(self._h, _f32(dataset)))

    def search_CEOs_Hash(self, queries, n_neighbors, verbose=False):
        return self._search(self._L.orc_ceos_search_hash, queries, n_neighbors)

    def buckets(self):
        """(ids, values) as [C][2][m]: end 0 = closest, end 1 = furthest."""
        Cc = self._D * self._R
        ids = np.zeros((Cc, 2, self._m), np.int32)
        vals = np.zeros((Cc, 2, self._m), np.float32)
        _check(self._L.orc_ceos_get_buckets(self._h, ids, vals))
        return ids, vals

    def projections(self):
        P = np.zeros((self.n_points, self._D * self._R), np.float32)
        _check(self._L.orc_ceos_get_projections(self._h, P))
        return P


class streamCEOs(_Attrs):
    """Oracle twin of the reference's ``CEOs.streamCEOs`` (src/streamCEOs.h).
    timed=True runs the natively optimised build of the same source."""

    def __init__(self, n_features: int, timed: bool = False):
        L = lib(timed)
        self._L = L
        self._h = L.orc_stream_create(int(n_features))
        self._get_q = L.orc_stream_get_query
        self._set_q = L.orc_stream_set_query
        self.n_features = int(n_features)
        self._D, self._R, self._m = 256, 1, 100

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.orc_stream_destroy(h)
            self._h = None

    def setIndexParam(self, n_proj, n_repeats=1, top_points=1, n_threads=-1, random_seed=-1):
        self._D, self._R, self._m = int(n_proj), int(n_repeats), int(top_points)
        self._L.orc_stream_set_param(self._h, self._D, self._R, self._m, int(n_threads), int(random_seed))

    def set_threads(self, n_threads):
        pass

    @property
    def size(self):
        return int(self._L.orc_stream_size(self._h))

    @property
    def precision(self):
        return getattr(self, "_precision", "fp32")

    @precision.setter
    def precision(self, v):
        self._precision = v
        self._L.orc_stream_set_split(self._h, 1 if v == "split_bf16" else 0, 4)

    def build(self, dataset):
        X = _f32(dataset)
        _check(self._L.orc_stream_build(self._h, X, X.shape[0]))

    def update(self, new_dataset, n_delPoints=0):
        X = _f32(new_dataset).reshape(-1, self.n_features)
        _check(self._L.orc_stream_update(self._h, X, X.shape[0], int(n_delPoints)))

    def set_reserve(self, reserve: int):
        """Exact maintenance (reserve >= 0): buckets recomputed over the live rows
        after every update / delete (the GPU keeps top_m + reserve per list)."""
        self._L.orc_stream_set_exact(self._h, 1 if int(reserve) >= 0 else 0)

    def delete(self, ids):
        ids = np.ascontiguousarray(np.asarray(ids, dtype=np.int32).ravel())
        _check(self._L.orc_stream_delete(self._h, ids, ids.size))

    def _search(self, fn, Q, k):
        Q = _f32(Q)
        nq = Q.shape[0]
        ids = np.zeros((nq, k), np.int32)
        d = np.zeros((nq, k), np.float32)
        _check(fn(self._h, Q, nq, int(k), ids, d))
        return ids, d

    def estimate_search(self, queries, n_neighbors, verbose=False):
        return self._search(self._L.orc_stream_estimate_search, queries, n_neighbors)

    def hash_search(self, queries, n_neighbors, verbose=False):
        return self._search(self._L.orc_stream_hash_search, queries, n_neighbors)

    def buckets(self):
        Cc = self._D * self._R
        ids = np.zeros((Cc, 2, self._m), np.int32)
        vals = np.zeros((Cc, 2, self._m), np.float32)
        _check(self._L.orc_stream_get_buckets(self._h, ids, vals))
        return ids, vals
