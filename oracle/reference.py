"""ctypes harness around the reference's own index classes, compiled unchanged
from its sources into oracle/_ref/libceos_ref.so (``make -C oracle ref``,
x86 only, where the reference sources are present).

TEST INFRASTRUCTURE ONLY: it pins the oracle restatement to the reference
(tests/test_oracle.py) and generates the golden fixtures under tests/golden/
(make_reference_golden.py). The product never loads it, and the GPU machine has
no reference sources, so GPU tests use the committed fixtures instead.

``RefCEOs`` wraps ``CEOs`` (src/CEOs.h:18-114) and ``RefStreamCEOs`` wraps
``streamCEOs`` (src/streamCEOs.h:12-107). Buckets come back in the layout the
oracle and the GPU library use: ids and values as [n_proj*n_repeats][2][top_m]
(end 0 = closest, values v; end 1 = furthest, values -v), read out of the
reference's column-major matrix_P (4m x C, ids stored as float,
src/CEOs.cpp:417-428) or matrix_H (2m x C, src/CEOs.cpp:819-828).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import oracle as _oracle

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_ref", "libceos_ref.so")
_F32P = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_I32P = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lib = None

KIND_DENSE, KIND_COCEOS, KIND_HASH = 0, 1, 2


def available() -> bool:
    """True when the reference library exists or can be built here."""
    if not os.path.exists(_LIB_PATH):
        _oracle.build_ref()
    return os.path.exists(_LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("the reference library oracle/_ref/libceos_ref.so is not built "
                               "(needs the reference sources and an x86 host)")
        L = C.CDLL(_LIB_PATH)
        vp = C.c_void_p
        L.ref_ceos_new.argtypes = [C.c_int, C.c_int]
        L.ref_ceos_new.restype = vp
        L.ref_ceos_free.argtypes = [vp]
        L.ref_ceos_set_param.argtypes = [vp] + [C.c_int] * 5
        L.ref_ceos_set_query.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        L.ref_ceos_build.argtypes = [vp, C.c_int, _F32P, C.c_int, C.c_int]
        L.ref_ceos_search.argtypes = [vp, C.c_int, _F32P, C.c_int, C.c_int, C.c_int, _I32P, _F32P]
        L.ref_ceos_buckets.argtypes = [vp, C.c_int, _F32P]
        L.ref_ceos_buckets.restype = C.c_int
        L.ref_stream_new.argtypes = [C.c_int]
        L.ref_stream_new.restype = vp
        L.ref_stream_free.argtypes = [vp]
        L.ref_stream_set_param.argtypes = [vp] + [C.c_int] * 5
        L.ref_stream_set_query.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        L.ref_stream_build.argtypes = [vp, _F32P, C.c_int, C.c_int]
        L.ref_stream_update.argtypes = [vp, _F32P, C.c_int, C.c_int, C.c_int]
        L.ref_stream_size.argtypes = [vp]
        L.ref_stream_size.restype = C.c_int
        L.ref_stream_search.argtypes = [vp, C.c_int, _F32P, C.c_int, C.c_int, C.c_int, _I32P, _F32P]
        L.ref_stream_buckets.argtypes = [vp, _F32P]
        L.ref_stream_buckets.restype = C.c_int
        _lib = L
    return _lib


def _rows(X, d):
    X = np.ascontiguousarray(X, dtype=np.float32)
    assert X.ndim == 2 and X.shape[1] == d
    return X


def _split_buckets(P: np.ndarray, m: int, with_values: bool):
    """Column-major (rows x C) reference bucket matrix -> ([C][2][m] ids, values)."""
    Pt = P.T  # [C][rows]
    Cn = Pt.shape[0]
    ids = np.empty((Cn, 2, m), np.int32)
    vals = np.zeros((Cn, 2, m), np.float32)
    if with_values:  # [ids close m | vals close m | ids far m | -vals far m]
        ids[:, 0] = Pt[:, 0:m].astype(np.int32)
        vals[:, 0] = Pt[:, m:2 * m]
        ids[:, 1] = Pt[:, 2 * m:3 * m].astype(np.int32)
        vals[:, 1] = Pt[:, 3 * m:4 * m]
    else:  # [ids close m | ids far m]
        ids[:, 0] = Pt[:, 0:m].astype(np.int32)
        ids[:, 1] = Pt[:, m:2 * m].astype(np.int32)
    return ids, vals


class RefCEOs:
    """The reference CEOs class (src/CEOs.h:18-114) with the parameters of
    setIndexParam (python/python_wrapper.cpp:23-30)."""

    def __init__(self, n_points: int, n_features: int):
        self._L = lib()
        self._h = self._L.ref_ceos_new(n_points, n_features)
        self.n, self.d = n_points, n_features
        self._kind = None
        self.n_probed_vectors = self.n_probed_points = self.n_cand = 10

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.ref_ceos_free(self._h)
            self._h = None

    def setIndexParam(self, n_proj, n_repeats=1, top_m=10, n_threads=-1, random_seed=-1):
        self._L.ref_ceos_set_param(self._h, n_proj, n_repeats, top_m, n_threads, random_seed)
        self.D, self.R, self.m = n_proj, n_repeats, top_m
        self.n_probed_points = top_m  # src/CEOs.h:70

    def _build(self, kind, X):
        self._L.ref_ceos_build(self._h, kind, _rows(X, self.d), self.n, self.d)
        self._kind = kind

    def build(self, X):
        self._build(KIND_DENSE, X)

    def build_coCEOs_Est(self, X):
        self._build(KIND_COCEOS, X)

    def build_CEOs_Hash(self, X):
        self._build(KIND_HASH, X)

    def _search(self, kind, Q, k):
        Q = _rows(Q, self.d)
        ids = np.zeros((Q.shape[0], k), np.int32)
        dists = np.zeros((Q.shape[0], k), np.float32)
        self._L.ref_ceos_set_query(self._h, self.n_probed_vectors, self.n_probed_points, self.n_cand)
        self._L.ref_ceos_search(self._h, kind, Q, Q.shape[0], self.d, k, ids, dists)
        return ids, dists

    def search(self, Q, k):
        return self._search(KIND_DENSE, Q, k)

    def search_coCEOs_Est(self, Q, k):
        return self._search(KIND_COCEOS, Q, k)

    def search_CEOs_Hash(self, Q, k):
        return self._search(KIND_HASH, Q, k)

    def buckets(self):
        rows = 4 * self.m if self._kind == KIND_COCEOS else 2 * self.m
        P = np.zeros((self.D * self.R, rows), np.float32)  # column-major rows x C
        got = self._L.ref_ceos_buckets(self._h, self._kind, P)
        assert got == rows
        return _split_buckets(P.T, self.m, self._kind == KIND_COCEOS)


class RefStreamCEOs:
    """The reference streamCEOs class (src/streamCEOs.h:12-107)."""

    def __init__(self, n_features: int):
        self._L = lib()
        self._h = self._L.ref_stream_new(n_features)
        self.d = n_features
        self.n_probed_vectors = self.n_probed_points = self.n_cand = 10

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.ref_stream_free(self._h)
            self._h = None

    def setIndexParam(self, n_proj, n_repeats=1, top_points=1, n_threads=-1, random_seed=-1):
        self._L.ref_stream_set_param(self._h, n_proj, n_repeats, top_points, n_threads, random_seed)
        self.D, self.R, self.m = n_proj, n_repeats, top_points
        self.n_probed_vectors = top_points  # src/streamCEOs.h:58

    @property
    def size(self) -> int:
        return self._L.ref_stream_size(self._h)

    def build(self, X):
        X = _rows(X, self.d)
        self._L.ref_stream_build(self._h, X, X.shape[0], self.d)

    def update(self, X, n_delPoints=0):
        X = _rows(X, self.d)
        self._L.ref_stream_update(self._h, X, X.shape[0], self.d, n_delPoints)

    def _search(self, kind, Q, k):
        Q = _rows(Q, self.d)
        ids = np.zeros((Q.shape[0], k), np.int32)
        dists = np.zeros((Q.shape[0], k), np.float32)
        self._L.ref_stream_set_query(self._h, self.n_probed_vectors, self.n_probed_points, self.n_cand)
        self._L.ref_stream_search(self._h, kind, Q, Q.shape[0], self.d, k, ids, dists)
        return ids, dists

    def estimate_search(self, Q, k):
        return self._search(KIND_COCEOS, Q, k)

    def hash_search(self, Q, k):
        return self._search(KIND_HASH, Q, k)

    def buckets(self):
        P = np.zeros((self.D * self.R, 4 * self.m), np.float32)
        got = self._L.ref_stream_buckets(self._h, P)
        assert got == 4 * self.m
        return _split_buckets(P.T, self.m, True)
