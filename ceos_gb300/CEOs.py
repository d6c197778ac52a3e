"""Drop-in Python module for the CEOs index path, on one GB300 GPU.

Mirrors the reference's pybind11 module ``CEOs`` (python/python_wrapper.cpp
:13-74): the classes, constructor arguments, ``setIndexParam`` keywords and
defaults, read/write attributes and method names are the same, so

    import ceos_gb300.CEOs as CEOs
    index = CEOs.CEOs(n, d)
    index.setIndexParam(D, n_repeats, top_m, n_threads, seed)
    index.build_coCEOs_Est(X)
    index.n_probed_vectors, index.n_cand = 40, 2000
    ids, dists = index.search_coCEOs_Est(Q, 10)

works unchanged. The work runs in the CUDA library through the C ABI of
include/ceos_gb300.h; there is no CPU fallback. Differences, all deliberate:
invalid parameters raise ValueError instead of printing and calling exit(1);
ties between exactly equal values are broken towards the smaller id.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _capi

__all__ = ["CEOs", "streamCEOs"]


def _rows(a, n_features: int, what: str) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] != n_features:
        raise ValueError(f"{what} must be a 2-D array with {n_features} columns, got shape {a.shape}")
    return a


class _QueryAttrs:
    """n_probed_vectors / n_probed_points / n_cand read-write attributes
    (python/python_wrapper.cpp:32-34, :59-61)."""

    _get = None
    _set = None

    def _q(self):
        s, p, c = C.c_int(), C.c_int(), C.c_int()
        _capi.check(self._get(self._h, C.byref(s), C.byref(p), C.byref(c)))
        return s.value, p.value, c.value

    @property
    def n_probed_vectors(self) -> int:
        return self._q()[0]

    @n_probed_vectors.setter
    def n_probed_vectors(self, v):
        s, p, c = self._q()
        _capi.check(self._set(self._h, int(v), p, c))

    @property
    def n_probed_points(self) -> int:
        return self._q()[1]

    @n_probed_points.setter
    def n_probed_points(self, v):
        s, p, c = self._q()
        _capi.check(self._set(self._h, s, int(v), c))

    @property
    def n_cand(self) -> int:
        return self._q()[2]

    @n_cand.setter
    def n_cand(self, v):
        s, p, c = self._q()
        _capi.check(self._set(self._h, s, p, int(v)))


class CEOs(_QueryAttrs):
    """CEOs(n_points, n_features): src/CEOs.h:18-114."""

    def __init__(self, n_points: int, n_features: int):
        L = _capi.lib()
        self._L = L
        h = C.c_void_p()
        _capi.check(L.ceos_create(int(n_points), int(n_features), C.byref(h)))
        self._h = h
        self._get = L.ceos_get_query_param
        self._set = L.ceos_set_query_param
        self.n_points = int(n_points)
        self.n_features = int(n_features)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.ceos_destroy(h)
            self._h = None

    def build_from_file(self, path, algo="coceos"):
        """Build from a raw row-major float32 file of n_points x n_features values (the
        reference's loadbinData format, src/Utilities.cpp:142-214), streamed to the GPU.
        algo: "dense" (build), "coceos" (build_coCEOs_Est) or "hash" (build_CEOs_Hash)."""
        code = {"dense": _capi.ALGO_DENSE, "coceos": _capi.ALGO_COCEOS, "hash": _capi.ALGO_HASH}[algo]
        _capi.check(self._L.ceos_build_from_file(self._h, os.fsencode(path), code))

    # -- save / load (no reference counterpart) --------------------------
    def save(self, path):
        """Write the built index to `path` (versioned binary file with checksum)."""
        _capi.check(self._L.ceos_save(self._h, os.fsencode(path)))

    @classmethod
    def load(cls, path):
        """A device-resident index restored from `path`, ready to search."""
        L = _capi.lib()
        h = C.c_void_p()
        _capi.check(L.ceos_load(os.fsencode(path), C.byref(h)))
        self = cls.__new__(cls)
        self._L, self._h = L, h
        self._get, self._set = L.ceos_get_query_param, L.ceos_set_query_param
        n, d = C.c_int(), C.c_int()
        _capi.check(L.ceos_get_shape(h, C.byref(n), C.byref(d)))
        self.n_points, self.n_features = n.value, d.value
        p = C.c_int()
        _capi.check(L.ceos_get_precision(h, C.byref(p)))
        self._precision = "split_bf16" if p.value == _capi.PRECISION_SPLIT_BF16 else "fp32"
        return self

    # -- parameters -----------------------------------------------------
    def setIndexParam(self, n_proj, n_repeats=1, top_m=10, n_threads=-1, random_seed=-1):
        _capi.check(self._L.ceos_set_index_param(self._h, int(n_proj), int(n_repeats), int(top_m),
                                                 int(n_threads), int(random_seed)))

    def _index_param(self):
        v = [C.c_int() for _ in range(6)]
        _capi.check(self._L.ceos_get_index_param(self._h, *[C.byref(x) for x in v]))
        return [x.value for x in v]

    @property
    def n_proj(self):
        return self._index_param()[0]

    @property
    def n_repeats(self):
        return self._index_param()[1]

    @property
    def top_m(self):
        return self._index_param()[2]

    @property
    def fhtDim(self):
        return self._index_param()[5]

    def set_threads(self, n_threads):
        _capi.check(self._L.ceos_set_threads(self._h, int(n_threads)))

    def clear(self):
        _capi.check(self._L.ceos_clear(self._h))

    @property
    def centering(self) -> bool:
        v = C.c_int()
        _capi.check(self._L.ceos_get_centering(self._h, C.byref(v)))
        return bool(v.value)

    @centering.setter
    def centering(self, v):
        _capi.check(self._L.ceos_set_centering(self._h, 1 if v else 0))

    @property
    def precision(self) -> str:
        return self._precision if hasattr(self, "_precision") else "fp32"

    @precision.setter
    def precision(self, v: str):
        code = {"fp32": _capi.PRECISION_FP32, "split_bf16": _capi.PRECISION_SPLIT_BF16}.get(v)
        if code is None:
            raise ValueError("precision must be 'fp32' or 'split_bf16'")
        _capi.check(self._L.ceos_set_precision(self._h, code))
        self._precision = v

    # -- build / search ---------------------------------------------------
    def _build(self, fn, dataset):
        X = _rows(dataset, self.n_features, "dataset")
        if X.shape[0] != self.n_points:
            raise ValueError(f"dataset has {X.shape[0]} rows, the index was created for {self.n_points}")
        _capi.check(fn(self._h, X))

    def _search(self, fn, queries, n_neighbors, verbose):
        Q = _rows(queries, self.n_features, "queries")
        k = int(n_neighbors)
        if k < 0:
            raise ValueError("n_neighbors must be >= 0")
        ids = np.zeros((Q.shape[0], k), np.int32)
        dists = np.zeros((Q.shape[0], k), np.float32)
        _capi.check(fn(self._h, Q, Q.shape[0], k, 1 if verbose else 0, ids, dists))
        return ids, dists

    def build(self, dataset):
        """CEOs-Est build (src/CEOs.cpp:18-98)."""
        self._build(self._L.ceos_build, dataset)

    def search(self, queries, n_neighbors, verbose=False):
        """CEOs-Est search (src/CEOs.cpp:107-297)."""
        return self._search(self._L.ceos_search, queries, n_neighbors, verbose)

    def build_coCEOs_Est(self, dataset):
        """coCEOs-Est build (src/CEOs.cpp:311-441)."""
        self._build(self._L.ceos_build_coceos_est, dataset)

    def search_coCEOs_Est(self, queries, n_neighbors, verbose=False):
        """coCEOs-Est search (src/CEOs.cpp:450-694)."""
        return self._search(self._L.ceos_search_coceos_est, queries, n_neighbors, verbose)

    def build_CEOs_Hash(self, dataset):
        """CEOs-Hash build (src/CEOs.cpp:708-840)."""
        self._build(self._L.ceos_build_ceos_hash, dataset)

    def search_CEOs_Hash(self, queries, n_neighbors, verbose=False):
        """CEOs-Hash search (src/CEOs.cpp:850-1066)."""
        return self._search(self._L.ceos_search_ceos_hash, queries, n_neighbors, verbose)

    # -- extensions (no reference counterpart) ----------------------------
    def search_device(self, algo: int, d_queries: int, n_queries: int, n_neighbors: int,
                      d_ids: int, d_dists: int, stream: int = 0):
        """Search with queries and results already in device memory
        (raw CUDA pointers as ints)."""
        _capi.check(self._L.ceos_search_device(self._h, int(algo), C.c_void_p(d_queries),
                                               int(n_queries), int(n_neighbors), C.c_void_p(d_ids),
                                               C.c_void_p(d_dists), C.c_void_p(stream or None)))

    def buckets(self):
        """(ids, values) of a coCEOs-Est / CEOs-Hash index as [n_proj*n_repeats][2][top_m]."""
        D, R, m = self._index_param()[:3]
        ids = np.zeros((D * R, 2, m), np.int32)
        vals = np.zeros((D * R, 2, m), np.float32)
        _capi.check(self._L.ceos_get_buckets(self._h, ids, vals))
        return ids, vals

    def projections(self):
        """Dense CEOs-Est projections, n_points x (n_proj*n_repeats)."""
        D, R = self._index_param()[:2]
        P = np.zeros((self.n_points, D * R), np.float32)
        _capi.check(self._L.ceos_get_projections(self._h, P))
        return P

    def sign_bits(self):
        D, R, _, _, _, F = self._index_param()
        b = np.zeros(3 * R * F, np.uint8)
        _capi.check(self._L.ceos_get_sign_bits(self._h, b))
        return b

    def last_timings(self) -> dict:
        """Per-phase device time (ms) of the last build or search."""
        buf = np.zeros(32, np.float32)
        n = self._L.ceos_last_timings(self._h, buf, 32)
        return {self._L.ceos_timing_name(self._h, i).decode(): float(buf[i]) for i in range(n)}


class streamCEOs(_QueryAttrs):
    """streamCEOs(n_features): src/streamCEOs.h:12-107."""

    def __init__(self, n_features: int):
        L = _capi.lib()
        self._L = L
        h = C.c_void_p()
        _capi.check(L.ceos_stream_create(int(n_features), C.byref(h)))
        self._h = h
        self._get = L.ceos_stream_get_query_param
        self._set = L.ceos_stream_set_query_param
        self.n_features = int(n_features)
        self._D, self._R, self._m = 256, 1, 100

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.ceos_stream_destroy(h)
            self._h = None

    def setIndexParam(self, n_proj, n_repeats=1, top_points=1, n_threads=-1, random_seed=-1):
        _capi.check(self._L.ceos_stream_set_index_param(self._h, int(n_proj), int(n_repeats),
                                                        int(top_points), int(n_threads),
                                                        int(random_seed)))
        self._D, self._R, self._m = int(n_proj), int(n_repeats), int(top_points)

    def set_threads(self, n_threads):
        _capi.check(self._L.ceos_stream_set_threads(self._h, int(n_threads)))

    @property
    def precision(self) -> str:
        return getattr(self, "_precision", "fp32")

    @precision.setter
    def precision(self, v: str):
        code = {"fp32": _capi.PRECISION_FP32, "split_bf16": _capi.PRECISION_SPLIT_BF16}.get(v)
        if code is None:
            raise ValueError("precision must be 'fp32' or 'split_bf16'")
        _capi.check(self._L.ceos_stream_set_precision(self._h, code))
        self._precision = v

    def clear(self):
        _capi.check(self._L.ceos_stream_clear(self._h))

    @property
    def size(self) -> int:
        n = C.c_int()
        _capi.check(self._L.ceos_stream_size(self._h, C.byref(n)))
        return n.value

    def build(self, dataset):
        """src/streamCEOs.cpp:9-161"""
        X = _rows(dataset, self.n_features, "dataset")
        _capi.check(self._L.ceos_stream_build(self._h, X, X.shape[0]))

    def update(self, new_dataset, n_delPoints=0):
        """src/streamCEOs.cpp:174-369: append new rows, drop n_delPoints from the front."""
        X = np.ascontiguousarray(new_dataset, dtype=np.float32)
        if X.size == 0:
            X = X.reshape(0, self.n_features)
        X = _rows(X, self.n_features, "new_dataset")
        ptr = X.ctypes.data if X.shape[0] else None
        _capi.check(self._L.ceos_stream_update(self._h, C.c_void_p(ptr), X.shape[0], int(n_delPoints)))

    def build_from_file(self, path, n_points):
        """build() from the first n_points rows of a raw row-major float32 file."""
        _capi.check(self._L.ceos_stream_build_from_file(self._h, os.fsencode(path), int(n_points)))

    def save(self, path):
        """Write the built stream index to `path` (versioned binary file with checksum)."""
        _capi.check(self._L.ceos_stream_save(self._h, os.fsencode(path)))

    @classmethod
    def load(cls, path):
        """A device-resident stream index restored from `path`."""
        L = _capi.lib()
        h = C.c_void_p()
        _capi.check(L.ceos_stream_load(os.fsencode(path), C.byref(h)))
        self = cls.__new__(cls)
        self._L, self._h = L, h
        self._get, self._set = L.ceos_stream_get_query_param, L.ceos_stream_set_query_param
        v = [C.c_int() for _ in range(5)]
        _capi.check(L.ceos_stream_get_index_param(h, *[C.byref(x) for x in v]))
        self._D, self._R, self._m = v[0].value, v[1].value, v[2].value
        self.n_features = v[4].value
        p = C.c_int()
        _capi.check(L.ceos_stream_get_precision(h, C.byref(p)))
        self._precision = "split_bf16" if p.value == _capi.PRECISION_SPLIT_BF16 else "fp32"
        return self

    def set_reserve(self, reserve: int):
        """Exact maintenance (no reference counterpart): with reserve >= 0, set before
        build, each column end keeps top_points + reserve entries and every bucket is
        the exact top-m over the live points after each update and delete; -1 keeps
        the reference's maintenance (src/streamCEOs.cpp:262-358)."""
        _capi.check(self._L.ceos_stream_set_reserve(self._h, int(reserve)))

    @property
    def reserve(self) -> int:
        r = C.c_int()
        _capi.check(self._L.ceos_stream_get_reserve(self._h, C.byref(r)))
        return r.value

    def delete(self, ids):
        """Delete points by current id (0 .. size-1); later ids move down, as
        erasing from the reference's deque would. Needs set_reserve before build."""
        a = np.ascontiguousarray(np.asarray(ids, dtype=np.int32).ravel())
        _capi.check(self._L.ceos_stream_delete(self._h, a.ctypes.data if a.size else None, a.size))

    def _search(self, fn, queries, n_neighbors, verbose):
        Q = _rows(queries, self.n_features, "queries")
        k = int(n_neighbors)
        if k < 0:
            raise ValueError("n_neighbors must be >= 0")
        ids = np.zeros((Q.shape[0], k), np.int32)
        dists = np.zeros((Q.shape[0], k), np.float32)
        _capi.check(fn(self._h, Q, Q.shape[0], k, 1 if verbose else 0, ids, dists))
        return ids, dists

    def estimate_search(self, queries, n_neighbors, verbose=False):
        """src/streamCEOs.cpp:378-612"""
        return self._search(self._L.ceos_stream_estimate_search, queries, n_neighbors, verbose)

    def hash_search(self, queries, n_neighbors, verbose=False):
        """src/streamCEOs.cpp:621-877"""
        return self._search(self._L.ceos_stream_hash_search, queries, n_neighbors, verbose)

    def buckets(self):
        ids = np.zeros((self._D * self._R, 2, self._m), np.int32)
        vals = np.zeros((self._D * self._R, 2, self._m), np.float32)
        _capi.check(self._L.ceos_stream_get_buckets(self._h, ids, vals))
        return ids, vals
