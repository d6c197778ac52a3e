"""Continuous-batching request loop over a device-resident index.

The reference answers one blocking batch per call (python/python_wrapper.cpp
:36-48, :62-71); a ``Server`` keeps a built ``CEOs`` (coCEOs-Est or CEOs-Hash)
or ``streamCEOs`` index on the GPU and answers requests submitted from any
thread, each with its own ``n_neighbors`` and ``n_probed_vectors``::

    srv = Server(index, algo="coceos", n_slots=4, max_batch=256)
    req = srv.submit(Q, n_neighbors=10, n_probed_vectors=40)
    ids, dists = srv.wait(req)
    srv.stats()   # p50 / p99 latency, batches, graph replays, ...

The loop itself is native (ceos_server_* in include/ceos_gb300.h): one worker
thread packs queued requests into batches on device slots as slots free up,
replays each batch as a CUDA graph and copies results back; Python only
submits and waits. While a server exists the index's own build / update /
search calls raise RuntimeError.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi

__all__ = ["Server", "Request"]

_ALGOS = {"coceos": _capi.ALGO_COCEOS, "estimate": _capi.ALGO_COCEOS, "hash": _capi.ALGO_HASH}


class Request:
    """A submitted request: its ticket and (for queries) the output arrays the
    worker fills before the request completes."""

    __slots__ = ("ticket", "ids", "dists", "done")

    def __init__(self, ticket, ids=None, dists=None):
        self.ticket = ticket
        self.ids = ids
        self.dists = dists
        self.done = False


class Server:
    def __init__(self, index, algo: str = "coceos", n_slots: int = 4, max_batch: int = 256,
                 max_neighbors: int = 100, max_probed_vectors: int = 80,
                 mem_budget_bytes: int = 0, use_graphs: bool = True):
        L = _capi.lib()
        self._L = L
        if algo not in _ALGOS:
            raise ValueError(f"algo must be one of {sorted(_ALGOS)}")
        cfg = _capi.ServerConfig()
        _capi.check(L.ceos_server_config_init(C.byref(cfg)))
        cfg.algo = _ALGOS[algo]
        cfg.n_slots = int(n_slots)
        cfg.max_batch = int(max_batch)
        cfg.max_neighbors = int(max_neighbors)
        cfg.max_probed_vectors = int(max_probed_vectors)
        cfg.mem_budget_bytes = int(mem_budget_bytes)
        cfg.use_graphs = 1 if use_graphs else 0
        h = C.c_void_p()
        self._is_stream = hasattr(index, "update")
        fn = L.ceos_server_create_stream if self._is_stream else L.ceos_server_create
        _capi.check(fn(index._h, C.byref(cfg), C.byref(h)))
        self._h = h
        self._index = index  # the index must outlive the server
        self.n_features = index.n_features
        self._pending = {}

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.ceos_server_destroy(h)
            self._h = None
            self._pending.clear()

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, queries, n_neighbors: int, n_probed_vectors: int = 0) -> Request:
        Q = np.ascontiguousarray(queries, dtype=np.float32)
        if Q.ndim != 2 or Q.shape[1] != self.n_features:
            raise ValueError(f"queries must be a 2-D array with {self.n_features} columns")
        nq, k = Q.shape[0], int(n_neighbors)
        ids = np.zeros((nq, max(k, 0)), np.int32)
        dists = np.zeros((nq, max(k, 0)), np.float32)
        t = C.c_uint64()
        _capi.check(self._L.ceos_server_submit(self._h, Q.ctypes.data, nq, k, int(n_probed_vectors),
                                               ids.ctypes.data, dists.ctypes.data, C.byref(t)))
        req = Request(t.value, ids, dists)
        self._pending[t.value] = req
        return req

    def submit_update(self, new_dataset, n_delPoints: int = 0) -> Request:
        X = np.ascontiguousarray(new_dataset, dtype=np.float32)
        if X.ndim != 2 or X.shape[1] != self.n_features:
            raise ValueError(f"new_dataset must be a 2-D array with {self.n_features} columns")
        t = C.c_uint64()
        _capi.check(self._L.ceos_server_submit_update(self._h, X.ctypes.data if X.size else None,
                                                      X.shape[0], int(n_delPoints), C.byref(t)))
        req = Request(t.value)
        self._pending[t.value] = req
        return req

    def submit_delete(self, ids) -> Request:
        a = np.ascontiguousarray(np.asarray(ids, dtype=np.int32).ravel())
        t = C.c_uint64()
        _capi.check(self._L.ceos_server_submit_delete(self._h, a.ctypes.data if a.size else None,
                                                      a.size, C.byref(t)))
        req = Request(t.value)
        self._pending[t.value] = req
        return req

    def wait(self, req: Request, timeout: float | None = None):
        """Block until `req` completes; returns (ids, dists) for a query request."""
        ms = -1 if timeout is None else int(timeout * 1000)
        st = self._L.ceos_server_wait(self._h, req.ticket, ms)
        if st == _capi.ERR_TIMEOUT:
            _capi.check(st)
        self._pending.pop(req.ticket, None)
        req.done = True
        _capi.check(st)
        return (req.ids, req.dists) if req.ids is not None else None

    def stats(self) -> dict:
        s = _capi.ServerStats()
        _capi.check(self._L.ceos_server_get_stats(self._h, C.byref(s)))
        return {name: getattr(s, name) for name, _ in s._fields_}

    def reset_stats(self):
        _capi.check(self._L.ceos_server_reset_stats(self._h))
