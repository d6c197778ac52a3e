"""The allocation-free coCEOs-Est search, ceos_search_coceos_est_device_noalloc.

It exists for callers that cannot let this library call cudaMalloc: a host
process that owns all device memory through its own arena (a database or
search engine that loads the index as a plugin), or a latency-critical
serving loop where an allocation could stall the device or fail in the middle
of a request. Its scratch comes from one fixed device array instead.

Checked through the C ABI against the allocating device search
(ceos_search_device), on two calls in a row - the second call finds the
array holding the first call's contents - for a query table that fits in
shared memory, for one that lives in the scratch array, and for a
split-precision index (bfloat16 scan, FP32 rescore); a batch larger than the
array is refused, and so is a split-precision index whose bfloat16 row copy
does not exist yet. This file is collected last on purpose.
"""
import ctypes as C
import ctypes.util
import os

import numpy as np
import pytest

from conftest import gaussian_queries, netflix_like

pytestmark = pytest.mark.gpu


class _Cudart:
    def __init__(self):
        for cand in ("/usr/local/cuda/lib64/libcudart.so", ctypes.util.find_library("cudart")):
            if cand and (not cand.startswith("/") or os.path.exists(cand)):
                self.L = C.CDLL(cand)
                break
        self.L.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        self.L.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        self.L.cudaFree.argtypes = [C.c_void_p]
        self.bufs = []

    def alloc(self, nbytes):
        p = C.c_void_p()
        assert self.L.cudaMalloc(C.byref(p), nbytes) == 0
        self.bufs.append(p.value)
        return p.value

    def put(self, arr):
        p = self.alloc(arr.nbytes)
        assert self.L.cudaMemcpy(C.c_void_p(p), arr.ctypes.data, arr.nbytes, 1) == 0
        return p

    def get(self, p, shape, dtype):
        out = np.zeros(shape, dtype)
        assert self.L.cudaMemcpy(out.ctypes.data, C.c_void_p(p), out.nbytes, 2) == 0
        return out

    def sync(self):
        assert self.L.cudaDeviceSynchronize() == 0

    def free_all(self):
        for p in self.bufs:
            self.L.cudaFree(C.c_void_p(p))
        self.bufs = []


@pytest.mark.parametrize("n,d,D,R,m,s,c,k", [
    (5000, 300, 1024, 2, 100, 20, 500, 10),   # hash table in shared memory
    (6000, 64, 256, 1, 1000, 60, 3000, 25),   # 60,000 probed pairs: tables in the scratch array
])
def test_noalloc_matches_allocating_search(gpu, n, d, D, R, m, s, c, k):
    from ceos_gb300 import _capi

    L = _capi.lib()
    X = netflix_like(n, d, seed=n)
    Q = gaussian_queries(48, d, seed=d)
    nq = Q.shape[0]
    idx = gpu.CEOs(n, d)
    idx.setIndexParam(D, R, m, 1, 42)
    idx.build_coCEOs_Est(X)
    idx.n_probed_vectors, idx.n_cand = s, c
    rt = _Cudart()
    try:
        dQ = rt.put(Q)
        dI, dD = rt.alloc(nq * k * 4), rt.alloc(nq * k * 4)
        dI2, dD2 = rt.alloc(nq * k * 4), rt.alloc(nq * k * 4)
        _capi.check(L.ceos_search_device(idx._h, _capi.ALGO_COCEOS, C.c_void_p(dQ), nq, k,
                                         C.c_void_p(dI), C.c_void_p(dD), None))
        ref_i = rt.get(dI, (nq, k), np.int32)
        ref_d = rt.get(dD, (nq, k), np.float32)
        for _ in range(2):
            _capi.check(L.ceos_search_coceos_est_device_noalloc(
                idx._h, C.c_void_p(dQ), nq, k, C.c_void_p(dI2), C.c_void_p(dD2), None))
            rt.sync()
            got_i = rt.get(dI2, (nq, k), np.int32)
            got_d = rt.get(dD2, (nq, k), np.float32)
            assert np.array_equal(got_i, ref_i)
            assert np.array_equal(got_d.view(np.uint32), ref_d.view(np.uint32))
    finally:
        rt.free_all()


def test_noalloc_rejects_oversized_batch(gpu):
    from ceos_gb300 import _capi

    L = _capi.lib()
    n, d = 3000, 128
    idx = gpu.CEOs(n, d)
    idx.setIndexParam(256, 8, 50, 1, 1)
    idx.build_coCEOs_Est(netflix_like(n, d, seed=5))
    # 9,000 queries need 9000 * (128 + 2048) * 4 bytes > 64 MiB of scratch
    nq, k = 9000, 10
    rt = _Cudart()
    try:
        dQ = rt.put(np.zeros((nq, d), np.float32))
        dI, dD = rt.alloc(nq * k * 4), rt.alloc(nq * k * 4)
        st = L.ceos_search_coceos_est_device_noalloc(idx._h, C.c_void_p(dQ), nq, k, C.c_void_p(dI),
                                                     C.c_void_p(dD), None)
        assert st == _capi.ERR_UNSUPPORTED
        assert "scratch" in _capi.last_error()
        # a batch within the limit on the same index still works afterwards
        _capi.check(L.ceos_search_coceos_est_device_noalloc(idx._h, C.c_void_p(dQ), 100, k,
                                                            C.c_void_p(dI), C.c_void_p(dD), None))
        rt.sync()
    finally:
        rt.free_all()


def test_noalloc_split_precision(gpu):
    """On a split-precision index the allocation-free search scans the bfloat16
    row copy and rescores the best 4k in FP32, like ceos_search_device. The copy
    is made by the first allocating split search; before that the entry point
    refuses rather than allocate it or fall back to a plain FP32 rerank."""
    from ceos_gb300 import _capi

    L = _capi.lib()
    n, d, k = 6000, 256, 10
    X = netflix_like(n, d, seed=11)
    Q = gaussian_queries(40, d, seed=12)
    nq = Q.shape[0]
    idx = gpu.CEOs(n, d)
    idx.setIndexParam(256, 2, 100, 1, 42)
    idx.precision = "split_bf16"
    idx.build_coCEOs_Est(X)
    idx.n_probed_vectors, idx.n_cand = 20, 500
    rt = _Cudart()
    try:
        dQ = rt.put(Q)
        dI, dD = rt.alloc(nq * k * 4), rt.alloc(nq * k * 4)
        dI2, dD2 = rt.alloc(nq * k * 4), rt.alloc(nq * k * 4)
        st = L.ceos_search_coceos_est_device_noalloc(idx._h, C.c_void_p(dQ), nq, k,
                                                     C.c_void_p(dI2), C.c_void_p(dD2), None)
        assert st == _capi.ERR_UNSUPPORTED
        assert "bfloat16" in _capi.last_error()
        _capi.check(L.ceos_search_device(idx._h, _capi.ALGO_COCEOS, C.c_void_p(dQ), nq, k,
                                         C.c_void_p(dI), C.c_void_p(dD), None))
        ref_i = rt.get(dI, (nq, k), np.int32)
        ref_d = rt.get(dD, (nq, k), np.float32)
        for _ in range(2):
            _capi.check(L.ceos_search_coceos_est_device_noalloc(
                idx._h, C.c_void_p(dQ), nq, k, C.c_void_p(dI2), C.c_void_p(dD2), None))
            rt.sync()
            got_i = rt.get(dI2, (nq, k), np.int32)
            got_d = rt.get(dD2, (nq, k), np.float32)
            assert np.array_equal(got_i, ref_i)
            assert np.array_equal(got_d.view(np.uint32), ref_d.view(np.uint32))
    finally:
        rt.free_all()
