"""The sorted coCEOs-Est accumulation kernel (k_query_sorted) against the
oracle: bit-exact ids and scores.

The library picks this kernel by itself only when the per-query hash table
would not fit shared memory twice per SM (large n_probed_vectors x
n_probed_points); CEOS_GB300_QUERY=sorted forces it here at sizes the oracle
finishes quickly. Covered:
  * the partitioned accumulation (ids below 2^20): one stable scatter by
    id >> 10, then per-warp shared-memory tables, at 1, 4, 32 and 1024
    partitions, with ids repeated across many probed buckets;
  * the LSD radix path (ids of 2^20 and above);
  * stale streamCEOs bucket rows, which both paths drop;
  * n_probed_points below top_m and k from 1 to 100.
"""
import os

import numpy as np
import pytest

from conftest import gaussian_queries, gist_like, netflix_like, sift_like

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32),
                          np.asarray(b, np.float32).view(np.uint32))


@pytest.fixture
def force_sorted():
    old = os.environ.get("CEOS_GB300_QUERY")
    os.environ["CEOS_GB300_QUERY"] = "sorted"
    yield
    if old is None:
        del os.environ["CEOS_GB300_QUERY"]
    else:
        os.environ["CEOS_GB300_QUERY"] = old


def small_rows(n, d, seed):
    """Cheap SIFT-like rows for the large-n cases (float32, nonnegative)."""
    rng = np.random.default_rng(seed)
    X = rng.gamma(0.8, 30.0, size=(n, d)).astype(np.float32)
    X[rng.random((n, d)) < 0.3] = 0.0
    return X


# (generator, n, d, n_proj, n_repeats, top_m, n_probed_vectors, n_cand, k)
CASES = [
    ("gist", 700, 96, 128, 2, 150, 12, 200, 1),         # ids < 2^10: one partition
    ("sift", 3000, 128, 256, 4, 64, 40, 300, 100),      # 4 partitions, k = 100
    ("netflix", 20000, 64, 256, 2, 200, 60, 2000, 10),  # 32 partitions
]


@pytest.mark.parametrize("dist,n,d,D,R,m,s,c,k", CASES)
def test_sorted_search_exact(gpu, oracle, force_sorted, dist, n, d, D, R, m, s, c, k):
    gen = {"netflix": netflix_like, "sift": sift_like, "gist": gist_like}[dist]
    X = gen(n, d, seed=21)
    Q = gen(48, d, seed=22) if dist != "netflix" else gaussian_queries(48, d, seed=22)
    g, o = gpu.CEOs(n, d), oracle.CEOs(n, d)
    for idx in (g, o):
        idx.setIndexParam(D, R, m, 4, 42)
        idx.build_coCEOs_Est(X)
        idx.n_probed_vectors, idx.n_cand = s, c
    gi, gd = g.search_coCEOs_Est(Q, k)
    oi, od = o.search_coCEOs_Est(Q, k)
    assert np.array_equal(gi, oi) and bits_equal(gd, od)
    for idx in (g, o):
        idx.n_probed_points = max(1, m // 3)
    gi, gd = g.search_coCEOs_Est(Q, k)
    oi, od = o.search_coCEOs_Est(Q, k)
    assert np.array_equal(gi, oi) and bits_equal(gd, od)


@pytest.mark.parametrize("n", [600_000, 1_100_000])
def test_sorted_search_exact_large_ids(gpu, oracle, force_sorted, n):
    """600k rows: ids need 20 bits, 1024 partitions of 1024 ids. 1.1M rows:
    ids need 21 bits, the LSD radix path."""
    d = 16
    X = small_rows(n, d, seed=31)
    Q = small_rows(24, d, seed=32)
    g, o = gpu.CEOs(n, d), oracle.CEOs(n, d)
    for idx in (g, o):
        idx.setIndexParam(32, 1, 400, 8, 42)
        idx.build_coCEOs_Est(X)
        idx.n_probed_vectors, idx.n_cand = 24, 3000
    gi, gd = g.search_coCEOs_Est(Q, 10)
    oi, od = o.search_coCEOs_Est(Q, 10)
    assert np.array_equal(gi, oi) and bits_equal(gd, od)


def test_sorted_repeated_ids(gpu, oracle, force_sorted):
    """Rows 0..149 have ten times the norm of the others, so they fill both
    ends of every bucket: most probed pairs fall in the first partition, and
    every one of those ids is summed over many probed buckets."""
    n, d = 20000, 48
    X = gist_like(n, d, seed=61)
    X[:150] *= 10.0
    Q = gist_like(32, d, seed=62)
    g, o = gpu.CEOs(n, d), oracle.CEOs(n, d)
    for idx in (g, o):
        idx.setIndexParam(256, 4, 100, 4, 9)
        idx.build_coCEOs_Est(X)
        idx.n_probed_vectors, idx.n_cand = 60, 120
    gi, gd = g.search_coCEOs_Est(Q, 10)
    oi, od = o.search_coCEOs_Est(Q, 10)
    assert np.array_equal(gi, oi) and bits_equal(gd, od)


def test_sorted_matches_table_path(gpu, force_sorted):
    """Both accumulation kernels give the same bits on the same index."""
    X = sift_like(5000, 64, seed=41)
    Q = sift_like(64, 64, seed=42)
    g = gpu.CEOs(5000, 64)
    g.setIndexParam(256, 2, 100, 4, 7)
    g.build_coCEOs_Est(X)
    g.n_probed_vectors, g.n_cand = 30, 600
    a = g.search_coCEOs_Est(Q, 10)
    os.environ["CEOS_GB300_QUERY"] = "table"
    b = g.search_coCEOs_Est(Q, 10)
    assert np.array_equal(a[0], b[0]) and bits_equal(a[1], b[1])


def test_sorted_stream_stale_rows(gpu, oracle, force_sorted):
    """FIFO deletes that leave stale bucket rows (src/streamCEOs.cpp:331-352):
    the sorted kernel drops the rows whose id is no longer a live point, as
    the reference's estimate does."""
    d = 16
    X = netflix_like(400, d, seed=51)
    Q = gaussian_queries(16, d, seed=52)
    g, o = gpu.streamCEOs(d), oracle.streamCEOs(d)
    for s in (g, o):
        s.setIndexParam(32, 1, 30, 1, 3)
        s.build(X[:200])
        s.update(X[200:215], 180)
        s.update(X[215:230], 5)
        s.n_probed_vectors, s.n_probed_points, s.n_cand = 20, 30, 40
    ai, ad = g.estimate_search(Q, 10)
    bi, bd = o.estimate_search(Q, 10)
    assert np.array_equal(ai, bi) and bits_equal(ad, bd)
