"""GPU parity at the benchmark configurations' full sizes.

* 1M x 960 GIST-shaped coCEOs-Est index (n_proj 1024, n_repeats 8,
  top_m 1000): every bucket id and value, then 32 queries at
  n_probed_vectors 60 / n_cand 4000, k = 10, bit for bit against the oracle
  (src/CEOs.cpp:311-441 build, :450-694 search).
* 500k x 300 streamCEOs start (n_proj 1024, n_repeats 4, top_m 200) under a
  sequence of FIFO updates (src/streamCEOs.cpp:174-369): buckets and both
  searches bit for bit against the oracle after every call.

The oracle is pinned to the reference's own code by tests/test_reference_pins.py.
"""
import numpy as np
import pytest

from conftest import gaussian_queries, gist_like, netflix_like

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32),
                          np.asarray(b, np.float32).view(np.uint32))


def chunked(gen, n, d, seed, step=100_000):
    """gen's distribution over n rows, drawn in chunks to bound temporaries."""
    out = np.empty((n, d), np.float32)
    for i, a in enumerate(range(0, n, step)):
        b = min(n, a + step)
        out[a:b] = gen(b - a, d, seed=seed * 1000 + i)
    return out


def test_gist_1m_x_960_parity(gpu, oracle):
    n, d = 1_000_000, 960
    X = chunked(gist_like, n, d, seed=3)
    Q = gist_like(32, d, seed=4)
    g, o = gpu.CEOs(n, d), oracle.CEOs(n, d)
    for idx in (g, o):
        idx.setIndexParam(1024, 8, 1000, -1, 42)
        idx.build_coCEOs_Est(X)
        idx.n_probed_vectors, idx.n_cand = 60, 4000
    gi, gv = g.buckets()
    oi, ov = o.buckets()
    assert np.array_equal(gi, oi)
    assert bits_equal(gv, ov)
    del gi, gv, oi, ov
    a = g.search_coCEOs_Est(Q, 10)
    b = o.search_coCEOs_Est(Q, 10)
    assert np.array_equal(a[0], b[0]) and bits_equal(a[1], b[1])


def test_stream_500k_x_300_fifo_parity(gpu, oracle):
    d = 300
    X = chunked(netflix_like, 540_000, d, seed=21)
    Q = gaussian_queries(64, d, seed=22)
    g, o = gpu.streamCEOs(d), oracle.streamCEOs(d)
    for st in (g, o):
        st.setIndexParam(1024, 4, 200, -1, 42)
        st.build(X[:500_000])
        st.n_probed_vectors, st.n_probed_points, st.n_cand = 20, 200, 500
    pos = 500_000
    for b, nd in [(10_000, 500), (1, 0), (20_000, 20_000), (9_999, 3)]:
        for st in (g, o):
            st.update(X[pos:pos + b], nd)
        pos += b
        assert g.size == o.size
        gi, gv = g.buckets()
        oi, ov = o.buckets()
        assert np.array_equal(gi, oi) and bits_equal(gv, ov), (b, nd)
        ai, ad = g.estimate_search(Q, 10)
        bi, bd = o.estimate_search(Q, 10)
        assert np.array_equal(ai, bi) and bits_equal(ad, bd), (b, nd)
        ai, ad = g.hash_search(Q, 10)
        bi, bd = o.hash_search(Q, 10)
        assert np.array_equal(ai, bi) and bits_equal(ad, bd), (b, nd)
