"""GPU parity: the CUDA library (through its C ABI) against the CPU oracle.

Bit-exact expectations (same tie rule on both sides):
  * projections (sign flips + FWHT, src/CEOs.cpp:58-88) - every bit;
  * bucket ids and values (src/CEOs.cpp:377-428);
  * search ids and scores (both compute each score in the same fixed order:
    8 strided FMA chains over float4 chunks, then a butterfly).
Estimates are accumulated in the reference's probe pop order on both sides,
so candidate sets match exactly too.
"""
import os

import numpy as np
import pytest

from conftest import gaussian_queries, gist_like, netflix_like, recall, sift_like

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def bits_equal(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32),
                          np.asarray(b, np.float32).view(np.uint32))


def build_pair(gpu, oracle, X, D, R, m, seed, kind="coceos"):
    n, d = X.shape
    g = gpu.CEOs(n, d)
    o = oracle.CEOs(n, d)
    for idx in (g, o):
        idx.setIndexParam(D, R, m, 4, seed)
        if kind == "coceos":
            idx.build_coCEOs_Est(X)
        elif kind == "hash":
            idx.build_CEOs_Hash(X)
        else:
            idx.build(X)
    return g, o


@pytest.mark.parametrize("n,d,D,R", [
    (200, 300, 1024, 2),   # the Netflix-shaped workload: F = 1024
    (300, 128, 256, 3),    # F = 256
    (257, 150, 256, 2),    # row padding (150 -> 152)
    (100, 5, 4, 2),        # F = 8
    (64, 1, 2, 1),         # F = 2
    (80, 33, 16, 2),       # n_proj < n_features: F = 64, keep 16
    (45, 700, 512, 1),     # F = 1024 from d, D < F
    (40, 2000, 512, 1),    # F = 2048
    (33, 3000, 4096, 1),   # F = 4096
    (90, 20, 32, 5),       # F = 32 (single phase)
])
def test_projection_bitexact(gpu, oracle, n, d, D, R):
    X = netflix_like(n, d, seed=n + d)
    X[3] = 0.0  # a zero row: signs of zero must match too
    g = gpu.CEOs(n, d)
    g.setIndexParam(D, R, 10, 1, 42)
    g.build(X)
    P = g.projections()
    ref = oracle.project(X, D, R, 42)
    assert bits_equal(P, ref)
    assert np.array_equal(g.sign_bits(), oracle.sign_bits(3 * R * g.fhtDim, 42))


@pytest.mark.parametrize("dist,n,d,D,R,m", [
    ("netflix", 2000, 300, 1024, 2, 100),
    ("sift", 3000, 128, 256, 4, 64),      # integer projections: exact ties
    ("gist", 1500, 96, 128, 2, 150),
    ("netflix", 500, 17, 16, 3, 500),     # top_m == n
])
def test_coceos_buckets_exact(gpu, oracle, dist, n, d, D, R, m):
    gen = {"netflix": netflix_like, "sift": sift_like, "gist": gist_like}[dist]
    X = gen(n, d, seed=11)
    g, o = build_pair(gpu, oracle, X, D, R, m, 7)
    gi, gv = g.buckets()
    oi, ov = o.buckets()
    assert np.array_equal(gi, oi)
    assert bits_equal(gv, ov)


@pytest.mark.parametrize("dist,n,d,D,R,m,s,c,k", [
    ("netflix", 2000, 300, 1024, 2, 100, 20, 500, 10),
    ("sift", 3000, 128, 256, 4, 64, 40, 300, 100),
    ("gist", 1500, 96, 128, 2, 150, 12, 200, 1),
])
def test_coceos_search_exact(gpu, oracle, dist, n, d, D, R, m, s, c, k):
    gen = {"netflix": netflix_like, "sift": sift_like, "gist": gist_like}[dist]
    X = gen(n, d, seed=12)
    Q = gen(64, d, seed=13) if dist != "netflix" else gaussian_queries(64, d, seed=13)
    g, o = build_pair(gpu, oracle, X, D, R, m, 42)
    for idx in (g, o):
        idx.n_probed_vectors, idx.n_cand = s, c
    gi, gd = g.search_coCEOs_Est(Q, k)
    oi, od = o.search_coCEOs_Est(Q, k)
    assert np.array_equal(gi, oi)
    assert bits_equal(gd, od)
    # n_probed_points below top_m
    for idx in (g, o):
        idx.n_probed_points = m // 3
    gi, gd = g.search_coCEOs_Est(Q, k)
    oi, od = o.search_coCEOs_Est(Q, k)
    assert np.array_equal(gi, oi) and bits_equal(gd, od)


def test_dense_search_exact(gpu, oracle):
    n, d = 3000, 300
    X = netflix_like(n, d, seed=21)
    Q = gaussian_queries(40, d, seed=22)
    g, o = build_pair(gpu, oracle, X, 512, 2, 10, 42, kind="dense")
    for idx in (g, o):
        idx.n_probed_vectors, idx.n_cand = 20, 300
    gi, gd = g.search(Q, 10)
    oi, od = o.search(Q, 10)
    assert np.array_equal(gi, oi) and bits_equal(gd, od)


def test_hash_search_exact(gpu, oracle):
    n, d = 2500, 128
    X = sift_like(n, d, seed=31)
    Q = sift_like(40, d, seed=32)
    g, o = build_pair(gpu, oracle, X, 256, 2, 50, 42, kind="hash")
    gi, _ = g.buckets()
    oi, _ = o.buckets()
    assert np.array_equal(gi, oi)
    for idx in (g, o):
        idx.n_probed_vectors, idx.n_probed_points = 30, 20
    ai, ad = g.search_CEOs_Hash(Q, 10)
    bi, bd = o.search_CEOs_Hash(Q, 10)
    assert np.array_equal(ai, bi) and bits_equal(ad, bd)


def test_stream_fifo_exact(gpu, oracle):
    d = 64
    X = netflix_like(6000, d, seed=41)
    Q = gaussian_queries(32, d, seed=42)
    g, o = gpu.streamCEOs(d), oracle.streamCEOs(d)
    for s in (g, o):
        s.setIndexParam(128, 2, 40, 2, 42)
        s.build(X[:2000])
        s.n_probed_vectors, s.n_probed_points, s.n_cand = 20, 40, 200
    steps = [(2000, 2500, 300), (2500, 4000, 1000), (4000, 4000, 700), (4000, 4100, 0),
             (4100, 6000, 1900)]
    for a, b, nd in steps:
        for s in (g, o):
            s.update(X[a:b], nd)
        assert g.size == o.size
        gi, gv = g.buckets()
        oi, ov = o.buckets()
        assert np.array_equal(gi, oi) and bits_equal(gv, ov)
        ai, ad = g.estimate_search(Q, 10)
        bi, bd = o.estimate_search(Q, 10)
        assert np.array_equal(ai, bi) and bits_equal(ad, bd)
        ai, ad = g.hash_search(Q, 10)
        bi, bd = o.hash_search(Q, 10)
        assert np.array_equal(ai, bi) and bits_equal(ad, bd)


def test_stream_stale_rows_quirk(gpu, oracle):
    """Deleting most points with few new ones leaves stale bucket rows
    (src/streamCEOs.cpp:331-352); both sides keep them identically."""
    d = 16
    X = netflix_like(400, d, seed=51)
    g, o = gpu.streamCEOs(d), oracle.streamCEOs(d)
    for s in (g, o):
        s.setIndexParam(32, 1, 30, 1, 3)
        s.build(X[:200])
        s.update(X[200:215], 180)   # 35 points left, survivors + new may be < 30
        s.update(X[215:230], 5)
    gi, gv = g.buckets()
    oi, ov = o.buckets()
    assert np.array_equal(gi, oi) and bits_equal(gv, ov)


def test_stream_fifo_repeated_ids_exact(gpu, oracle):
    """FIFO stale tail rows (src/streamCEOs.cpp:331-352) can repeat a live id
    inside one column; the reference adds the repeats in entry order
    (src/streamCEOs.cpp:489-526). With s*p small enough that the hash-table
    kernel would be picked, every run must equal the oracle bit for bit."""
    d = 16
    X = netflix_like(400, d, seed=51)
    Q = gaussian_queries(64, d, seed=52)
    g, o = gpu.streamCEOs(d), oracle.streamCEOs(d)
    for s in (g, o):
        s.setIndexParam(32, 1, 30, 1, 3)
        s.build(X[:200])
        s.update(X[200:215], 180)
        s.update(X[215:230], 5)
        s.n_probed_vectors, s.n_probed_points, s.n_cand = 8, 30, 40
    gi, _ = g.buckets()
    live = g.size
    # the setup must hold a column end in which a live id appears twice
    rep = 0
    for col in gi.reshape(-1, gi.shape[-1]):
        ids = col[(col >= 0) & (col < live)]
        rep += len(ids) - len(np.unique(ids))
    assert rep > 0
    bi, bd = o.estimate_search(Q, 10)
    for _ in range(10):
        ai, ad = g.estimate_search(Q, 10)
        assert np.array_equal(ai, bi) and bits_equal(ad, bd)


def test_edge_cases(gpu, oracle):
    n, d = 600, 24
    X = netflix_like(n, d, seed=61)
    X[100:140] = X[99]      # duplicated rows -> exact ties
    X[200:210] = 0.0        # zero rows
    Q = gaussian_queries(9, d, seed=62)
    g, o = build_pair(gpu, oracle, X, 32, 2, 30, 5)
    # fewer candidates than n_cand and k > candidates: zero fill
    for s_, p_, c_, k_ in [(0, 30, 10, 5), (1, 3, 100, 8), (64, 30, 10000, 40), (5, 0, 10, 3)]:
        for idx in (g, o):
            idx.n_probed_vectors, idx.n_probed_points, idx.n_cand = s_, p_, c_
        a = g.search_coCEOs_Est(Q, k_)
        b = o.search_coCEOs_Est(Q, k_)
        assert np.array_equal(a[0], b[0]) and bits_equal(a[1], b[1]), (s_, p_, c_, k_)
    ids, dists = g.search_coCEOs_Est(Q[:0], 5)
    assert ids.shape == (0, 5)
    ids, dists = g.search_coCEOs_Est(Q, 0)
    assert ids.shape == (9, 0)


def test_param_errors_gpu(gpu):
    n, d = 300, 16
    g = gpu.CEOs(n, d)
    g.setIndexParam(32, 2, 20, 1, 1)
    g.build_coCEOs_Est(netflix_like(n, d))
    g.n_probed_points = 21
    with pytest.raises(ValueError, match="probed points"):
        g.search_coCEOs_Est(gaussian_queries(2, d), 3)
    g.n_probed_points = 20
    g.n_probed_vectors = 65
    with pytest.raises(ValueError, match="probed vectors"):
        g.search_coCEOs_Est(gaussian_queries(2, d), 3)
    with pytest.raises(ValueError):
        g.setIndexParam(32, 2, 301, 1, 1)
        g.build_coCEOs_Est(netflix_like(n, d))
    s = gpu.streamCEOs(d)
    s.setIndexParam(32, 2, 20, 1, 1)
    s.build(netflix_like(100, d))
    with pytest.raises(ValueError, match="removed points"):
        s.update(netflix_like(1, d), 200)
    with pytest.raises(ValueError, match="not enough"):
        s.update(netflix_like(1, d), 90)
    s.n_probed_points = 10
    s.n_probed_vectors = 33  # stream limit is n_proj (src/streamCEOs.cpp:386-390)
    with pytest.raises(ValueError, match="probed vectors"):
        s.estimate_search(gaussian_queries(2, d), 3)


def test_sampled_thresholds_large_n(gpu, oracle):
    """n > 65536 takes the strided-sample threshold path; buckets stay exact."""
    n, d = 150000, 32
    X = sift_like(n, d, seed=71)
    g, o = build_pair(gpu, oracle, X, 64, 2, 60, 9)
    gi, gv = g.buckets()
    oi, ov = o.buckets()
    assert np.array_equal(gi, oi) and bits_equal(gv, ov)


def test_exact_fallback_on_massive_ties(gpu, oracle):
    """70% identical rows overflow the candidate lists of the columns where
    they rank at the top; those column ends go through the exact fallback."""
    n, d = 100000, 16
    rng = np.random.default_rng(81)
    X = netflix_like(n, d, seed=81)
    dup = rng.random(n) < 0.7
    X[dup] = X[0] * 3.0
    g, o = build_pair(gpu, oracle, X, 32, 1, 50, 13)
    gi, gv = g.buckets()
    oi, ov = o.buckets()
    assert np.array_equal(gi, oi) and bits_equal(gv, ov)


def test_sampled_buckets_heavy_tied_bin(gpu, oracle):
    """50 identical high-norm rows rank first in most column ends of a
    top_m = 100 build: their 50 equal values share one histogram bin above the
    selection threshold, more than the per-bin insertion sort takes, so the
    bin-ordered selection falls back to its block sort. Ties go to the
    smaller id on both sides, so the buckets stay exact."""
    n, d = 120000, 32
    X = netflix_like(n, d, seed=91)
    norms = np.linalg.norm(X, axis=1)
    X[1000:1050] = X[7] * np.float32(3.0 * norms.max() / norms[7])  # leads 65 of 256 ends
    g, o = build_pair(gpu, oracle, X, 64, 2, 100, 17)
    gi, gv = g.buckets()
    oi, ov = o.buckets()
    assert np.array_equal(gi, oi) and bits_equal(gv, ov)


def test_sampled_buckets_signed_zero_thresholds(gpu, oracle):
    """Only 30 of 70,000 rows are nonzero, so every column end's top 100 ends
    in projections of zero rows, which are +0 or -0 by the exact sign-flip and
    butterfly arithmetic (fkey ranks -0 below +0). The sample thresholds land
    on zero keys, where the float prefilter admits both zeros and the exact
    key test decides. The overflowing lists take the exact fallback, and the
    buckets match the oracle bit for bit."""
    n, d = 70000, 24
    X = np.zeros((n, d), np.float32)
    rows = np.random.default_rng(93).choice(n, 30, replace=False)
    X[rows] = netflix_like(30, d, seed=93)
    g, o = build_pair(gpu, oracle, X, 32, 2, 100, 19)
    gi, gv = g.buckets()
    oi, ov = o.buckets()
    assert np.array_equal(gi, oi) and bits_equal(gv, ov)


def test_recall_vs_fp64(gpu, oracle):
    n, d = 20000, 300
    X = netflix_like(n, d, seed=91)
    Q = gaussian_queries(100, d, seed=92)
    gt, _ = oracle.bruteforce(X, Q, 10)
    g = gpu.CEOs(n, d)
    g.setIndexParam(1024, 2, 100, 1, 42)
    g.build_coCEOs_Est(X)
    g.n_probed_vectors, g.n_cand = 20, 500
    ids, dists = g.search_coCEOs_Est(Q, 10)
    assert recall(ids, gt) > 0.85


@pytest.mark.parametrize("kind", ["coceos", "dense", "hash"])
def test_split_bf16_exact(gpu, oracle, kind):
    """Split precision: bfloat16 scan of the candidates, exact FP32 rescore of
    the best 4k. Both sides round rows to bfloat16 the same way (nearest,
    ties to even) and use the same scan order, so even the approximate scan
    agrees and the final ids and scores are bit-exact."""
    n, d = 3000, 150  # d not a multiple of 8: padded rows
    X = gist_like(n, d, seed=101)
    Q = gist_like(40, d, seed=102)
    g, o = build_pair(gpu, oracle, X, 256, 2, 60, 42, kind=kind)
    for idx in (g, o):
        idx.n_probed_vectors, idx.n_cand = 24, 300
        idx.precision = "split_bf16"
    fn = {"coceos": "search_coCEOs_Est", "dense": "search", "hash": "search_CEOs_Hash"}[kind]
    a = getattr(g, fn)(Q, 10)
    b = getattr(o, fn)(Q, 10)
    assert np.array_equal(a[0], b[0]) and bits_equal(a[1], b[1])
    # switching back to FP32 gives the plain results again
    for idx in (g, o):
        idx.precision = "fp32"
    a = getattr(g, fn)(Q, 10)
    b = getattr(o, fn)(Q, 10)
    assert np.array_equal(a[0], b[0]) and bits_equal(a[1], b[1])


def test_stream_split_bf16_exact(gpu, oracle):
    d = 40
    X = gist_like(5000, d, seed=111)
    Q = gist_like(24, d, seed=112)
    g, o = gpu.streamCEOs(d), oracle.streamCEOs(d)
    for s in (g, o):
        s.setIndexParam(64, 2, 50, 2, 42)
        s.build(X[:1000])
        s.n_probed_vectors, s.n_probed_points, s.n_cand = 16, 50, 200
        s.precision = "split_bf16"
    for a, b, nd in [(1000, 1600, 300), (1600, 4000, 1000), (4000, 5000, 2500)]:
        for s in (g, o):
            s.update(X[a:b], nd)
        ai, ad = g.estimate_search(Q, 10)
        bi, bd = o.estimate_search(Q, 10)
        assert np.array_equal(ai, bi) and bits_equal(ad, bd)
        ai, ad = g.hash_search(Q, 10)
        bi, bd = o.hash_search(Q, 10)
        assert np.array_equal(ai, bi) and bits_equal(ad, bd)


def test_split_bf16_recall_matches_fp32(gpu, oracle):
    n, d = 20000, 256
    X = gist_like(n, d, seed=121)
    Q = gist_like(100, d, seed=122)
    gt, _ = oracle.bruteforce(X, Q, 10)
    g = gpu.CEOs(n, d)
    g.setIndexParam(256, 4, 200, 1, 42)
    g.build_coCEOs_Est(X)
    g.n_probed_vectors, g.n_cand = 30, 1000
    r32 = recall(g.search_coCEOs_Est(Q, 10)[0], gt)
    g.precision = "split_bf16"
    rsp = recall(g.search_coCEOs_Est(Q, 10)[0], gt)
    assert abs(r32 - rsp) <= 0.01, (r32, rsp)


@pytest.mark.gpu
@pytest.mark.parametrize("n,d,k,kind", [(50000, 100, 10, "netflix"), (20000, 16, 100, "sift"),
                                        (1000, 33, 1, "netflix"), (50, 7, 100, "sift")])
def test_bruteforce_fp64_matches_oracle(gpu, oracle, n, d, k, kind):
    """The GPU FP64 ground truth equals the oracle's sequential double sums bit for
    bit (float products are exact in double and both add in feature order), ties
    (integer data) broken towards the smaller id, zero-filled past n."""
    from ceos_gb300 import _capi

    X = netflix_like(n, d, seed=n) if kind == "netflix" else sift_like(n, d, seed=n)
    Q = gaussian_queries(70, d, seed=3) if kind == "netflix" else sift_like(70, d, seed=4)
    gi, gs = _capi.bruteforce_fp64(X, Q, k)
    oi, os_ = oracle.bruteforce(X, Q, k)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gs.view(np.uint64), os_.view(np.uint64))


@pytest.mark.gpu
def test_netflix_workload_full_size_parity(gpu, oracle):
    """The CPU-runnable configuration at full size: 17,770 x 300 rows g*s
    (g ~ N(0, I/300), s ~ LogNormal(0, 0.5)), 1000 N(0, I) queries, n_proj 1024,
    n_repeats 2, top_m 100, n_probed_vectors 20, n_cand 500, k 10, seed 42:
    buckets and search results bit-exact against the oracle, and recall@10
    against the FP64 ground truth."""
    from ceos_gb300 import _capi

    X = netflix_like(17770, 300, seed=0)
    Q = gaussian_queries(1000, 300, seed=1)
    g, o = build_pair(gpu, oracle, X, 1024, 2, 100, 42, kind="coceos")
    gi, gv = g.buckets()
    oi, ov = o.buckets()
    assert np.array_equal(gi, oi) and bits_equal(gv, ov)
    for idx in (g, o):
        idx.n_probed_vectors, idx.n_cand = 20, 500
    a = g.search_coCEOs_Est(Q, 10)
    b = o.search_coCEOs_Est(Q, 10)
    assert np.array_equal(a[0], b[0]) and bits_equal(a[1], b[1])
    gt, _ = _capi.bruteforce_fp64(X, Q, 10)
    assert recall(a[0], gt) > 0.3


@pytest.mark.gpu
def test_hash_centering_matches_oracle(gpu, oracle):
    """Opt-in CEOs-Hash centering by the column means (the reference's branch,
    src/CEOs.cpp:721-728, subtracts an n-vector of row means from d-vectors):
    buckets and search bit-exact against the oracle, scores are q . (x - mean),
    and the index differs from the uncentered one on nonnegative data."""
    n, d = 9000, 64
    X = sift_like(n, d, seed=77)
    Q = sift_like(30, d, seed=78)
    g, o = gpu.CEOs(n, d), oracle.CEOs(n, d)
    for idx in (g, o):
        idx.setIndexParam(128, 2, 50, 4, 21)
        idx.centering = True
        idx.build_CEOs_Hash(X)
        idx.n_probed_vectors, idx.n_probed_points = 20, 30
    gi, _ = g.buckets()
    oi, _ = o.buckets()
    assert np.array_equal(gi, oi)
    a, b = g.search_CEOs_Hash(Q, 10), o.search_CEOs_Hash(Q, 10)
    assert np.array_equal(a[0], b[0]) and bits_equal(a[1], b[1])
    mu = X.astype(np.float64).mean(axis=0)
    want = np.einsum("qkd,qd->qk", X[a[0]].astype(np.float64) - mu, Q.astype(np.float64))
    np.testing.assert_allclose(a[1], want, rtol=1e-4, atol=1e-2)
    u = gpu.CEOs(n, d)
    u.setIndexParam(128, 2, 50, 4, 21)
    u.build_CEOs_Hash(X)
    assert not np.array_equal(u.buckets()[0], gi)
