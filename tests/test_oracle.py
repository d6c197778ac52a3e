"""CPU tests of the oracle against the reference's own pins.

* sign bits: known-answer vectors of std::default_random_engine (libstdc++)
  as used by the reference's bitHD3Generator (src/Utilities.cpp:21-41);
* FWHT: outputs of the reference's FFHT fht_float, compiled from the
  reference sources (tests/golden/fwht_ref.npz, and live when oracle/_ref is
  buildable on this machine);
* selection and search logic: internal consistency (heap restatement vs
  sorting) and recall sanity against float64 brute force.
"""
import json
import os

import numpy as np
import pytest

from conftest import netflix_like, gaussian_queries, recall, sift_like

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_sign_bits_kat(oracle):
    kat = json.load(open(os.path.join(GOLD, "signs_kat.json")))
    for seed, rec in kat.items():
        bits = oracle.sign_bits(rec["n_bits"], int(seed))
        assert "".join(map(str, bits.tolist())) == rec["bits"]
        assert int(bits.sum()) == rec["ones"]
    # known answers of libstdc++ default_random_engine + uniform_int_distribution(0, 1):
    # first 64 bits of seeds 42 and 7
    assert "".join(map(str, oracle.sign_bits(64, 42))) == \
        "0110001110011000000111101010000001111110000100100000110101011010"
    assert "".join(map(str, oracle.sign_bits(64, 7))) == \
        "0100110111111001101011011111110010000011110011001000111000000110"


def test_sign_bits_restatement_matches_std(oracle):
    for seed in (0, 1, 42, 2**31 - 1, 2**31, 123456789):
        s = seed if seed < 2**31 else seed - 2**32  # int argument
        if s < 0:
            continue
        a = oracle.sign_bits(20000, s)
        b = oracle.sign_bits_std(20000, s)
        assert np.array_equal(a, b), seed


def test_fwht_matches_reference_ffht_golden(oracle):
    g = np.load(os.path.join(GOLD, "fwht_ref.npz"))
    for L in range(1, 13):
        x, y = g[f"x{L}"], g[f"y{L}"]
        got = oracle.fwht(x)
        assert np.array_equal(got.view(np.uint32), y.view(np.uint32)), L


def test_fwht_matches_reference_ffht_live(oracle):
    rng = np.random.default_rng(5)
    x = rng.standard_normal((64, 1024)).astype(np.float32)
    ref = oracle.ref_ffht(x)
    if ref is None:
        pytest.skip("reference FFHT is x86 asm and is built only where its sources are present")
    assert np.array_equal(oracle.fwht(x).view(np.uint32), ref.view(np.uint32))


def _fkey(v):
    u = v.view(np.uint32).astype(np.uint64)
    return np.where(u & 0x80000000, (~u) & 0xFFFFFFFF, u | 0x80000000)


def test_bucket_selection_matches_sort(oracle):
    """The heap restatement of the two-ended top-m (src/CEOs.cpp:377-428)
    equals a stable sort by (value desc, id asc)."""
    n, d = 3000, 40
    X = sift_like(n, d, seed=3)  # integer projections: many exact ties
    D, R, m, seed = 64, 2, 37, 11
    idx = oracle.CEOs(n, d)
    idx.setIndexParam(D, R, m, 2, seed)
    idx.build_coCEOs_Est(X)
    bids, bvals = idx.buckets()
    P = oracle.project(X, D, R, seed)
    for col in range(D * R):
        v = P[:, col]
        k = _fkey(v)
        order = np.lexsort((np.arange(n), -k.astype(np.float64)))[:m]
        assert np.array_equal(bids[col, 0], order)
        assert np.array_equal(bvals[col, 0].view(np.uint32), v[order].view(np.uint32))
        kf = _fkey(-v)
        order = np.lexsort((np.arange(n), -kf.astype(np.float64)))[:m]
        assert np.array_equal(bids[col, 1], order)
        assert np.array_equal(bvals[col, 1].view(np.uint32), (-v[order]).view(np.uint32))


def test_projection_rows_independent(oracle):
    X = netflix_like(50, 30, seed=2)
    P = oracle.project(X, 32, 3, 9)
    P2 = oracle.project(X[17:18], 32, 3, 9)
    assert np.array_equal(P[17:18].view(np.uint32), P2.view(np.uint32))
    assert oracle.fht_dim(32, 30) == 32 and oracle.fht_dim(16, 30) == 32 and oracle.fht_dim(100, 30) == 128


def test_oracle_search_recall_sanity(oracle):
    n, d = 4000, 48
    X = netflix_like(n, d, seed=7)
    Q = gaussian_queries(30, d, seed=8)
    gt, _ = oracle.bruteforce(X, Q, 10)
    idx = oracle.CEOs(n, d)
    idx.setIndexParam(128, 2, 100, 4, 42)
    idx.build_coCEOs_Est(X)
    idx.n_probed_vectors, idx.n_cand = 20, 400
    ids, dists = idx.search_coCEOs_Est(Q, 10)
    assert recall(ids, gt) > 0.8
    # reported scores are the exact inner products of the reported ids
    for q in range(len(Q)):
        ref = X[ids[q]].astype(np.float64) @ Q[q].astype(np.float64)
        np.testing.assert_allclose(dists[q], ref, rtol=1e-5, atol=1e-6)
        assert np.all(np.diff(dists[q]) <= 0)


def test_oracle_param_errors(oracle):
    idx = oracle.CEOs(100, 8)
    idx.setIndexParam(16, 1, 10, 1, 1)
    idx.build_coCEOs_Est(netflix_like(100, 8))
    idx.n_probed_points = 11
    with pytest.raises(ValueError, match="probed points"):
        idx.search_coCEOs_Est(gaussian_queries(2, 8), 3)
    idx.n_probed_points = 10
    idx.n_probed_vectors = 17
    with pytest.raises(ValueError, match="probed vectors"):
        idx.search_coCEOs_Est(gaussian_queries(2, 8), 3)


def test_oracle_stream_fifo(oracle):
    d = 24
    X = netflix_like(700, d, seed=4)
    s = oracle.streamCEOs(d)
    s.setIndexParam(32, 2, 20, 2, 5)
    assert s.n_probed_vectors == 20 and s.n_probed_points == 10  # src/streamCEOs.h:58
    s.build(X[:400])
    s.update(X[400:500], 100)
    assert s.size == 400
    bids, _ = s.buckets()
    assert bids.min() >= 0 and bids.max() < 400
    with pytest.raises(ValueError):
        s.update(X[:1], 1000)


def test_bf16_rounding_nearest_even(oracle):
    rng = np.random.default_rng(9)
    x = np.concatenate([rng.standard_normal(5000).astype(np.float32) * 100,
                        np.array([1.00390625, 1.005859375, -1.00390625, 0.0, -0.0, 65504.0,
                                  3.3895314e38, 1e-40], np.float32)])
    u = x.view(np.uint32).astype(np.uint64)
    ref = (((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000) & 0xFFFFFFFF).astype(np.uint32).view(np.float32)
    got = oracle.bf16_round(x)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_oracle_exact_stream_equals_fresh_build(oracle):
    """Exact maintenance (random-delete extension): after inserts and random
    deletes the stream's buckets are the buckets of a coCEOs index built from
    scratch on the live rows."""
    d = 20
    pool = netflix_like(1500, d, seed=12)
    s = oracle.streamCEOs(d)
    s.setIndexParam(32, 2, 15, 2, 9)
    s.set_reserve(0)
    s.build(pool[:600])
    live = pool[:600]
    s.update(pool[600:900], 50)
    live = np.concatenate([live[50:], pool[600:900]])
    dels = np.array([0, 5, 6, 100, 849])
    s.delete(dels)
    live = np.delete(live, dels, axis=0)
    assert s.size == len(live)
    f = oracle.CEOs(len(live), d)
    f.setIndexParam(32, 2, 15, 2, 9)
    f.build_coCEOs_Est(live)
    a, b = s.buckets()
    c, e = f.buckets()
    assert np.array_equal(a, c) and np.array_equal(b, e)
    with pytest.raises(ValueError):
        s.delete([len(live)])
