"""Pins against the reference itself.

The golden fixtures under tests/golden/reference_*.npz are outputs of the
reference's own CEOs / streamCEOs classes (src/CEOs.cpp, src/streamCEOs.cpp),
compiled unchanged (tests/golden/make_reference_golden.py). The same checks
run against the oracle on the CPU and against the CUDA library on the GPU:

* bucket values bit-identical, bucket ids identical up to the order inside
  runs of exactly tied values (tests/parity.py);
* search ids equal in >= 99.9% of queries (the rest only at near-ties) and
  scores within 1e-5 relative.

Where the reference library can be built (x86 with the reference sources),
the oracle is also compared with it live on further seeded cases.
"""
import os

import numpy as np
import pytest

from conftest import gaussian_queries, gist_like, netflix_like, sift_like
from golden.make_reference_golden import NETFLIX, STREAM, netflix_inputs, stream_inputs
from parity import compare_buckets, compare_results, sha256

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    return np.load(os.path.join(GOLD, name))


def _check_results(got, want, what):
    ok, stats = compare_results(got[0], got[1], want[0], want[1])
    assert ok, (what, stats)
    return stats


def _check_buckets(got, want_ids, want_vals, what, check_values=True):
    ok, reordered, msg = compare_buckets(got[0], got[1], want_ids, want_vals, check_values)
    assert ok, (what, msg)
    return reordered


def run_small(impl):
    f = _load("reference_small.npz")
    X, Q = f["X"], f["Q"]
    D, R, m, s, c, k, seed = [int(v) for v in f["params"]]
    for kind, b, srch in (("coceos", "build_coCEOs_Est", "search_coCEOs_Est"),
                          ("hash", "build_CEOs_Hash", "search_CEOs_Hash"),
                          ("dense", "build", "search")):
        idx = impl.CEOs(*X.shape)
        idx.setIndexParam(D, R, m, 4, seed)
        getattr(idx, b)(X)
        if kind == "coceos":
            _check_buckets(idx.buckets(), f["coceos_bucket_ids"], f["coceos_bucket_vals"], kind)
        elif kind == "hash":
            # CEOs-Hash keeps the same two-ended top-m ids as coCEOs-Est
            # (src/CEOs.cpp:779-831): the coCEOs values order their ties
            gi, _ = idx.buckets()
            v = f["coceos_bucket_vals"]
            _check_buckets((gi, v), f["hash_bucket_ids"], v, kind)
        idx.n_probed_vectors, idx.n_cand = s, c
        _check_results(getattr(idx, srch)(Q, k), (f[f"{kind}_ids"], f[f"{kind}_dists"]), kind)
    # integer data: exact ties in projections and scores
    D, R, m, s, c, k, seed = [int(v) for v in f["sift_params"]]
    Xs, Qs = f["sift_X"], f["sift_Q"]
    idx = impl.CEOs(*Xs.shape)
    idx.setIndexParam(D, R, m, 4, seed)
    idx.build_coCEOs_Est(Xs)
    _check_buckets(idx.buckets(), f["sift_bucket_ids"], f["sift_bucket_vals"], "sift")
    idx.n_probed_vectors, idx.n_cand = s, c
    ok, stats = compare_results(*idx.search_coCEOs_Est(Qs, k), f["sift_ids"], f["sift_dists"])
    # with integer scores a tie at the k-th place may keep another id: the
    # score lists must agree, ids may differ only inside tied scores
    assert stats["max_rel_score_err"] <= 1e-5 and not stats["other_rows"], stats
    # FIFO streamCEOs
    Xt, Qt = f["stream_X"], f["stream_Q"]
    st = impl.streamCEOs(Xt.shape[1])
    st.setIndexParam(128, 2, 40, 4, 42)
    st.build(Xt[:2000])
    st.n_probed_vectors, st.n_probed_points, st.n_cand = 20, 40, 200
    for i, (a, b, nd) in enumerate(f["stream_steps"].tolist()):
        st.update(Xt[a:b], nd)
        _check_buckets(st.buckets(), f[f"stream_{i}_bucket_ids"], f[f"stream_{i}_bucket_vals"],
                       f"stream step {i}")
        _check_results(st.estimate_search(Qt, 10), (f[f"stream_{i}_est_ids"], f[f"stream_{i}_est_dists"]),
                       f"stream estimate {i}")
        _check_results(st.hash_search(Qt, 10), (f[f"stream_{i}_hash_ids"], f[f"stream_{i}_hash_dists"]),
                       f"stream hash {i}")


def run_netflix(impl):
    """The full Netflix-shaped 17,770 x 300 workload: 17,770 x 300, 1,000 queries."""
    f = _load("reference_netflix.npz")
    X, Q = netflix_inputs()
    assert sha256(X) == str(f["x_sha256"]) and sha256(Q) == str(f["q_sha256"]), \
        "the seeded input generator differs from the one the fixture was made with"
    cols = f["columns"]
    stats = {}
    for kind, b, srch in (("coceos", "build_coCEOs_Est", "search_coCEOs_Est"),
                          ("hash", "build_CEOs_Hash", "search_CEOs_Hash"),
                          ("dense", "build", "search")):
        idx = impl.CEOs(NETFLIX["n"], NETFLIX["d"])
        idx.setIndexParam(NETFLIX["D"], NETFLIX["R"], NETFLIX["m"], 8, NETFLIX["seed"])
        getattr(idx, b)(X)
        if kind == "coceos":
            bi, bv = idx.buckets()
            assert sha256(bv) == str(f["bucket_vals_sha256"]), "bucket values differ"
            _check_buckets((bi[cols], bv[cols]), f["bucket_ids_sampled"], f["bucket_vals_sampled"], kind)
        elif kind == "hash":
            bi, _ = idx.buckets()
            v = f["bucket_vals_sampled"]
            _check_buckets((bi[cols], v), f["hash_bucket_ids_sampled"], v, kind)
        idx.n_probed_vectors, idx.n_cand = NETFLIX["s"], NETFLIX["c"]
        stats[kind] = _check_results(getattr(idx, srch)(Q, NETFLIX["k"]), (f[f"{kind}_ids"], f[f"{kind}_dists"]),
                                     kind)
    return stats


def run_stream(impl):
    """FIFO stream shaped like the streaming benchmark: 60,000 x 300 start, three updates."""
    f = _load("reference_stream.npz")
    X, Q = stream_inputs()
    assert sha256(X) == str(f["x_sha256"]) and sha256(Q) == str(f["q_sha256"]), \
        "the seeded input generator differs from the one the fixture was made with"
    cols = f["columns"]
    st = impl.streamCEOs(STREAM["d"])
    st.setIndexParam(STREAM["D"], STREAM["R"], STREAM["m"], 8, STREAM["seed"])
    st.build(X[:STREAM["n0"]])
    st.n_probed_vectors, st.n_probed_points, st.n_cand = STREAM["s"], STREAM["m"], STREAM["c"]
    a = STREAM["n0"]
    for i, (b, nd) in enumerate(STREAM["steps"]):
        st.update(X[a:a + b], nd)
        a += b
        assert st.size == int(f[f"size_{i}"])
        bi, bv = st.buckets()
        assert sha256(bv) == str(f[f"bucket_vals_sha256_{i}"]), f"bucket values differ after step {i}"
        _check_buckets((bi[cols], bv[cols]), f[f"bucket_ids_sampled_{i}"], f[f"bucket_vals_sampled_{i}"],
                       f"step {i}")
        _check_results(st.estimate_search(Q, STREAM["k"]), (f[f"est_ids_{i}"], f[f"est_dists_{i}"]),
                       f"estimate {i}")
        _check_results(st.hash_search(Q, STREAM["k"]), (f[f"hash_ids_{i}"], f[f"hash_dists_{i}"]),
                       f"hash {i}")


# ---------------------------------------------------------------------------
# oracle (CPU)

def test_oracle_matches_reference_small(oracle):
    run_small(oracle)


def test_oracle_matches_reference_netflix(oracle):
    run_netflix(oracle)


def test_oracle_matches_reference_stream(oracle):
    run_stream(oracle)


@pytest.mark.parametrize("gen,n,d,D,R,m,s,c,k,seed", [
    ("netflix", 3000, 300, 1024, 2, 100, 20, 500, 10, 42),
    ("gist", 2500, 96, 128, 3, 150, 24, 400, 10, 5),
    ("netflix", 1200, 17, 16, 3, 300, 10, 200, 5, 9),
    ("netflix", 4000, 128, 256, 2, 60, 40, 300, 100, 1),
])
def test_oracle_matches_reference_live(oracle, gen, n, d, D, R, m, s, c, k, seed):
    from oracle import reference as REF

    if not REF.available():
        pytest.skip("the reference library is built only where its sources are (x86)")
    g = {"netflix": netflix_like, "gist": gist_like, "sift": sift_like}[gen]
    X = g(n, d, seed=seed + 100)
    Q = gaussian_queries(60, d, seed=seed + 200) if gen == "netflix" else g(60, d, seed=seed + 200)
    for kind, b, srch in (("coceos", "build_coCEOs_Est", "search_coCEOs_Est"),
                          ("hash", "build_CEOs_Hash", "search_CEOs_Hash"),
                          ("dense", "build", "search")):
        r, o = REF.RefCEOs(n, d), oracle.CEOs(n, d)
        for idx in (r, o):
            idx.setIndexParam(D, R, m, 8, seed)
            getattr(idx, b)(X)
            idx.n_probed_vectors, idx.n_cand = s, c
        if kind == "coceos":
            ri, rv = r.buckets()
            _check_buckets(o.buckets(), ri, rv, kind)
            vals = rv
        elif kind == "hash":
            ri, _ = r.buckets()
            _check_buckets((o.buckets()[0], vals), ri, vals, kind)
        _check_results(getattr(o, srch)(Q, k), getattr(r, srch)(Q, k), kind)


# ---------------------------------------------------------------------------
# CUDA library (GPU)

@pytest.mark.gpu
def test_gpu_matches_reference_small(gpu):
    run_small(gpu)


@pytest.mark.gpu
def test_gpu_matches_reference_netflix(gpu):
    run_netflix(gpu)


@pytest.mark.gpu
def test_gpu_matches_reference_stream(gpu):
    run_stream(gpu)
