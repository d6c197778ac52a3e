"""Generate the golden fixtures that pin this library to the reference itself.

The reference's index classes (src/CEOs.cpp, src/streamCEOs.cpp,
src/Utilities.cpp, src/fht.c) are compiled unchanged into
oracle/_ref/libceos_ref.so by ``make -C oracle ref`` (x86, with
oracle/refshim standing in for the Eigen / Boost headers). This script runs
them on seeded synthetic inputs and writes their outputs:

* reference_small.npz  - small cases with their inputs stored: coCEOs-Est,
                         CEOs-Hash and CEOs-Est (dense) on Netflix-shaped (17,770 x 300)
                         data, coCEOs-Est on integer (SIFT-shaped) data with
                         exact ties, and a FIFO streamCEOs sequence; full
                         buckets and search results.
* reference_netflix.npz     - the full Netflix-shaped 17,770 x 300 workload (17,770 x 300, D=1024,
                         R=2, m=100, s=20, c=500, k=10, 1,000 queries, index
                         seed 42): search results of all three methods,
                         checksums of the bucket values and 64 sampled
                         columns. Inputs are regenerated from their seeds;
                         their sha256 is stored so a test can tell a changed
                         generator from a changed result.
* reference_stream.npz - a FIFO stream shaped like the streaming benchmark (rows as the Netflix-shaped workload,
                         d=300, D=1024, R=4, m=200, p=m as the reference's
                         scripts set it) with a reduced start of 60,000 rows
                         and three update calls; per step the search results
                         and bucket checksums.

Run where the reference sources are (CEOS_REFERENCE, default /root/reference):

    python tests/golden/make_reference_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from conftest import gaussian_queries, netflix_like, sift_like  # noqa: E402
from oracle import reference as REF  # noqa: E402
from parity import sha256  # noqa: E402

# Workload definitions shared with the tests that read these fixtures.
NETFLIX = dict(n=17770, d=300, nq=1000, D=1024, R=2, m=100, s=20, c=500, k=10, seed=42,
          x_seed=1770, q_seed=300)
STREAM = dict(n0=60000, d=300, nq=100, D=1024, R=4, m=200, s=20, c=500, k=10, seed=42,
              x_seed=4242, q_seed=4343, steps=((20000, 6000), (15000, 3000), (5000, 1000)))
SAMPLED_COLUMNS = 64


def netflix_inputs():
    return (netflix_like(NETFLIX["n"], NETFLIX["d"], seed=NETFLIX["x_seed"]),
            gaussian_queries(NETFLIX["nq"], NETFLIX["d"], seed=NETFLIX["q_seed"]))


def stream_inputs():
    total = STREAM["n0"] + sum(b for b, _ in STREAM["steps"])
    return (netflix_like(total, STREAM["d"], seed=STREAM["x_seed"]),
            gaussian_queries(STREAM["nq"], STREAM["d"], seed=STREAM["q_seed"]))


def sampled_columns(n_cols: int) -> np.ndarray:
    return np.linspace(0, n_cols - 1, SAMPLED_COLUMNS).astype(np.int64)


def lists_full(ids: np.ndarray, live: int) -> bool:
    """True when no column end holds a stale row: every id live and distinct
    (the reference keeps stale tail rows when survivors + new < top_m,
    src/streamCEOs.cpp:331-352)."""
    flat = ids.reshape(-1, ids.shape[-1])
    if np.any(flat < 0) or np.any(flat >= live):
        return False
    srt = np.sort(flat, axis=1)
    return not np.any(srt[:, 1:] == srt[:, :-1])


def small_cases(out):
    rng = np.random.default_rng(20240315)
    # Netflix-shaped (17,770 x 300): coCEOs-Est, CEOs-Hash, dense CEOs-Est
    n, d, nq = 900, 44, 40
    X = (rng.standard_normal((n, d)) / np.sqrt(d) * rng.lognormal(0, 0.5, (n, 1))).astype(np.float32)
    Q = rng.standard_normal((nq, d)).astype(np.float32)
    D, R, m, s, c, k, seed = 128, 2, 50, 10, 80, 10, 42
    out.update(X=X, Q=Q, params=np.array([D, R, m, s, c, k, seed], np.int32))
    for kind, b, srch in (("coceos", "build_coCEOs_Est", "search_coCEOs_Est"),
                          ("hash", "build_CEOs_Hash", "search_CEOs_Hash"),
                          ("dense", "build", "search")):
        r = REF.RefCEOs(n, d)
        r.setIndexParam(D, R, m, 4, seed)
        getattr(r, b)(X)
        r.n_probed_vectors, r.n_cand = s, c
        ids, dists = getattr(r, srch)(Q, k)
        out[f"{kind}_ids"], out[f"{kind}_dists"] = ids, dists
        if kind != "dense":
            bi, bv = r.buckets()
            out[f"{kind}_bucket_ids"] = bi
            if kind == "coceos":
                out["coceos_bucket_vals"] = bv
    # integer data with exact ties
    n, d, nq = 1500, 24, 30
    Xs = sift_like(n, d, seed=77)
    Qs = sift_like(nq, d, seed=78)
    r = REF.RefCEOs(n, d)
    r.setIndexParam(64, 2, 40, 4, 7)
    r.build_coCEOs_Est(Xs)
    r.n_probed_vectors, r.n_cand = 12, 150
    out["sift_X"], out["sift_Q"] = Xs, Qs
    out["sift_params"] = np.array([64, 2, 40, 12, 150, 10, 7], np.int32)
    out["sift_ids"], out["sift_dists"] = r.search_coCEOs_Est(Qs, 10)
    out["sift_bucket_ids"], out["sift_bucket_vals"] = r.buckets()
    # FIFO stream with its inputs stored
    d = 32
    Xt = netflix_like(5200, d, seed=91)
    Qt = gaussian_queries(32, d, seed=92)
    st = REF.RefStreamCEOs(d)
    st.setIndexParam(128, 2, 40, 4, 42)
    st.build(Xt[:2000])
    st.n_probed_vectors, st.n_probed_points, st.n_cand = 20, 40, 200
    out["stream_X"], out["stream_Q"] = Xt, Qt
    steps = [(2000, 3000, 300), (3000, 4500, 600), (4500, 5200, 200)]
    out["stream_steps"] = np.array(steps, np.int32)
    for i, (a, b, nd) in enumerate(steps):
        st.update(Xt[a:b], nd)
        bi, bv = st.buckets()
        assert lists_full(bi, st.size), f"stale rows after small stream step {i}"
        out[f"stream_{i}_bucket_ids"], out[f"stream_{i}_bucket_vals"] = bi, bv
        out[f"stream_{i}_est_ids"], out[f"stream_{i}_est_dists"] = st.estimate_search(Qt, 10)
        out[f"stream_{i}_hash_ids"], out[f"stream_{i}_hash_dists"] = st.hash_search(Qt, 10)


def netflix_case(out):
    X, Q = netflix_inputs()
    out["x_sha256"], out["q_sha256"] = np.array(sha256(X)), np.array(sha256(Q))
    cols = sampled_columns(NETFLIX["D"] * NETFLIX["R"])
    out["columns"] = cols
    for kind, b, srch in (("coceos", "build_coCEOs_Est", "search_coCEOs_Est"),
                          ("hash", "build_CEOs_Hash", "search_CEOs_Hash"),
                          ("dense", "build", "search")):
        r = REF.RefCEOs(NETFLIX["n"], NETFLIX["d"])
        r.setIndexParam(NETFLIX["D"], NETFLIX["R"], NETFLIX["m"], 8, NETFLIX["seed"])
        getattr(r, b)(X)
        r.n_probed_vectors, r.n_cand = NETFLIX["s"], NETFLIX["c"]
        out[f"{kind}_ids"], out[f"{kind}_dists"] = getattr(r, srch)(Q, NETFLIX["k"])
        if kind == "coceos":
            bi, bv = r.buckets()
            out["bucket_vals_sha256"] = np.array(sha256(bv))
            out["bucket_ids_sampled"], out["bucket_vals_sampled"] = bi[cols], bv[cols]
        elif kind == "hash":
            bi, _ = r.buckets()
            out["hash_bucket_ids_sampled"] = bi[cols]


def stream_case(out):
    X, Q = stream_inputs()
    out["x_sha256"], out["q_sha256"] = np.array(sha256(X)), np.array(sha256(Q))
    st = REF.RefStreamCEOs(STREAM["d"])
    st.setIndexParam(STREAM["D"], STREAM["R"], STREAM["m"], 8, STREAM["seed"])
    st.build(X[:STREAM["n0"]])
    st.n_probed_vectors, st.n_probed_points, st.n_cand = STREAM["s"], STREAM["m"], STREAM["c"]
    cols = sampled_columns(STREAM["D"] * STREAM["R"])
    out["columns"] = cols
    a = STREAM["n0"]
    for i, (b, nd) in enumerate(STREAM["steps"]):
        st.update(X[a:a + b], nd)
        a += b
        bi, bv = st.buckets()
        assert lists_full(bi, st.size), f"stale rows after stream step {i}"
        out[f"size_{i}"] = np.array(st.size)
        out[f"bucket_vals_sha256_{i}"] = np.array(sha256(bv))
        out[f"bucket_ids_sampled_{i}"], out[f"bucket_vals_sampled_{i}"] = bi[cols], bv[cols]
        out[f"est_ids_{i}"], out[f"est_dists_{i}"] = st.estimate_search(Q, STREAM["k"])
        out[f"hash_ids_{i}"], out[f"hash_dists_{i}"] = st.hash_search(Q, STREAM["k"])


def main():
    if not REF.available():
        raise SystemExit("the reference library could not be built here")
    for name, fn in (("reference_small.npz", small_cases), ("reference_netflix.npz", netflix_case),
                     ("reference_stream.npz", stream_case)):
        out = {}
        fn(out)
        np.savez_compressed(os.path.join(HERE, name), **out)
        print("wrote", name)


if __name__ == "__main__":
    main()
