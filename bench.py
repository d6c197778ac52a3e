"""Benchmark of the CEOs index path on GB300.

Workload (default): plain FP32 coCEOs-Est build + search at scale,
X = 1,000,000 x 128 float32 (70% round(Gamma(0.8, 30)) clipped to [0, 255],
30% exact zeros), 10,000 queries from the same distribution, n_proj=256,
n_repeats=8, top_m=500, k=10 (seeded synthetic data with the shapes and value
distribution of the SIFT benchmark). The metric asks for queries/s at
recall@10 >= 0.9; the configured probe budget (n_probed_vectors=40,
n_cand=2000) reaches 0.64 on this data, so the headline runs at
n_probed_vectors=120, n_cand=8000 (recall 0.92) and the configured budget is
reported beside it, as are k = 1 and k = 100.

A step is one search of the 10,000-query batch. ``value`` is queries/s with
the queries already resident in HBM, timed with the library's CUDA events on
its launch stream; ``e2e`` is the same metric through the host-buffer C-ABI
call (host->device copy of the queries and device->host copy of ids and
scores inside the timed region). The L2 is flushed before every timed step.
``parity`` compares the GPU's buckets and search results at the headline and
the configured budget (k = 1, 10, 100) with the CPU oracle's on the same
index, and ``cpu_baseline`` times the natively optimised oracle build on the
host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(the path is replicated, not sharded) and rank 0 prints the aggregate.
"""
from __future__ import annotations

import argparse
import ctypes as C
import ctypes.util
import json
import os
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Index and data of the plain-FP32 at-scale configuration. The metric asks for
# queries/s at recall@10 >= 0.9: on this data the configured probe budget
# (n_probed_vectors=40, n_cand=2000) reaches recall@10 = 0.64, so the headline
# is taken at the smallest budget measured to clear 0.9 (s=120, c=8000,
# recall 0.916); the configured point is reported beside it.
CFG = dict(n=1_000_000, d=128, nq=10_000, D=256, R=8, m=500, s=120, c=8000, k=10, seed=42)
CONFIG_POINT = dict(s=40, c=2000)
WORKLOAD = "coCEOs-Est FP32 build+search, SIFT-shaped 1Mx128, 10k queries"
METRIC = "queries/s at recall@10 \u22650.9; served p50/p99 ms; build s \u2014 split-BF16 vs FP32"


def sift_like(n, d, seed, out=None):
    rng = np.random.default_rng(seed)
    out = np.empty((n, d), np.float32) if out is None else out
    step = 200_000
    for i in range(0, n, step):
        j = min(n, i + step)
        v = np.clip(np.round(rng.gamma(0.8, 30.0, (j - i, d))), 0, 255).astype(np.float32)
        v[rng.random((j - i, d)) < 0.3] = 0.0
        out[i:j] = v
    return out


# Served-queries configuration: ImageNet-shaped 2.34M x 150 index, open-loop
# Poisson request stream.
SERVE = dict(n=2_340_000, d=150, D=256, R=16, m=1000, p=1000, c=1000, seed=42,
             rate=2000.0, stream_seed=7, requests=4000, ks=(1, 10, 100), ss=(10, 20, 40, 80),
             n_slots=4, max_batch=256)


def imagenet_like(n, d, seed):
    """Rows N(0, I_d) scaled by LogNormal(0, 0.7)."""
    rng = np.random.default_rng(seed)
    out = np.empty((n, d), np.float32)
    step = 250_000
    for i in range(0, n, step):
        j = min(n, i + step)
        out[i:j] = rng.standard_normal((j - i, d), dtype=np.float32)
        out[i:j] *= rng.lognormal(0.0, 0.7, (j - i, 1)).astype(np.float32)
    return out


def request_stream(cfg, pool):
    """Open-loop Poisson arrivals (rate cfg['rate'] requests/s, seed
    cfg['stream_seed']); each request is clip(round(LogNormal(2.5, 1.0)), 1, 256)
    queries taken from `pool`, with k and n_probed_vectors drawn uniformly from
    cfg['ks'] and cfg['ss']."""
    rng = np.random.default_rng(cfg["stream_seed"])
    n = cfg["requests"]
    t = np.cumsum(rng.exponential(1.0 / cfg["rate"], n))
    sizes = np.clip(np.round(rng.lognormal(2.5, 1.0, n)), 1, 256).astype(int)
    ks = rng.choice(cfg["ks"], n)
    ss = rng.choice(cfg["ss"], n)
    offs = rng.integers(0, len(pool) - 256, n)
    return [(float(t[i]), pool[offs[i]:offs[i] + sizes[i]], int(ks[i]), int(ss[i]))
            for i in range(n)]


def run_served(idx, reqs, precision, open_loop=True):
    """Drive the serving loop with `reqs`; returns (stats, results)."""
    from ceos_gb300.serving import Server

    idx.precision = precision
    srv = Server(idx, algo="coceos", n_slots=SERVE["n_slots"], max_batch=SERVE["max_batch"],
                 max_neighbors=max(SERVE["ks"]), max_probed_vectors=max(SERVE["ss"]))
    # warm up: capture every batch-size graph of every slot
    warm = [srv.submit(reqs[i][1], reqs[i][2], reqs[i][3]) for i in range(min(64, len(reqs)))]
    for r in warm:
        srv.wait(r)
    srv.reset_stats()
    out = []
    t0 = time.perf_counter()
    for t_arr, Qr, k, s in reqs:
        if open_loop:
            while time.perf_counter() - t0 < t_arr:
                pass
        out.append(srv.submit(Qr, k, s))
    res = [srv.wait(r) for r in out]
    st = srv.stats()
    srv.close()
    return st, res


def served_leg(args):
    """Served queries (config of the request loop): build the 2.34M x 150 index,
    drive the open-loop stream through the server in FP32 and split-BF16, and at
    saturation (all requests queued at once); then the same requests through the
    plain FP32 path (one search call per request). recall@k per request against
    the GPU FP64 ground truth on a sample of requests."""
    import ceos_gb300.CEOs as CEOs
    from ceos_gb300 import _capi

    cfg = SERVE
    X = imagenet_like(cfg["n"], cfg["d"], 11)
    pool = imagenet_like(50_000, cfg["d"], 12)
    idx = CEOs.CEOs(cfg["n"], cfg["d"])
    idx.setIndexParam(cfg["D"], cfg["R"], cfg["m"], -1, cfg["seed"])
    t0 = time.perf_counter()
    idx.build_coCEOs_Est(X)
    build_s = time.perf_counter() - t0
    idx.n_probed_points, idx.n_cand = cfg["p"], cfg["c"]
    reqs = request_stream(cfg, pool)
    out = {"config": {k: v for k, v in cfg.items()}, "build_s": build_s,
           "build_phases_ms": idx.last_timings()}
    sample = reqs[:100]
    nsq = sum(len(r[1]) for r in sample)
    gtQ = np.concatenate([r[1] for r in sample])
    gt_ids, _ = _capi.bruteforce_fp64(X, gtQ, max(cfg["ks"]))
    def recall_by_probes(res):
        """recall@min(k, 10) of the sampled requests, by n_probed_vectors"""
        rec = {}
        row = 0
        for (t_arr, Qr, k, s), (ids, _) in zip(sample, res[:len(sample)]):
            kk = min(k, 10)
            g = gt_ids[row:row + len(Qr), :kk]
            row += len(Qr)
            rec.setdefault(s, []).extend(len(np.intersect1d(a[:kk], b)) / kk for a, b in zip(ids, g))
        return {str(s): float(np.mean(v)) for s, v in sorted(rec.items())}

    def sample_score_error(res):
        """largest relative error of the sampled requests' reported scores"""
        worst = 0.0
        for (t_arr, Qr, k, s), (ids, dists) in zip(sample, res[:len(sample)]):
            worst = max(worst, score_error(X, Qr, ids, dists))
        return worst

    for prec in ("fp32", "split_bf16"):
        st, res = run_served(idx, reqs, prec, open_loop=True)
        sat, _ = run_served(idx, reqs, prec, open_loop=False)
        out[prec] = {
            "open_loop": {"offered_req_per_s": cfg["rate"], "queries": st["queries"],
                          "requests": st["requests"], "wall_s": st["busy_s"],
                          "queries_per_s": st["queries"] / st["busy_s"],
                          "p50_ms": st["p50_ms"], "p90_ms": st["p90_ms"], "p99_ms": st["p99_ms"],
                          "max_ms": st["max_ms"], "mean_batch_queries": st["mean_batch_queries"],
                          "graph_launches": st["graph_launches"]},
            "saturation": {"queries_per_s": sat["queries"] / sat["busy_s"], "p50_ms": sat["p50_ms"],
                           "p99_ms": sat["p99_ms"], "mean_batch_queries": sat["mean_batch_queries"]},
            "recall_at_min_k_10_by_probes": recall_by_probes(res),
            "recall_queries": nsq,
            "max_rel_score_err": sample_score_error(res),
        }
    # the plain FP32 path: the same requests back to back, one search call each
    # (host buffers in and out, no serving loop, no request batching)
    idx.precision = "fp32"
    for t_arr, Qr, k, s in reqs[:64]:
        idx.n_probed_vectors = s
        idx.search_coCEOs_Est(Qr, k)
    lat, res = [], []
    t0 = time.perf_counter()
    for t_arr, Qr, k, s in reqs:
        t1 = time.perf_counter()
        idx.n_probed_vectors = s
        res.append(idx.search_coCEOs_Est(Qr, k))
        lat.append(time.perf_counter() - t1)
    wall = time.perf_counter() - t0
    nq = sum(len(r[1]) for r in reqs)
    out["plain_fp32"] = {"queries_per_s": nq / wall, "requests": len(reqs), "queries": nq,
                         "p50_ms": float(np.percentile(lat, 50) * 1e3),
                         "p99_ms": float(np.percentile(lat, 99) * 1e3),
                         "recall_at_min_k_10_by_probes": recall_by_probes(res),
                         "max_rel_score_err": sample_score_error(res)}
    sp, pl, fp = out["split_bf16"], out["plain_fp32"], out["fp32"]
    # the served target as stated (served split vs the plain FP32 path, one
    # search call per request) and, beside it, served split vs served FP32 at
    # the same operating points; each throughput with its own p99
    out["served_split_vs_plain_fp32_qps"] = sp["saturation"]["queries_per_s"] / pl["queries_per_s"]
    out["same_operating_point"] = {
        "saturation": {"fp32": {"queries_per_s": fp["saturation"]["queries_per_s"],
                                "p99_ms": fp["saturation"]["p99_ms"]},
                       "split_bf16": {"queries_per_s": sp["saturation"]["queries_per_s"],
                                      "p99_ms": sp["saturation"]["p99_ms"]},
                       "split_vs_fp32_qps": sp["saturation"]["queries_per_s"] / fp["saturation"]["queries_per_s"]},
        "open_loop": {"fp32": {"queries_per_s": fp["open_loop"]["queries_per_s"], "p99_ms": fp["open_loop"]["p99_ms"]},
                      "split_bf16": {"queries_per_s": sp["open_loop"]["queries_per_s"],
                                     "p99_ms": sp["open_loop"]["p99_ms"]}},
        "plain_fp32": {"queries_per_s": pl["queries_per_s"], "p99_ms": pl["p99_ms"]},
    }
    out["recall_gap_served_split_vs_plain_fp32"] = max(
        abs(sp["recall_at_min_k_10_by_probes"][s] - pl["recall_at_min_k_10_by_probes"][s])
        for s in pl["recall_at_min_k_10_by_probes"])
    return out


# Streaming configuration: 500k x 300 start index (rows g * s, g ~ N(0, I/300),
# s ~ LogNormal(0, 0.5)), then about 2M inserted rows in batches of U[1, 10000],
# 0.1% of the live ids deleted at random after every batch, and query requests
# of U[1, 128] queries between batches; exact maintenance with a reserve of
# top_m / 2 entries per list.
STREAM = dict(n0=500_000, d=300, D=1024, R=4, m=200, p=200, s=20, c=500, k=10, seed=42,
              reserve=100, insert_rows=2_000_000, max_batch_rows=10_000, delete_frac=0.001,
              query_requests_per_batch=4, max_request=128, stream_seed=7)


def netflix_like(n, d, seed):
    rng = np.random.default_rng(seed)
    out = np.empty((n, d), np.float32)
    step = 250_000
    for i in range(0, n, step):
        j = min(n, i + step)
        out[i:j] = rng.standard_normal((j - i, d), dtype=np.float32) / np.float32(np.sqrt(d))
        out[i:j] *= rng.lognormal(0.0, 0.5, (j - i, 1)).astype(np.float32)
    return out


def stream_leg(args):
    """streamCEOs at scale through the serving loop, batch by batch: insert,
    random delete, query requests; insert/delete throughput, query latency,
    recall@10 over the live rows against the GPU FP64 ground truth, and the
    final buckets compared with a fresh build on the live rows."""
    import ceos_gb300.CEOs as CEOs
    from ceos_gb300 import _capi
    from ceos_gb300.serving import Server

    cfg = STREAM
    d = cfg["d"]
    rng = np.random.default_rng(cfg["stream_seed"])
    sizes = []
    tot = 0
    while tot < cfg["insert_rows"]:
        b = int(rng.integers(1, cfg["max_batch_rows"] + 1))
        sizes.append(b)
        tot += b
    X_all = netflix_like(cfg["n0"] + tot, d, 21)
    pool = netflix_like(20_000, d, 22) * np.float32(np.sqrt(d))  # N(0, I)-scale queries
    st = CEOs.streamCEOs(d)
    st.setIndexParam(cfg["D"], cfg["R"], cfg["m"], -1, cfg["seed"])
    st.set_reserve(cfg["reserve"])
    t0 = time.perf_counter()
    st.build(X_all[:cfg["n0"]])
    build_s = time.perf_counter() - t0
    st.n_probed_vectors, st.n_probed_points, st.n_cand = cfg["s"], cfg["p"], cfg["c"]
    live = np.arange(cfg["n0"], dtype=np.int64)  # global row index of every current id
    srv = Server(st, algo="estimate", n_slots=4, max_batch=256, max_neighbors=cfg["k"],
                 max_probed_vectors=cfg["s"])
    warm = srv.submit(pool[:64], cfg["k"], cfg["s"])
    srv.wait(warm)
    srv.reset_stats()
    pos = cfg["n0"]
    t_ins = t_del = 0.0
    n_del_total = 0
    n_queries = 0
    t_start = time.perf_counter()
    for b in sizes:
        t = time.perf_counter()
        srv.wait(srv.submit_update(X_all[pos:pos + b]))
        t_ins += time.perf_counter() - t
        live = np.concatenate([live, np.arange(pos, pos + b)])
        pos += b
        nd = max(1, int(round(cfg["delete_frac"] * len(live))))
        dels = rng.choice(len(live), size=nd, replace=False).astype(np.int32)
        t = time.perf_counter()
        srv.wait(srv.submit_delete(dels))
        t_del += time.perf_counter() - t
        live = np.delete(live, dels)
        n_del_total += nd
        reqs = []
        for _ in range(cfg["query_requests_per_batch"]):
            nq = int(rng.integers(1, cfg["max_request"] + 1))
            o = int(rng.integers(0, len(pool) - nq))
            reqs.append(srv.submit(pool[o:o + nq], cfg["k"], cfg["s"]))
            n_queries += nq
        for r in reqs:
            srv.wait(r)
    wall = time.perf_counter() - t_start
    stats = srv.stats()
    # recall@10 over the live rows
    Qr = pool[:500]
    ids, dists = srv.wait(srv.submit(Qr, cfg["k"], cfg["s"]))
    srv.close()
    Xlive = X_all[live]
    gt, _ = _capi.bruteforce_fp64(Xlive, Qr, cfg["k"])
    rec = float(np.mean([len(np.intersect1d(a, g)) / cfg["k"] for a, g in zip(ids, gt)]))
    err = score_error(Xlive, Qr, ids, dists)
    # size-independent property: the maintained buckets equal a fresh build
    fresh = CEOs.CEOs(len(live), d)
    fresh.setIndexParam(cfg["D"], cfg["R"], cfg["m"], -1, cfg["seed"])
    fresh.build_coCEOs_Est(Xlive)
    fi, fv = fresh.buckets()
    si, sv = st.buckets()
    same = bool(np.array_equal(fi, si) and np.array_equal(fv.view(np.uint32), sv.view(np.uint32)))
    return {"config": dict(cfg), "batches": len(sizes), "inserted_rows": int(tot),
            "deleted_ids": int(n_del_total), "final_size": int(st.size), "build_s": build_s,
            "insert_rows_per_s": tot / t_ins, "delete_ids_per_s": n_del_total / t_del,
            "wall_s": wall, "query_requests": stats["requests"], "queries": n_queries,
            "query_p50_ms": stats["p50_ms"], "query_p99_ms": stats["p99_ms"],
            "recall@10_live": rec, "recall_queries": len(Qr), "max_rel_score_err": err,
            "buckets_equal_fresh_build": same}


# Split-precision configuration: GIST-shaped 1M x 960 index, 1000 queries.
SPLIT = dict(n=1_000_000, d=960, nq=1000, D=1024, R=8, m=1000, s=60, c=4000, k=10, seed=42)


def gist_like(n, d, seed, out=None):
    """|N(0,1)| * 0.05 with row norms scaled by LogNormal(0, 0.3)."""
    rng = np.random.default_rng(seed)
    out = np.empty((n, d), np.float32) if out is None else out
    step = 100_000
    for i in range(0, n, step):
        j = min(n, i + step)
        v = np.abs(rng.standard_normal((j - i, d), dtype=np.float32)) * np.float32(0.05)
        out[i:j] = v * rng.lognormal(0.0, 0.3, (j - i, 1)).astype(np.float32)
    return out


def split_leg(args):
    """FP32 vs split-BF16 on the 1M x 960 index: build time (device phases and
    the host copy apart), search queries/s (device time, queries resident),
    recall@10 and the largest relative error of the reported scores against
    the GPU FP64 ground truth; the oracle port's search on the host cores on a
    bounded sample of the same workload."""
    import ceos_gb300.CEOs as CEOs
    from ceos_gb300 import _capi

    cfg = SPLIT
    rt = Cudart()
    X = gist_like(cfg["n"], cfg["d"], 3, out=rt.pinned((cfg["n"], cfg["d"])))
    Q = gist_like(cfg["nq"], cfg["d"], 4)
    gt, gts = _capi.bruteforce_fp64(X, Q, cfg["k"])
    out = {"config": dict(cfg)}
    for prec in ("fp32", "split_bf16"):
        idx = CEOs.CEOs(cfg["n"], cfg["d"])
        idx.setIndexParam(cfg["D"], cfg["R"], cfg["m"], -1, cfg["seed"])
        idx.precision = prec
        builds = []
        for _ in range(2):
            t0 = time.perf_counter()
            idx.build_coCEOs_Est(X)
            builds.append((time.perf_counter() - t0, idx.last_timings()))
        idx.n_probed_vectors, idx.n_cand = cfg["s"], cfg["c"]
        ms = []
        for i in range(args.warmup + max(3, args.steps // 3)):
            ids, dists = idx.search_coCEOs_Est(Q, cfg["k"])
            t = idx.last_timings()
            if i >= args.warmup:
                ms.append(t["estimate+rerank"] + t["project"])
        rec = float(np.mean([len(np.intersect1d(a, b)) / cfg["k"] for a, b in zip(ids, gt)]))
        out[prec] = {"build_s": builds[-1][0], "build_phases_ms": builds[-1][1],
                     "build": build_split(builds[-1][1]),
                     "queries_per_s": cfg["nq"] / (float(np.mean(ms)) / 1e3),
                     "recall@10": rec, "max_rel_score_err": score_error(X, Q, ids, dists)}
        del idx
    out["split_vs_fp32_qps"] = out["split_bf16"]["queries_per_s"] / out["fp32"]["queries_per_s"]
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        qps, cpu_build_s, o = cpu_baseline_run(X, Q, 32, threads, cfg=cfg)
        out["cpu_baseline"] = {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
                               "sample": "32 queries (s=60, c=4000, k=10) on the full 1Mx960 index built by "
                                         "the natively optimised oracle port", "build_s": cpu_build_s}
        del o
    rt.free_pinned(X)
    return out


def profile_case(args, which):
    """Small cases sized for ncu captures (inputs larger than L2, a few GB on
    the device): "query-case" builds the bench index and searches 2000
    queries at the headline probe budget; "build-case" builds a 100k x 960
    GIST-shaped coCEOs index (n_proj 1024, n_repeats 8, top_m 100, which keeps
    the candidate pass rate of the 1M-row build) in FP32 and, with --split, in
    split precision. The other cases run one kernel family each on a
    SIFT-shaped index: "hash-case" CEOs-Hash (1M x 128, 2000 queries at
    s=40), "dense-case" CEOs-Est (200k x 128, its 1.6 GB projection matrix,
    500 queries), "stream-case" streamCEOs with exact maintenance (200k x 128
    start, 20k inserts, 5k random deletes, one FIFO update of a second
    stream), "bruteforce-case" the FP64 ground truth (1M x 128, 100
    queries) and "split-case" a split-precision search (GIST-shaped 200k x
    960, 500 queries)."""
    import ceos_gb300.CEOs as CEOs
    from ceos_gb300 import _capi

    if which == "hash-case":
        X = sift_like(CFG["n"], CFG["d"], 7)
        Q = sift_like(2000, CFG["d"], 8)
        idx = CEOs.CEOs(CFG["n"], CFG["d"])
        idx.setIndexParam(CFG["D"], CFG["R"], CFG["m"], -1, CFG["seed"])
        idx.build_CEOs_Hash(X)
        idx.n_probed_vectors, idx.n_cand = 40, CFG["c"]
        idx.search_CEOs_Hash(Q, CFG["k"])
        return {"case": which, "timings_ms": idx.last_timings()}
    if which == "dense-case":
        X = sift_like(200_000, CFG["d"], 7)
        Q = sift_like(500, CFG["d"], 8)
        idx = CEOs.CEOs(200_000, CFG["d"])
        idx.setIndexParam(CFG["D"], CFG["R"], CFG["m"], -1, CFG["seed"])
        idx.build(X)
        idx.n_probed_vectors, idx.n_cand = 10, 2000
        idx.search(Q, CFG["k"])
        return {"case": which, "timings_ms": idx.last_timings()}
    if which == "stream-case":
        X = sift_like(230_000, CFG["d"], 7)
        st = CEOs.streamCEOs(CFG["d"])
        st.setIndexParam(CFG["D"], CFG["R"], CFG["m"], -1, CFG["seed"])
        st.set_reserve(CFG["m"] // 2)
        st.build(X[:200_000])
        st.update(X[200_000:220_000])
        st.delete(np.random.default_rng(5).choice(220_000, 5000, replace=False).astype(np.int32))
        fifo = CEOs.streamCEOs(CFG["d"])
        fifo.setIndexParam(CFG["D"], CFG["R"], CFG["m"], -1, CFG["seed"])
        fifo.build(X[:200_000])
        fifo.update(X[220_000:230_000], 10_000)
        return {"case": which, "size": int(st.size)}
    if which == "bruteforce-case":
        X = sift_like(CFG["n"], CFG["d"], 7)
        Q = sift_like(100, CFG["d"], 8)
        _capi.bruteforce_fp64(X, Q, CFG["k"])
        return {"case": which}
    if which == "split-case":
        X = gist_like(200_000, 960, 3)
        Q = gist_like(500, 960, 4)
        idx = CEOs.CEOs(200_000, 960)
        idx.setIndexParam(1024, 8, 200, -1, 42)
        idx.precision = "split_bf16"
        idx.build_coCEOs_Est(X)
        idx.n_probed_vectors, idx.n_cand = 60, 4000
        idx.search_coCEOs_Est(Q, CFG["k"])
        return {"case": which, "timings_ms": idx.last_timings()}
    if which == "query-case":
        X = sift_like(CFG["n"], CFG["d"], 7)
        Q = sift_like(2000, CFG["d"], 8)
        idx = CEOs.CEOs(CFG["n"], CFG["d"])
        idx.setIndexParam(CFG["D"], CFG["R"], CFG["m"], -1, CFG["seed"])
        idx.build_coCEOs_Est(X)
        idx.n_probed_vectors, idx.n_cand = CFG["s"], CFG["c"]
        idx.search_coCEOs_Est(Q, CFG["k"])
    else:
        X = gist_like(100_000, 960, 3)
        idx = CEOs.CEOs(100_000, 960)
        idx.setIndexParam(1024, 8, 100, -1, 42)
        idx.precision = "split_bf16" if args.split else "fp32"
        idx.build_coCEOs_Est(X)
    return {"case": which, "timings_ms": idx.last_timings()}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        j = json.load(open(p))
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Cudart:
    """Minimal cudart access for device buffers (the product itself does not
    need it: this is only how the benchmark places its queries in HBM)."""

    def __init__(self):
        cands = ["/usr/local/cuda/lib64/libcudart.so", ctypes.util.find_library("cudart")]
        for c in cands:
            if c and (os.path.exists(c) or not c.startswith("/")):
                try:
                    self.L = C.CDLL(c)
                    break
                except OSError:
                    continue
        else:
            raise RuntimeError("libcudart not found")
        self.L.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        self.L.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        self.L.cudaFree.argtypes = [C.c_void_p]

    def malloc(self, nbytes):
        p = C.c_void_p()
        if self.L.cudaMalloc(C.byref(p), nbytes) != 0:
            raise RuntimeError("cudaMalloc failed")
        return p.value

    def h2d(self, dst, arr):
        if self.L.cudaMemcpy(C.c_void_p(dst), arr.ctypes.data, arr.nbytes, 1) != 0:
            raise RuntimeError("cudaMemcpy H2D failed")

    def d2h(self, arr, src):
        if self.L.cudaMemcpy(arr.ctypes.data, C.c_void_p(src), arr.nbytes, 2) != 0:
            raise RuntimeError("cudaMemcpy D2H failed")

    def free(self, p):
        self.L.cudaFree(C.c_void_p(p))

    def pinned(self, shape, dtype=np.float32):
        """A numpy array in page-locked host memory (cudaMallocHost), so that
        host->device copies of it run at DMA speed and do not depend on page
        residency; freed with free_pinned."""
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = C.c_void_p()
        self.L.cudaMallocHost.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        if self.L.cudaMallocHost(C.byref(p), max(nbytes, 1)) != 0:
            raise RuntimeError("cudaMallocHost failed")
        buf = (C.c_byte * nbytes).from_address(p.value)
        arr = np.frombuffer(buf, dtype=dtype).reshape(shape)
        self._pinned = getattr(self, "_pinned", {})
        self._pinned[arr.ctypes.data] = p.value
        return arr

    def free_pinned(self, arr):
        p = getattr(self, "_pinned", {}).pop(arr.ctypes.data, None)
        if p:
            self.L.cudaFreeHost.argtypes = [C.c_void_p]
            self.L.cudaFreeHost(C.c_void_p(p))


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        # raw samples (200 ms apart) go to a scratch file; the JSON line carries
        # their summary
        self.path = os.path.join(os.environ.get("CEOS_BENCH_CLOCKS_DIR", tempfile.gettempdir()),
                                 f"ceos_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=10)
        self.fh.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        # one replica per GPU: pin this rank to its GPU before the library
        # creates a CUDA context
        os.environ["CUDA_VISIBLE_DEVICES"] = os.environ.get("LOCAL_RANK", "0")
        import torch.distributed as dist

        dist.init_process_group("gloo")
        return ws, rank, dist
    return 1, 0, None


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def cpu_baseline_run(X, Q, n_queries, threads, cfg=None, s=None, c=None, k=None):
    """The reference's OpenMP path on the host cores, as the oracle source built
    the way the reference builds itself (-O3, native instruction set): build
    the index, then search a bounded sample of queries."""
    from oracle import oracle as O

    cfg = cfg or CFG
    idx = O.CEOs(*X.shape, timed=True)
    idx.setIndexParam(cfg["D"], cfg["R"], cfg["m"], threads, cfg["seed"])
    t0 = time.perf_counter()
    idx.build_coCEOs_Est(X)
    build_s = time.perf_counter() - t0
    idx.n_probed_vectors, idx.n_cand = s or cfg["s"], c or cfg["c"]
    idx.search_coCEOs_Est(Q[:min(4, n_queries)], k or cfg["k"])  # warm the threads
    t0 = time.perf_counter()
    idx.search_coCEOs_Est(Q[:n_queries], k or cfg["k"])
    dt = time.perf_counter() - t0
    return n_queries / dt, build_s, idx


def compare_with(a, b):
    """Agreement of two (ids, scores) results: fraction of queries whose ids
    are all equal, largest relative score difference over equal ids, and
    whether ids and score bits are identical."""
    ai, ad = a
    bi, bd = b
    same = ai == bi
    scale = np.maximum(np.maximum(np.abs(ad), np.abs(bd)), 1e-30).astype(np.float64)
    rel = np.where(same, np.abs(ad.astype(np.float64) - bd) / scale, 0.0)
    return {"ids_equal_frac": float(np.all(same, axis=1).mean()) if len(ai) else 1.0,
            "max_rel_score_err": float(rel.max()) if rel.size else 0.0,
            "bit_exact": bool(np.array_equal(ai, bi) and np.array_equal(ad.view(np.uint32), bd.view(np.uint32)))}


def parity_at_scale(idx, X, Q, n_queries, cfg, points, ks, threads):
    """The GPU index against the CPU oracle (the checker build, itself pinned
    to the reference's own code by the golden-fixture tests) on the same data:
    bucket ids and values, then the searches of `n_queries` queries at each
    (n_probed_vectors, n_cand) of `points` and each k of `ks`."""
    from oracle import oracle as O

    o = O.CEOs(*X.shape)
    o.setIndexParam(cfg["D"], cfg["R"], cfg["m"], threads, cfg["seed"])
    t0 = time.perf_counter()
    o.build_coCEOs_Est(X)
    ob = time.perf_counter() - t0
    gi, gv = idx.buckets()
    oi, ov = o.buckets()
    out = {"vs": "CPU oracle (checker build), pinned to the reference's own code", "queries": n_queries,
           "buckets_bit_exact": bool(np.array_equal(gi, oi) and np.array_equal(gv.view(np.uint32),
                                                                                 ov.view(np.uint32))),
           "oracle_build_s": ob, "points": []}
    del gi, gv, oi, ov
    Qp = Q[:n_queries]
    keep = idx.n_probed_vectors, idx.n_cand
    for s_, c_ in points:
        for k in ks:
            for x in (idx, o):
                x.n_probed_vectors, x.n_cand = s_, c_
            r = compare_with(idx.search_coCEOs_Est(Qp, k), o.search_coCEOs_Est(Qp, k))
            out["points"].append({"n_probed_vectors": s_, "n_cand": c_, "k": k, **r})
    idx.n_probed_vectors, idx.n_cand = keep
    out["all_bit_exact"] = out["buckets_bit_exact"] and all(p["bit_exact"] for p in out["points"])
    return out


def score_error(X, Q, ids, dists):
    """Largest relative error of reported scores against the float64 inner
    products of the reported ids (zero-filled slots excluded)."""
    exact = np.einsum("qkd,qd->qk", X[ids].astype(np.float64), Q.astype(np.float64))
    rel = np.abs(dists.astype(np.float64) - exact) / np.maximum(np.abs(exact), 1e-30)
    rel = rel[~((ids == 0) & (dists == 0))]
    return float(rel.max()) if rel.size else 0.0


def build_split(phases):
    """Device build time (every phase but the host->device copy) and the copy."""
    h2d = sum(v for k, v in phases.items() if k.startswith("h2d"))
    return {"device_ms": sum(phases.values()) - h2d, "h2d_ms": h2d}


def bench_config(ws):
    return {"workload": WORKLOAD, **CFG, "l2": "flushed (512 MiB write) before every step",
            "parallelism": "replicas" if ws > 1 else "single GPU"}


def run_reference(args, X, Q):
    ws, rank, dist = dist_setup()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    sample = args.ref_queries
    qps, build_s, idx = cpu_baseline_run(X, Q, 16, threads)
    for _ in range(args.warmup):
        idx.search_coCEOs_Est(Q[:sample], CFG["k"])
    t0 = time.perf_counter()
    for i in range(args.steps):
        off = (i * sample) % (len(Q) - sample)
        idx.search_coCEOs_Est(Q[off:off + sample], CFG["k"])
    dt = time.perf_counter() - t0
    value = args.steps * sample / dt
    line = {"impl": "reference", "metric": METRIC,
            "value": value, "unit": "queries/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(1),
            "build_s": build_s,
            "cpu_baseline": {"value": value, "unit": "queries/s", "cores": threads, "kind": "port",
                             "sample": f"{sample} queries per step on the full 1Mx128 index, searched by the "
                                       "oracle port compiled -O3 with the native instruction set, all host "
                                       "threads"},
            "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=15)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--ref-queries", type=int, default=32)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true")
    ap.add_argument("--parity-queries", type=int, default=48)
    ap.add_argument("--recall-queries", type=int, default=200)
    ap.add_argument("--split", action="store_true", help="build-case in split precision")
    ap.add_argument("--only", choices=["served", "stream", "split", "query-case", "build-case", "hash-case",
                                       "dense-case", "stream-case", "bruteforce-case", "split-case"],
                    default=None,
                    help="run one secondary leg alone and print its JSON")
    ap.add_argument("--no-legs", action="store_true",
                    help="skip the served / streaming / split-precision legs")
    args = ap.parse_args()
    os.environ.setdefault("CEOS_GB300_LOG", "0")
    if args.only:
        from ceos_gb300 import _capi

        _capi.lib().ceos_set_log_level(0)
        if args.only.endswith("-case"):
            leg = profile_case(args, args.only)
        else:
            leg = {"served": served_leg, "stream": stream_leg, "split": split_leg}[args.only](args)
        print(json.dumps({args.only: leg}))
        return 0

    if args.impl == "reference":
        X = sift_like(CFG["n"], CFG["d"], 7)
        Q = sift_like(CFG["nq"], CFG["d"], 8)
        return run_reference(args, X, Q)

    ws, rank, dist = dist_setup()
    import ceos_gb300.CEOs as CEOs
    from ceos_gb300 import _capi

    L = _capi.lib()
    L.ceos_set_log_level(0)
    if L.ceos_device_count() < 1:
        raise SystemExit("bench.py needs a CUDA device")
    rt = Cudart()
    # rows and queries in page-locked host memory, as a caller that cares about
    # copy time would hold them
    X = sift_like(CFG["n"], CFG["d"], 7, out=rt.pinned((CFG["n"], CFG["d"])))
    Q = sift_like(CFG["nq"], CFG["d"], 8, out=rt.pinned((CFG["nq"], CFG["d"])))

    idx = CEOs.CEOs(CFG["n"], CFG["d"])
    idx.setIndexParam(CFG["D"], CFG["R"], CFG["m"], -1, CFG["seed"])
    builds = []
    for _ in range(2):  # the second build runs warm
        t0 = time.perf_counter()
        idx.build_coCEOs_Est(X)
        builds.append((time.perf_counter() - t0, idx.last_timings()))
    build_s, build_phases = builds[-1]
    idx.n_probed_vectors, idx.n_cand = CFG["s"], CFG["c"]
    nq, k, d = CFG["nq"], CFG["k"], CFG["d"]
    kmax = 100

    dQ = rt.malloc(Q.nbytes)
    dI = rt.malloc(nq * kmax * 4)
    dD = rt.malloc(nq * kmax * 4)
    rt.h2d(dQ, Q)
    flush = 512 << 20

    def dev_step(kk=k):
        idx.search_device(_capi.ALGO_COCEOS, dQ, nq, kk, dI, dD)
        return idx.last_timings()

    for _ in range(args.warmup):
        dev_step()
    clocks = ClockSampler(0)
    barrier(dist)
    clocks.start()
    step_ms, kern_ms = [], []
    for _ in range(args.steps):
        _capi.check(L.ceos_flush_l2(flush))
        t = dev_step()
        step_ms.append(sum(t.values()))
        kern_ms.append(t["estimate+rerank"])
    barrier(dist)
    clk = clocks.stop()
    dev_total_s = max_over_ranks(dist, sum(step_ms) / 1e3)
    value = ws * args.steps * nq / dev_total_s

    # end to end through the host-buffer C ABI
    e2e_t = []
    for _ in range(max(1, args.warmup)):
        idx.search_coCEOs_Est(Q, k)
    for _ in range(args.steps):
        _capi.check(L.ceos_flush_l2(flush))
        t0 = time.perf_counter()
        ids, dists = idx.search_coCEOs_Est(Q, k)
        e2e_t.append(time.perf_counter() - t0)
    e2e_total = max_over_ranks(dist, sum(e2e_t))
    e2e_value = ws * args.steps * nq / e2e_total

    # device results equal host-call results
    hi = np.zeros((nq, k), np.int32)
    rt.d2h(hi, dI)
    assert np.array_equal(hi, ids), "device-resident and host-call results differ"

    # recall@k against float64 brute force on a sample of queries, and the
    # error of the reported scores
    from oracle import oracle as O

    rq = args.recall_queries
    gt, _ = O.bruteforce(X, Q[:rq], kmax, 0)

    def recall_at(found, kk):
        return float(np.mean([len(np.intersect1d(a[:kk], b[:kk])) / kk for a, b in zip(found, gt)]))

    rec = recall_at(ids[:rq], 10)
    err = score_error(X, Q[:rq], ids[:rq], dists[:rq])

    # the other k of the configuration, same probe budget
    by_k = {}
    for kk in (1, 100):
        ms = []
        for i in range(args.warmup + args.steps):
            _capi.check(L.ceos_flush_l2(flush))
            t = dev_step(kk)
            if i >= args.warmup:
                ms.append(sum(t.values()))
        ki, kd = idx.search_coCEOs_Est(Q[:rq], kk)
        by_k[str(kk)] = {"value": ws * nq * len(ms) / (sum(ms) / 1e3), "unit": "queries/s",
                         f"recall@{kk}": recall_at(ki, kk), "max_rel_score_err": score_error(X, Q[:rq], ki, kd)}

    # the configured probe budget (recall below the metric's floor)
    idx.n_probed_vectors, idx.n_cand = CONFIG_POINT["s"], CONFIG_POINT["c"]
    cp_ms = []
    for i in range(args.warmup + args.steps):
        _capi.check(L.ceos_flush_l2(flush))
        t = dev_step()
        if i >= args.warmup:
            cp_ms.append(sum(t.values()))
    cp_ids, cp_d = idx.search_coCEOs_Est(Q[:rq], k)
    cp_rec = recall_at(cp_ids, 10)
    idx.n_probed_vectors, idx.n_cand = CFG["s"], CFG["c"]

    # roofline of the dominant kernel (query estimate + rerank)
    s, p, c, m, C_ = CFG["s"], CFG["m"], CFG["c"], CFG["m"], CFG["D"] * CFG["R"]
    bytes_per_query = s * p * 8 + c * d * 4 + C_ * 4 + d * 4 + k * 8
    kern_s = float(np.mean(kern_ms)) / 1e3
    achieved = bytes_per_query * nq / kern_s / 1e9
    peak, peak_kind = load_peaks()
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        tj = json.load(open(tp))
        traffic = tj.get("query_estimate_rerank_bytes_per_launch")
        traffic_rw = {k_: tj.get(k_) for k_ in ("read_bytes_per_launch", "write_bytes_per_launch")
                      if tj.get(k_) is not None}
    else:
        traffic_rw = {}

    threads = os.cpu_count() or 1
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        qps, cpu_build_s, _ = cpu_baseline_run(X, Q, 48, threads)
        cpu = {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
               "sample": "48 queries (same probe budget) searched on the full 1Mx128 index built by "
                         "the oracle port compiled -O3 with the native instruction set",
               "build_s": cpu_build_s}
    parity = None
    if rank == 0 and not args.no_parity:
        parity = parity_at_scale(idx, X, Q, args.parity_queries, CFG,
                                 [(CFG["s"], CFG["c"]), (CONFIG_POINT["s"], CONFIG_POINT["c"])],
                                 (1, 10, 100), threads)

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value, "unit": "queries/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_total_s / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": bench_config(ws),
            "recall@10": rec, "recall_queries": rq, "max_rel_score_err": err,
            "by_k": by_k,
            "at_configured_budget": {"n_probed_vectors": CONFIG_POINT["s"], "n_cand": CONFIG_POINT["c"],
                                     "value": ws * nq * len(cp_ms) / (sum(cp_ms) / 1e3),
                                     "unit": "queries/s", "recall@10": cp_rec,
                                     "max_rel_score_err": score_error(X, Q[:rq], cp_ids, cp_d)},
            "build_s": build_s, "build_phases_ms": build_phases,
            "build": {**build_split(build_phases), "host_rows": "page-locked",
                      "first_build_s": builds[0][0]},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, **traffic_rw, "peak_kind": peak_kind,
                         "kernel": "k_query_sorted (coCEOs-Est, sorted accumulation)",
                         "bytes_per_query": bytes_per_query, "kernel_ms": kern_s * 1e3},
            "cpu_baseline": cpu,
            "parity": parity,
            "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": Q.nbytes,
                    "d2h_bytes_per_step": nq * k * 8},
            # per step: k_pad_rows (queries padded to ldx), k_project (query
            # projections), k_probe_select, k_query_sorted
            "gpu_launches": 4 * args.steps,
            "clocks": clk,
        }
    rt.free(dQ)
    rt.free(dI)
    rt.free(dD)
    del idx
    rt.free_pinned(X)
    rt.free_pinned(Q)
    if rank == 0:
        if ws == 1 and not args.no_legs:
            # the metric's other parts, each on its own configuration
            line["served"] = served_leg(args)
            line["stream"] = stream_leg(args)
            line["split"] = split_leg(args)
        print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
