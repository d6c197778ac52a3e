"""Serving loop (ceos_server_*): requests of uneven size, n_neighbors and
n_probed_vectors packed into continuously refilled batches on several device
slots, replayed as CUDA graphs. The results of every request must be
bit-identical to the index's own search with the same parameters (alone), to
the same request run alone through a one-slot server, and to the oracle."""
import numpy as np
import pytest

from conftest import gaussian_queries, netflix_like

pytestmark = pytest.mark.gpu


def _requests(d, n_req, seed, max_nq=70, ks=(1, 10, 100), ss=(5, 10, 20, 40)):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_req):
        nq = int(rng.integers(1, max_nq + 1))
        out.append((gaussian_queries(nq, d, seed=1000 + i), int(rng.choice(ks)), int(rng.choice(ss))))
    return out


def _alone(idx, search, reqs):
    res = []
    for Q, k, s in reqs:
        idx.n_probed_vectors = s
        res.append(search(Q, k))
    return res


def _serve(srv, reqs):
    tickets = [srv.submit(Q, k, s) for Q, k, s in reqs]
    return [srv.wait(t) for t in tickets]


def _same(a, b):
    for (i1, d1), (i2, d2) in zip(a, b):
        assert np.array_equal(i1, i2)
        assert np.array_equal(d1.view(np.uint32), d2.view(np.uint32))


@pytest.mark.parametrize("algo,precision", [("coceos", "fp32"), ("hash", "fp32"),
                                            ("coceos", "split_bf16")])
def test_server_mix_equals_alone(gpu, oracle, algo, precision):
    from ceos_gb300.serving import Server

    n, d = 30000, 72
    X = netflix_like(n, d, seed=21)
    idx = gpu.CEOs(n, d)
    idx.setIndexParam(256, 2, 150, 8, 42)
    idx.precision = precision
    (idx.build_coCEOs_Est if algo == "coceos" else idx.build_CEOs_Hash)(X)
    idx.n_probed_points, idx.n_cand = 60, 400
    search = idx.search_coCEOs_Est if algo == "coceos" else idx.search_CEOs_Hash
    reqs = _requests(d, 40, seed=3)
    alone = _alone(idx, search, reqs)
    # several slots, batches smaller than some requests (split across slots)
    srv = Server(idx, algo=algo, n_slots=3, max_batch=64, max_neighbors=100, max_probed_vectors=40)
    mixed = _serve(srv, reqs)
    st = srv.stats()
    with pytest.raises(RuntimeError):
        search(reqs[0][0], 10)  # the index is owned by the server
    srv.close()
    _same(alone, mixed)
    assert st["requests"] == len(reqs) and st["queries"] == sum(len(r[0]) for r in reqs)
    assert st["graph_launches"] == st["batches"] >= sum(len(r[0]) for r in reqs) // 64
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    # one request at a time through a one-slot server without graphs
    srv1 = Server(idx, algo=algo, n_slots=1, max_batch=256, use_graphs=False)
    one = [srv1.wait(srv1.submit(Q, k, s)) for Q, k, s in reqs[:12]]
    assert srv1.stats()["graph_launches"] == 0
    srv1.close()
    _same(alone[:12], one)
    if precision != "fp32":
        return  # split precision builds with the tensor-core transform: no bit-exact oracle
    # the oracle, on a few requests
    o = oracle.CEOs(n, d)
    o.setIndexParam(256, 2, 150, 8, 42)
    o.precision = precision
    (o.build_coCEOs_Est if algo == "coceos" else o.build_CEOs_Hash)(X)
    o.n_probed_points, o.n_cand = 60, 400
    osearch = o.search_coCEOs_Est if algo == "coceos" else o.search_CEOs_Hash
    for (Q, k, s), (ids, dists) in list(zip(reqs, mixed))[:6]:
        o.n_probed_vectors = s
        oi, od = osearch(Q, k)
        assert np.array_equal(ids, oi)
        assert np.array_equal(dists.view(np.uint32), od.view(np.uint32))


def test_server_concurrent_submitters(gpu):
    """Requests submitted from several host threads at once."""
    import threading

    from ceos_gb300.serving import Server

    n, d = 20000, 40
    X = netflix_like(n, d, seed=5)
    idx = gpu.CEOs(n, d)
    idx.setIndexParam(128, 2, 100, 8, 7)
    idx.build_coCEOs_Est(X)
    idx.n_probed_points, idx.n_cand = 50, 300
    reqs = _requests(d, 60, seed=9, max_nq=40, ss=(10, 20))
    alone = _alone(idx, idx.search_coCEOs_Est, reqs)
    srv = Server(idx, n_slots=4, max_batch=32, max_neighbors=100, max_probed_vectors=20)
    out = [None] * len(reqs)

    def client(j):
        for i in range(j, len(reqs), 4):
            Q, k, s = reqs[i]
            out[i] = srv.wait(srv.submit(Q, k, s))

    th = [threading.Thread(target=client, args=(j,)) for j in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    srv.close()
    _same(alone, out)


def test_server_memory_budget(gpu):
    from ceos_gb300.serving import Server

    n, d = 5000, 32
    idx = gpu.CEOs(n, d)
    idx.setIndexParam(64, 2, 50, 8, 1)
    idx.build_coCEOs_Est(netflix_like(n, d, seed=1))
    idx.n_probed_points, idx.n_cand = 20, 100
    srv = Server(idx, n_slots=8, max_batch=128, max_neighbors=10, max_probed_vectors=16)
    per = srv.stats()["slot_bytes"]
    assert srv.stats()["slots"] == 8
    srv.close()
    srv = Server(idx, n_slots=8, max_batch=128, max_neighbors=10, max_probed_vectors=16,
                 mem_budget_bytes=int(per * 2.5))
    assert srv.stats()["slots"] == 2
    Q = gaussian_queries(300, d, seed=2)
    ids, dists = srv.wait(srv.submit(Q, 10, 16))  # larger than a batch: split
    srv.close()
    idx.n_probed_vectors = 16
    ri, rd = idx.search_coCEOs_Est(Q, 10)
    assert np.array_equal(ids, ri) and np.array_equal(dists, rd)
    with pytest.raises(ValueError, match="budget"):
        Server(idx, n_slots=2, max_batch=128, max_neighbors=10, max_probed_vectors=16,
               mem_budget_bytes=per // 2)
    with pytest.raises(ValueError):
        Server(idx, max_probed_vectors=129)  # > n_proj * n_repeats
    srv = Server(idx, max_neighbors=10, max_probed_vectors=16)
    with pytest.raises(ValueError):
        srv.submit(Q[:2], 11)
    with pytest.raises(ValueError):
        srv.submit(Q[:2], 5, 17)
    # an empty request completes at once
    ids, dists = srv.wait(srv.submit(Q[:0], 5))
    assert ids.shape == (0, 5)
    srv.close()


def test_stream_server_updates_in_order(gpu):
    """Queries and updates interleaved through a stream server give the same
    results as the same sequence of direct calls on an identical index."""
    from ceos_gb300.serving import Server

    d = 48
    X = netflix_like(9000, d, seed=31)

    def make():
        s = gpu.streamCEOs(d)
        s.setIndexParam(128, 2, 60, 8, 3)
        s.build(X[:5000])
        s.n_probed_vectors, s.n_probed_points, s.n_cand = 20, 30, 200
        return s

    ops = []
    rng = np.random.default_rng(4)
    pos = 5000
    for i in range(10):
        ops.append(("q", gaussian_queries(int(rng.integers(1, 50)), d, seed=50 + i), 10))
        b = int(rng.integers(1, 600))
        ops.append(("u", X[pos:pos + b], int(rng.integers(0, b))))
        pos += b
    ref = make()
    want = []
    for op in ops:
        if op[0] == "q":
            want.append(ref.estimate_search(op[1], op[2]))
        else:
            ref.update(op[1], op[2])
    s = make()
    srv = Server(s, algo="estimate", n_slots=2, max_batch=32, max_neighbors=10, max_probed_vectors=20)
    reqs = []
    for op in ops:
        reqs.append(srv.submit(op[1], op[2], 20) if op[0] == "q" else srv.submit_update(op[1], op[2]))
    got = [srv.wait(r) for r in reqs]
    st = srv.stats()
    srv.close()
    got = [g for g in got if g is not None]
    _same(want, got)
    assert st["updates"] == 10
    assert s.size == ref.size
