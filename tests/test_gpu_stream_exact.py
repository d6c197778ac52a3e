"""streamCEOs exact maintenance and random-id deletes (a library extension:
the reference deletes only from the front and refills buckets from new points
only, src/streamCEOs.cpp:207-208, :337-352). With set_reserve(r >= 0) every
bucket must equal the exact two-ended top-m over the live rows after each
update and delete: checked against the oracle (which recomputes the buckets
from scratch), against a coCEOs index built from scratch on the live rows,
and through the serving loop."""
import numpy as np
import pytest

from conftest import gaussian_queries, netflix_like

pytestmark = pytest.mark.gpu

D, R, M, SEED = 128, 2, 40, 17


def _pair(gpu, oracle, X0, reserve):
    g = gpu.streamCEOs(X0.shape[1])
    g.setIndexParam(D, R, M, 8, SEED)
    g.set_reserve(reserve)
    g.build(X0)
    o = oracle.streamCEOs(X0.shape[1])
    o.setIndexParam(D, R, M, 8, SEED)
    o.set_reserve(reserve)
    o.build(X0)
    for s in (g, o):
        s.n_probed_vectors, s.n_probed_points, s.n_cand = 30, 25, 150
    return g, o


def _same_buckets(g, o):
    gi, gv = g.buckets()
    oi, ov = o.buckets()
    assert np.array_equal(gi, oi)
    assert np.array_equal(gv.view(np.uint32), ov.view(np.uint32))


@pytest.mark.parametrize("reserve", [0, 24])
def test_exact_maintenance_matches_oracle(gpu, oracle, reserve):
    d = 48
    pool = netflix_like(9000, d, seed=41)
    live = pool[:3000].copy()
    g, o = _pair(gpu, oracle, live, reserve)
    assert g.reserve == reserve
    rng = np.random.default_rng(3)
    pos = 3000
    Q = gaussian_queries(40, d, seed=5)
    for step in range(6):
        b = int(rng.integers(1, 700))
        new = pool[pos:pos + b]
        pos += b
        n_del = int(rng.integers(0, 200)) if step % 2 else 0
        g.update(new, n_del)
        o.update(new, n_del)
        live = np.concatenate([live[n_del:], new])
        _same_buckets(g, o)
        dels = rng.choice(len(live), size=int(rng.integers(1, 120)), replace=False)
        g.delete(dels)
        o.delete(dels)
        live = np.delete(live, dels, axis=0)
        assert g.size == o.size == len(live)
        _same_buckets(g, o)
        gi, gd = g.estimate_search(Q, 10)
        oi, od = o.estimate_search(Q, 10)
        assert np.array_equal(gi, oi) and np.array_equal(gd.view(np.uint32), od.view(np.uint32))
        gi, gd = g.hash_search(Q, 10)
        oi, od = o.hash_search(Q, 10)
        assert np.array_equal(gi, oi) and np.array_equal(gd.view(np.uint32), od.view(np.uint32))
    # the live rows are the ones the index holds: buckets equal a fresh coCEOs build
    fresh = gpu.CEOs(len(live), d)
    fresh.setIndexParam(D, R, M, 8, SEED)
    fresh.build_coCEOs_Est(live)
    fi, fv = fresh.buckets()
    gi, gv = g.buckets()
    assert np.array_equal(fi, gi) and np.array_equal(fv.view(np.uint32), gv.view(np.uint32))
    fresh.n_probed_vectors, fresh.n_probed_points, fresh.n_cand = 30, 25, 150
    a = fresh.search_coCEOs_Est(Q, 10)
    b_ = g.estimate_search(Q, 10)
    assert np.array_equal(a[0], b_[0]) and np.array_equal(a[1], b_[1])


def test_delete_errors(gpu):
    d = 16
    X = netflix_like(500, d, seed=2)
    s = gpu.streamCEOs(d)
    s.setIndexParam(32, 1, 20, 8, 1)
    s.build(X)
    with pytest.raises(ValueError, match="set_reserve"):
        s.delete([1, 2])
    with pytest.raises(ValueError, match="before build"):
        s.set_reserve(5)
    s = gpu.streamCEOs(d)
    s.setIndexParam(32, 1, 20, 8, 1)
    s.set_reserve(5)
    s.build(X)
    with pytest.raises(ValueError):
        s.delete([500])
    with pytest.raises(ValueError):
        s.delete([-1])
    with pytest.raises(ValueError, match="enough"):
        s.delete(np.arange(481))
    s.delete([3, 3, 7])  # duplicates ignored
    assert s.size == 498
    s.delete([])
    assert s.size == 498


def test_server_deletes_in_order(gpu):
    from ceos_gb300.serving import Server

    d = 32
    pool = netflix_like(6000, d, seed=8)

    def make():
        s = gpu.streamCEOs(d)
        s.setIndexParam(64, 2, 30, 8, 5)
        s.set_reserve(10)
        s.build(pool[:2500])
        s.n_probed_vectors, s.n_probed_points, s.n_cand = 16, 20, 100
        return s

    rng = np.random.default_rng(1)
    ops, pos, size = [], 2500, 2500
    for i in range(8):
        ops.append(("q", gaussian_queries(int(rng.integers(1, 40)), d, seed=70 + i)))
        b = int(rng.integers(1, 300))
        ops.append(("u", pool[pos:pos + b]))
        pos += b
        size += b
        dels = rng.choice(size, size=int(rng.integers(1, 30)), replace=False)
        ops.append(("d", dels))
        size -= len(dels)
    ref = make()
    want = []
    for kind, arg in ops:
        if kind == "q":
            want.append(ref.estimate_search(arg, 10))
        elif kind == "u":
            ref.update(arg)
        else:
            ref.delete(arg)
    s = make()
    srv = Server(s, algo="estimate", n_slots=2, max_batch=16, max_neighbors=10, max_probed_vectors=16)
    reqs = []
    for kind, arg in ops:
        if kind == "q":
            reqs.append(srv.submit(arg, 10, 16))
        elif kind == "u":
            reqs.append(srv.submit_update(arg))
        else:
            reqs.append(srv.submit_delete(arg))
    got = [r for r in (srv.wait(q) for q in reqs) if r is not None]
    srv.close()
    assert s.size == ref.size == size
    for (a, b), (c, e) in zip(want, got):
        assert np.array_equal(a, c) and np.array_equal(b.view(np.uint32), e.view(np.uint32))
