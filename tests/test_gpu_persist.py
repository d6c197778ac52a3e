"""Index save / load (a library extension; the reference rebuilds every
index). A loaded index must search, and for streams keep updating, exactly
like the one that was saved; truncated, corrupt or mismatched files are
rejected."""
import numpy as np
import pytest

from conftest import gaussian_queries, netflix_like

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["coceos", "hash", "dense"])
def test_save_load_index(gpu, tmp_path, kind):
    n, d = 5000, 100
    X = netflix_like(n, d, seed=3)
    Q = gaussian_queries(30, d, seed=4)
    g = gpu.CEOs(n, d)
    g.setIndexParam(128, 2, 60, 8, 11)
    build = {"coceos": g.build_coCEOs_Est, "hash": g.build_CEOs_Hash, "dense": g.build}[kind]
    build(X)
    g.n_probed_vectors, g.n_probed_points, g.n_cand = 12, 40, 300
    search = {"coceos": "search_coCEOs_Est", "hash": "search_CEOs_Hash", "dense": "search"}[kind]
    want = getattr(g, search)(Q, 10)
    path = tmp_path / "index.ceos"
    g.save(str(path))
    h = gpu.CEOs.load(str(path))
    assert (h.n_points, h.n_features) == (n, d)
    assert (h.n_probed_vectors, h.n_probed_points, h.n_cand) == (12, 40, 300)
    got = getattr(h, search)(Q, 10)
    assert np.array_equal(want[0], got[0]) and np.array_equal(want[1], got[1])
    if kind != "dense":
        a, b = g.buckets(), h.buckets()
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    # corrupt and truncated files are rejected
    raw = bytearray(path.read_bytes())
    bad = tmp_path / "bad.ceos"
    raw[len(raw) // 2] ^= 0xFF
    bad.write_bytes(bytes(raw))
    with pytest.raises(ValueError, match="corrupt"):
        gpu.CEOs.load(str(bad))
    bad.write_bytes(bytes(raw[: len(raw) // 3]))
    with pytest.raises(ValueError):
        gpu.CEOs.load(str(bad))
    with pytest.raises(ValueError):
        gpu.streamCEOs.load(str(path))  # a CEOs file is not a stream file


def test_save_load_stream_keeps_updating(gpu, tmp_path):
    d = 40
    pool = netflix_like(8000, d, seed=9)
    s = gpu.streamCEOs(d)
    s.setIndexParam(64, 2, 30, 8, 5)
    s.set_reserve(10)
    s.build(pool[:3000])
    s.n_probed_vectors, s.n_probed_points, s.n_cand = 16, 20, 100
    s.update(pool[3000:3500], 100)
    s.delete([0, 7, 1234])
    path = tmp_path / "stream.ceos"
    s.save(str(path))
    t = gpu.streamCEOs.load(str(path))
    assert t.size == s.size and t.reserve == 10
    Q = gaussian_queries(20, d, seed=1)
    for x in (s, t):
        x.update(pool[3500:4200], 50)
        x.delete([5, 99, 2000])
    a, b = s.estimate_search(Q, 10), t.estimate_search(Q, 10)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    a, b = s.buckets(), t.buckets()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_save_unbuilt_and_missing(gpu, tmp_path):
    g = gpu.CEOs(100, 8)
    with pytest.raises(RuntimeError):
        g.save(str(tmp_path / "x.ceos"))
    with pytest.raises(ValueError):
        gpu.CEOs.load(str(tmp_path / "missing.ceos"))


@pytest.mark.parametrize("kind", ["coceos", "hash", "dense"])
def test_build_from_file_equals_build(gpu, tmp_path, kind):
    """Rows streamed from a raw float32 file (the reference's loadbinData format,
    here 21 rows more than n_points and d = 50, not a multiple of 8) give the
    same index as the in-memory build."""
    n, d = 7000, 50
    X = netflix_like(n + 21, d, seed=12)
    path = tmp_path / "rows.bin"
    X.tofile(str(path))
    Q = gaussian_queries(25, d, seed=13)
    a, b = gpu.CEOs(n, d), gpu.CEOs(n, d)
    for g in (a, b):
        g.setIndexParam(64, 2, 40, 8, 3)
        g.n_probed_vectors, g.n_probed_points, g.n_cand = 10, 30, 200
    {"coceos": a.build_coCEOs_Est, "hash": a.build_CEOs_Hash, "dense": a.build}[kind](X[:n])
    b.build_from_file(str(path), kind)
    search = {"coceos": "search_coCEOs_Est", "hash": "search_CEOs_Hash", "dense": "search"}[kind]
    ra, rb = getattr(a, search)(Q, 10), getattr(b, search)(Q, 10)
    assert np.array_equal(ra[0], rb[0]) and np.array_equal(ra[1], rb[1])
    big = gpu.CEOs(n + 22, d)
    big.setIndexParam(64, 2, 40, 8, 3)
    with pytest.raises(ValueError, match="exceeds"):
        big.build_from_file(str(path), kind)
    s, t = gpu.streamCEOs(d), gpu.streamCEOs(d)
    for x in (s, t):
        x.setIndexParam(64, 2, 40, 8, 3)
    s.build(X[:n])
    t.build_from_file(str(path), n)
    assert np.array_equal(s.buckets()[0], t.buckets()[0])
