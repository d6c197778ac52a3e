"""The benchmark's synthetic workloads stand in for the reference's datasets and
request stream: shapes, value distributions and request parameters must be the
configured ones. Checked on small samples of each generator, without a GPU."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def log_norm_std(X):
    return float(np.std(np.log(np.linalg.norm(X.astype(np.float64), axis=1))))


def test_sift_like_integer_gamma_with_zeros():
    """1M x 128 config: 70% round(Gamma(0.8, 30)) clipped to [0, 255], 30% zeros."""
    X = bench.sift_like(20000, 128, 7)
    assert X.dtype == np.float32 and X.shape == (20000, 128)
    assert np.array_equal(X, np.round(X)) and X.min() >= 0 and X.max() <= 255
    # the planted 30% plus the Gamma draws that round to 0 (about 4% of the rest)
    assert 0.31 < float(np.mean(X == 0)) < 0.35
    nz = X[X > 0]
    assert 22.0 < float(nz.mean()) < 28.0


def test_gist_like_abs_normal_lognormal_norms():
    """1M x 960 config: |N(0,1)| * 0.05 with row norms scaled by LogNormal(0, 0.3)."""
    X = bench.gist_like(4000, 960, 3)
    assert X.dtype == np.float32 and X.min() >= 0
    assert 0.27 < log_norm_std(X) < 0.33
    # median row norm: 0.05 * sqrt(960) (a row of |N(0,1)| has norm ~ sqrt(d))
    assert abs(float(np.median(np.linalg.norm(X, axis=1))) / (0.05 * np.sqrt(960)) - 1) < 0.05


def test_imagenet_like_normal_lognormal_norms():
    """2.34M x 150 served config: N(0, I) scaled by LogNormal(0, 0.7)."""
    X = bench.imagenet_like(6000, 150, 11)
    assert X.dtype == np.float32
    assert abs(float(X.mean())) < 0.02
    assert 0.65 < log_norm_std(X) < 0.75


def test_netflix_like_row_scales():
    """Streaming config: rows g * s, g ~ N(0, I/300), s ~ LogNormal(0, 0.5)."""
    X = bench.netflix_like(6000, 300, 5)
    assert X.dtype == np.float32
    assert 0.46 < log_norm_std(X) < 0.54
    assert abs(float(np.median(np.linalg.norm(X, axis=1))) - 1.0) < 0.05


def test_request_stream_matches_served_config():
    """Poisson arrivals at 2000 requests/s (seed 7); request sizes
    clip(round(LogNormal(2.5, 1.0)), 1, 256); k from {1, 10, 100} and
    n_probed_vectors from {10, 20, 40, 80}; deterministic."""
    cfg = bench.SERVE
    pool = np.arange(2 * 50_000, dtype=np.float32).reshape(50_000, 2)
    reqs = bench.request_stream(cfg, pool)
    again = bench.request_stream(cfg, pool)
    assert len(reqs) == cfg["requests"] == 4000
    t = np.array([r[0] for r in reqs])
    assert np.all(np.diff(t) > 0)
    assert abs(t[-1] - cfg["requests"] / cfg["rate"]) < 0.1  # about 2 s of arrivals
    sizes = np.array([len(r[1]) for r in reqs])
    assert sizes.min() >= 1 and sizes.max() <= 256
    assert 10 <= np.median(sizes) <= 14  # median of LogNormal(2.5, 1) is e^2.5 = 12.2
    assert {r[2] for r in reqs} == set(cfg["ks"]) == {1, 10, 100}
    assert {r[3] for r in reqs} == set(cfg["ss"]) == {10, 20, 40, 80}
    assert all(a[0] == b[0] and np.array_equal(a[1], b[1]) and a[2:] == b[2:]
               for a, b in zip(reqs, again))
