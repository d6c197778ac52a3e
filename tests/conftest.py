import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

os.environ.setdefault("CEOS_GB300_LOG", "0")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA (GB300) device")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.lib()
    return O


@pytest.fixture(scope="session")
def ceos():
    import ceos_gb300.CEOs as CEOs
    from ceos_gb300 import _capi

    _capi.lib().ceos_set_log_level(0)
    return CEOs


def has_gpu() -> bool:
    try:
        from ceos_gb300 import _capi

        return _capi.lib().ceos_device_count() > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu(ceos):
    if not has_gpu():
        pytest.fail("GPU test run without a visible CUDA device")
    return ceos


# ---------------------------------------------------------------------------
# Synthetic data with the shapes and distributions of the benchmark configs.

def netflix_like(n, d, seed=0):
    """Rows g_i * s_i, g_i ~ N(0, I/d), s_i ~ LogNormal(0, 0.5)."""
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((n, d)).astype(np.float32) / np.float32(np.sqrt(d))
    return (g * rng.lognormal(0, 0.5, (n, 1)).astype(np.float32)).astype(np.float32)


def gaussian_queries(nq, d, seed=1):
    return np.random.default_rng(seed).standard_normal((nq, d)).astype(np.float32)


def sift_like(n, d, seed=0):
    """70% round(Gamma(0.8, 30)) clipped to [0, 255], 30% exact zeros."""
    rng = np.random.default_rng(seed)
    v = np.clip(np.round(rng.gamma(0.8, 30.0, (n, d))), 0, 255).astype(np.float32)
    v[rng.random((n, d)) < 0.3] = 0.0
    return v


def gist_like(n, d, seed=0):
    """|N(0,1)| * 0.05 with row norms scaled by LogNormal(0, 0.3)."""
    rng = np.random.default_rng(seed)
    v = np.abs(rng.standard_normal((n, d))).astype(np.float32) * np.float32(0.05)
    return (v * rng.lognormal(0, 0.3, (n, 1)).astype(np.float32)).astype(np.float32)


def recall(approx, exact):
    k = exact.shape[1]
    return float(np.mean([len(np.intersect1d(a, b)) / k for a, b in zip(approx, exact)]))
