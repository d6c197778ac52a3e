"""CPU checks of the C-ABI library: it loads, exports every symbol that
include/ceos_gb300.h declares, and validates parameters on the host exactly
as the reference does, without launching any device work."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(ceos_[a-z0-9_]+)\s*\(", src):
            syms.add(m.group(1))
    return syms


def test_library_exports_declared_symbols(ceos):
    from ceos_gb300 import _capi

    L = _capi.lib()
    syms = declared_symbols()
    assert len(syms) >= 40
    for s in sorted(syms):
        assert hasattr(L, s), s
        assert s in _capi.SIGNATURES, f"{s} has no ctypes signature"
    assert L.ceos_abi_version() == 1


def test_index_param_semantics(ceos):
    idx = ceos.CEOs(1000, 300)
    # class defaults (src/CEOs.h:52-54)
    assert (idx.n_probed_vectors, idx.n_probed_points, idx.n_cand) == (10, 10, 10)
    idx.setIndexParam(1024, 2, 100, 8, 42)
    # set_CEOsParam resets n_probed_points = top_m (src/CEOs.h:69)
    assert idx.n_probed_points == 100
    assert idx.fhtDim == 1024 and idx.n_proj == 1024 and idx.n_repeats == 2 and idx.top_m == 100
    idx.setIndexParam(256, 1, 10)
    assert idx.fhtDim == 512  # n_proj < n_features -> 2^ceil(log2 d)
    idx.n_probed_vectors = 20
    idx.n_cand = 500
    assert (idx.n_probed_vectors, idx.n_cand) == (20, 500)
    assert idx.centering is False
    idx.centering = True
    assert idx.centering is True


def test_stream_param_semantics(ceos):
    s = ceos.streamCEOs(128)
    s.setIndexParam(256, 2, 50)
    # set_streamCEOsParam sets n_probed_vectors = top_m, not n_probed_points
    # (src/streamCEOs.h:58)
    assert s.n_probed_vectors == 50 and s.n_probed_points == 10


def test_errors_without_device_work(ceos):
    with pytest.raises(ValueError):
        ceos.CEOs(0, 10)
    idx = ceos.CEOs(100, 16)
    idx.setIndexParam(32, 1, 10, 1, 0)
    with pytest.raises(RuntimeError):  # not built
        idx.search_coCEOs_Est(np.zeros((1, 16), np.float32), 5)
    with pytest.raises(ValueError):  # wrong shape
        idx.build(np.zeros((100, 15), np.float32))
    with pytest.raises(RuntimeError):
        s = ceos.streamCEOs(16)
        s.update(np.zeros((1, 16), np.float32), 0)


def test_no_cpu_fallback(ceos):
    """Without a CUDA device the library refuses instead of computing on the
    host."""
    from ceos_gb300 import _capi

    if _capi.lib().ceos_device_count() > 0:
        pytest.skip("a GPU is visible")
    idx = ceos.CEOs(64, 8)
    idx.setIndexParam(16, 1, 4, 1, 0)
    with pytest.raises(_capi.CEOsError, match="no CUDA device"):
        idx.build_coCEOs_Est(np.ones((64, 8), np.float32))


def test_server_rejects_unbuilt_index(ceos):
    from ceos_gb300 import _capi
    from ceos_gb300.serving import Server

    cfg = _capi.ServerConfig()
    assert _capi.lib().ceos_server_config_init(cfg) == 0
    assert (cfg.algo, cfg.n_slots, cfg.max_batch, cfg.max_neighbors, cfg.max_probed_vectors,
            cfg.mem_budget_bytes, cfg.use_graphs) == (_capi.ALGO_COCEOS, 4, 256, 100, 80, 0, 1)
    idx = ceos.CEOs(100, 8)
    with pytest.raises(RuntimeError, match="built"):
        Server(idx)
    with pytest.raises(ValueError):
        Server(idx, algo="dense")
