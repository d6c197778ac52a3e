"""The pybind11 drop-in module `CEOs` (ceos_gb300/pybind/ceos_module.cpp).

It carries the reference's module name and bindings (python/python_wrapper.cpp
:13-74): the same classes, constructor arguments, setIndexParam keywords and
defaults, read/write attributes and methods. The CPU tests check that surface
and that there is no CPU path; the GPU test runs the full Netflix-shaped 17,770 x 300 workload
through `import CEOs` against the committed outputs of the reference's own
code.
"""
import os
import sys

import numpy as np
import pytest

from conftest import has_gpu

LIBDIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "ceos_gb300", "_lib")


@pytest.fixture(scope="module")
def CEOs():
    from ceos_gb300 import build

    build.build()
    if LIBDIR not in sys.path:
        sys.path.insert(0, LIBDIR)
    import CEOs as mod

    assert os.path.dirname(os.path.abspath(mod.__file__)) == LIBDIR
    return mod


def _params(fn):
    """[(name, default or None)] of a pybind11 function, from its signature
    line (the type spelling differs between pybind11 versions)."""
    line = (fn.__doc__ or "").splitlines()[0]
    inner = line[line.index("(") + 1:line.rindex(")")]
    inner = inner[:inner.rindex(")")] if inner.count("(") < inner.count(")") else inner
    parts, depth, cur = [], 0, ""
    for ch in inner:
        if ch in "[(":
            depth += 1
        elif ch in "])":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    out = []
    for p_ in parts:
        name = p_.split(":")[0].strip()
        default = p_.split(" = ")[1].strip() if " = " in p_ else None
        if name != "self":
            out.append((name, default))
    return out


def test_module_surface(CEOs):
    assert CEOs.__name__ == "CEOs"
    for cls, methods in ((CEOs.CEOs, ["setIndexParam", "set_threads", "clear", "build", "search",
                                      "build_coCEOs_Est", "search_coCEOs_Est", "build_CEOs_Hash",
                                      "search_CEOs_Hash"]),
                         (CEOs.streamCEOs, ["setIndexParam", "set_threads", "clear", "build", "update",
                                            "estimate_search", "hash_search"])):
        for m in methods:
            assert hasattr(cls, m), (cls, m)
    assert _params(CEOs.CEOs.setIndexParam) == [("n_proj", None), ("n_repeats", "1"), ("top_m", "10"),
                                                ("n_threads", "-1"), ("random_seed", "-1")]
    assert _params(CEOs.streamCEOs.setIndexParam) == [("n_proj", None), ("n_repeats", "1"),
                                                      ("top_points", "1"), ("n_threads", "-1"),
                                                      ("random_seed", "-1")]
    for fn in (CEOs.CEOs.search, CEOs.CEOs.search_coCEOs_Est, CEOs.CEOs.search_CEOs_Hash,
               CEOs.streamCEOs.estimate_search, CEOs.streamCEOs.hash_search):
        assert _params(fn) == [("queries", None), ("n_neighbors", None), ("verbose", "False")]
    for fn in (CEOs.CEOs.build, CEOs.CEOs.build_coCEOs_Est, CEOs.CEOs.build_CEOs_Hash,
               CEOs.streamCEOs.build):
        assert _params(fn) == [("dataset", None)]
    assert _params(CEOs.streamCEOs.update) == [("new_dataset", None), ("n_delPoints", "0")]
    assert _params(CEOs.CEOs.__init__) == [("n_points", None), ("n_features", None)]
    assert _params(CEOs.streamCEOs.__init__) == [("n_features", None)]


def test_attribute_semantics(CEOs):
    i = CEOs.CEOs(1000, 20)
    assert (i.n_probed_vectors, i.n_probed_points, i.n_cand, i.centering) == (10, 10, 10, False)
    i.setIndexParam(32, 2, 77, 1, 42)
    assert i.n_probed_points == 77          # src/CEOs.h:70
    i.n_probed_vectors, i.n_cand = 12, 300
    assert (i.n_probed_vectors, i.n_cand) == (12, 300)
    i.centering = True
    assert i.centering
    s = CEOs.streamCEOs(20)
    s.setIndexParam(32, 2, 55, 1, 42)
    assert s.n_probed_vectors == 55 and s.n_probed_points == 10  # src/streamCEOs.h:42,58
    with pytest.raises(ValueError):
        i.precision = "fp16"


@pytest.mark.skipif(has_gpu(), reason="checks the behaviour without a device")
def test_no_cpu_path(CEOs):
    i = CEOs.CEOs(100, 8)
    i.setIndexParam(16, 2, 10, 1, 42)
    with pytest.raises(RuntimeError, match="no CUDA device"):
        i.build_coCEOs_Est(np.zeros((100, 8), np.float32))


@pytest.mark.gpu
def test_netflix_workload_through_import_CEOs(gpu, CEOs):
    """The full Netflix-shaped 17,770 x 300 workload through `import CEOs`, checked against the
    reference's own outputs and bit for bit against the ctypes module."""
    from golden.make_reference_golden import NETFLIX, netflix_inputs
    from parity import compare_results

    f = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_netflix.npz"))
    X, Q = netflix_inputs()
    for kind, b, srch in (("coceos", "build_coCEOs_Est", "search_coCEOs_Est"),
                          ("hash", "build_CEOs_Hash", "search_CEOs_Hash"),
                          ("dense", "build", "search")):
        idx = CEOs.CEOs(NETFLIX["n"], NETFLIX["d"])
        idx.setIndexParam(NETFLIX["D"], NETFLIX["R"], NETFLIX["m"], 8, NETFLIX["seed"])
        getattr(idx, b)(X.astype(np.float64))  # another dtype: converted like the reference's Ref
        idx.n_probed_vectors, idx.n_cand = NETFLIX["s"], NETFLIX["c"]
        ids, dists = getattr(idx, srch)(Q, NETFLIX["k"])
        assert ids.dtype == np.int32 and dists.dtype == np.float32 and ids.shape == (NETFLIX["nq"], NETFLIX["k"])
        ok, stats = compare_results(ids, dists, f[f"{kind}_ids"], f[f"{kind}_dists"])
        assert ok, (kind, stats)
        g = gpu.CEOs(NETFLIX["n"], NETFLIX["d"])
        g.setIndexParam(NETFLIX["D"], NETFLIX["R"], NETFLIX["m"], 8, NETFLIX["seed"])
        getattr(g, b)(X)
        g.n_probed_vectors, g.n_cand = NETFLIX["s"], NETFLIX["c"]
        gi, gd = getattr(g, srch)(Q, NETFLIX["k"])
        assert np.array_equal(gi, ids) and np.array_equal(gd.view(np.uint32), dists.view(np.uint32))
    # streamCEOs through the module, and the reference's error path
    st = CEOs.streamCEOs(NETFLIX["d"])
    st.setIndexParam(256, 2, 50, 1, 7)
    st.build(X[:5000])
    st.update(X[5000:6000], 500)
    st.n_probed_vectors, st.n_probed_points, st.n_cand = 20, 50, 200
    ids, _ = st.estimate_search(Q[:10], 10)
    assert ids.shape == (10, 10)
    with pytest.raises(ValueError):
        st.update(X[:10], 10 ** 6)
