"""Split-precision projection on the tensor cores (fhtDim 256 and 1024): a
build with precision "split_bf16" computes the three sign-flip + FWHT rounds
as H.X.H products of BF16 hi/lo operands with FP32 accumulation. The values
differ from the bit-exact FP32 butterflies by ~2^-16 relative per round, so
they are checked against the oracle's FP32 projection with a tolerance, and
the index they build against FP64 recall."""
import numpy as np
import pytest

from conftest import gist_like, netflix_like, recall

pytestmark = pytest.mark.gpu

# |split - fp32| <= TOL * max |projection| of the row (3 rounds of ~2^-16)
TOL = 2e-4


@pytest.mark.parametrize("d,D,R", [(150, 256, 2), (256, 256, 3), (960, 1024, 2), (300, 1024, 1),
                                   (1000, 256, 2)])
def test_tensor_projection_matches_fp32(gpu, oracle, d, D, R):
    n = 700
    X = netflix_like(n, d, seed=d)
    X[5] = 0.0  # zero row
    g = gpu.CEOs(n, d)
    g.setIndexParam(D, R, 10, 1, 7)
    g.precision = "split_bf16"
    g.build(X)
    P = g.projections()
    ref = oracle.project(X, D, R, 7)
    assert P.shape == ref.shape
    scale = np.maximum(np.abs(ref).max(axis=1, keepdims=True), 1e-30)
    err = np.abs(P.astype(np.float64) - ref) / scale
    fht = g.fhtDim
    if fht in (256, 1024):
        assert err.max() <= TOL, err.max()
        assert err.max() > 0  # the tensor path ran (the FP32 path is bit-exact)
    else:
        assert err.max() == 0
    assert np.all(P[5] == 0)


def test_tensor_build_recall_matches_fp32(gpu, oracle):
    n, d = 20000, 960
    X = gist_like(n, d, seed=5)
    Q = gist_like(100, d, seed=6)
    from ceos_gb300 import _capi

    gt, _ = _capi.bruteforce_fp64(X, Q, 10)
    rec = {}
    for prec in ("fp32", "split_bf16"):
        g = gpu.CEOs(n, d)
        g.setIndexParam(1024, 2, 200, 1, 42)
        g.precision = prec
        g.build_coCEOs_Est(X)
        g.n_probed_vectors, g.n_cand = 30, 600
        ids, dists = g.search_coCEOs_Est(Q, 10)
        rec[prec] = recall(ids, gt)
        exact = np.einsum("qkd,qd->qk", X[ids].astype(np.float64), Q.astype(np.float64))
        assert np.max(np.abs(dists - exact) / np.abs(exact)) < 1e-5
        if prec == "fp32":
            b32 = g.buckets()[0]
        else:
            bsp = g.buckets()[0]
    assert abs(rec["fp32"] - rec["split_bf16"]) <= 0.01, rec
    # the buckets are the same sets up to near-ties
    same = np.mean([len(np.intersect1d(a, b)) / a.size for a, b in
                    zip(b32.reshape(-1, b32.shape[-1]), bsp.reshape(-1, bsp.shape[-1]))])
    assert same > 0.98, same


@pytest.mark.parametrize("d,D,R", [(150, 128, 2),    # fhtDim 256
                                   (300, 1024, 1)])  # fhtDim 1024
def test_tensor_sampled_build_selects_exactly(gpu, d, D, R):
    """n > 65536 takes the sampled-threshold build; with the tensor-core
    projection its buckets must be exactly the two-ended top-m of the
    split-precision projections themselves. The dense build of the same index
    produces the same projection values (its row projection, the column dump
    and the fused emission run the same kernel; the threshold sample runs on
    the FP32 kernel and only filters the candidates), and the order is the
    library's: key of the value, then the smaller id."""
    n, m = 70000, 64
    X = netflix_like(n, d, seed=17)
    dense = gpu.CEOs(n, d)
    dense.setIndexParam(D, R, m, 1, 23)
    dense.precision = "split_bf16"
    dense.build(X)
    P = dense.projections()
    idx = gpu.CEOs(n, d)
    idx.setIndexParam(D, R, m, 1, 23)
    idx.precision = "split_bf16"
    idx.build_coCEOs_Est(X)
    bi, bv = idx.buckets()
    for col in range(D * R):
        for end, vals in ((0, P[:, col]), (1, -P[:, col])):
            u = vals.view(np.uint32).astype(np.int64)
            key = np.where(u & 0x80000000, ~u & 0xffffffff, u | 0x80000000)
            kth = np.partition(key, n - m)[n - m]
            cand = np.nonzero(key >= kth)[0]
            top = cand[np.lexsort((cand, -key[cand]))][:m]
            assert np.array_equal(bi[col, end], top), (col, end)
            assert np.array_equal(bv[col, end].view(np.uint32), vals[top].view(np.uint32)), (col, end)


def test_tensor_projection_stall_is_reported(gpu):
    """A tcgen05 projection whose products never complete (test hook: no
    products are issued and every wait gives up after 64 polls) ends its
    blocks and frees their tensor memory; the build reports CEOS_ERR_CUDA, and
    the device stays usable: the same build then succeeds and searches."""
    from ceos_gb300 import _capi

    n, d = 20000, 960
    X = gist_like(n, d, seed=31)
    L = _capi.lib()
    g = gpu.CEOs(n, d)
    g.setIndexParam(1024, 1, 50, 1, 42)
    g.precision = "split_bf16"
    assert L.ceos_debug_stall_tensor_products(64) == 0
    try:
        with pytest.raises(_capi.CEOsError, match="did not complete"):
            g.build_coCEOs_Est(X)
    finally:
        L.ceos_debug_stall_tensor_products(0)
    h = gpu.CEOs(n, d)
    h.setIndexParam(1024, 1, 50, 1, 42)
    h.precision = "split_bf16"
    h.build_coCEOs_Est(X)
    h.n_probed_vectors, h.n_cand = 10, 200
    ids, dists = h.search_coCEOs_Est(X[:16], 5)
    assert ids.shape == (16, 5) and np.all((ids >= 0) & (ids < n))
    exact = np.einsum("qkd,qd->qk", X[ids].astype(np.float64), X[:16].astype(np.float64))
    assert np.max(np.abs(dists - exact) / np.abs(exact)) < 1e-5
