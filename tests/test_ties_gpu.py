"""Tie-inclusive kNN (fuelg_knn_ties) and the precomputed kNN table on the GPU.

fuel's KnnSearch::search_knn returns the k nearest points plus every point tied
with the k-th distance (KNNHeap::into_vec, src/api/search.rs:80-151);
PrecomputedKnnSearcher builds those lists to max_k for every indexed point and
slices them with subset_with_ties (src/search/precomputed.rs:36-89).  The GPU
lists must equal the oracle's list for list (indices and f32 distance bits),
for every exclude rule and precision tier, including rows whose tie run is
longer than the call's spare ranks (those rows are completed by a range scan).
"""
import ctypes

import numpy as np
import pytest

import fuel_gb300
from fuel_gb300 import _lib

pytestmark = pytest.mark.gpu

from conftest import f32_bits  # noqa: E402


def _csr(lib, X, Q, k, mode, precision, metric="sqeuclidean", order=None, queries_none=False):
    order = order or _lib.default_order()
    h = ctypes.c_void_p()
    _lib.check(lib.fuelg_index_create(_lib.ptr(X), X.shape[0], X.shape[1], _lib.METRIC[metric], _lib.ORDER[order],
                                      ctypes.byref(h)))
    try:
        res = ctypes.c_void_p()
        st = _lib.Stats()
        m = X.shape[0] if queries_none else Q.shape[0]
        _lib.check(lib.fuelg_knn_ties(h, None if queries_none else _lib.ptr(Q), m, k, mode,
                                      _lib.PRECISION[precision], ctypes.byref(res), ctypes.byref(st)))
        try:
            from fuel_gb300.search import _take_csr
            off, idx, dist = _take_csr(lib, res, m)
        finally:
            lib.fuelg_range_free(res)
        return off, idx, dist, st.as_dict()
    finally:
        lib.fuelg_index_destroy(h)


def _assert_same(got, ref):
    go, gi, gd = got[:3]
    ro, ri, rd = ref
    assert np.array_equal(go, ro), "row lengths differ from the oracle"
    assert np.array_equal(gi, ri), "neighbour indices differ from the oracle"
    assert np.array_equal(f32_bits(gd), f32_bits(rd)), "distances differ from the oracle"


MODES = {"none": _lib.EXCLUDE_NONE, "linear": _lib.EXCLUDE_LINEAR, "kplus1": _lib.EXCLUDE_KPLUS1}


@pytest.mark.parametrize("exclude", ["none", "linear", "kplus1"])
@pytest.mark.parametrize("k", [1, 5, 40])
def test_ties_plain_tie_heavy(gpu, lib, oracle, exclude, k):
    """Integer data with few distinct values: long tie runs at the k-th distance."""
    rng = np.random.default_rng(k)
    X = rng.integers(0, 3, size=(1500, 4)).astype(np.float32)  # 81 distinct points, ~18 copies each
    got = _csr(lib, X, X, k, MODES[exclude], "fp32")
    ref = oracle.knn_ties(X, X, k, exclude=exclude)
    _assert_same(got, ref)
    lens = np.diff(ref[0])
    assert lens.max() > k + 1 + max(8, (k + 1) // 4), "the data must produce tie runs longer than the spare ranks"


@pytest.mark.parametrize("metric", ["sqeuclidean", "euclidean"])
def test_ties_duplicates_take_the_range_path(gpu, lib, oracle, metric):
    """300 copies of one point: every copy's tie run at distance 0 holds 300
    entries, far beyond the spare ranks of k=4."""
    rng = np.random.default_rng(5)
    X = rng.normal(size=(2000, 10)).astype(np.float32)
    X[100:400] = X[7]
    Q = np.concatenate([X[:500], rng.normal(size=(50, 10)).astype(np.float32)])
    got = _csr(lib, X, Q, 4, _lib.EXCLUDE_NONE, "fp32", metric=metric)
    ref = oracle.knn_ties(X, Q, 4, metric=metric)
    _assert_same(got, ref)
    assert np.diff(ref[0]).max() >= 300


@pytest.mark.parametrize("precision", ["bf16", "split_bf16", "fp16"])
def test_ties_tensor_core_tiers(gpu, lib, oracle, precision):
    rng = np.random.default_rng(11)
    # integer data (exact BF16 / FP16 screen, many ties) and real-valued data (re-scored)
    Xi = np.minimum(rng.geometric(0.3, size=(3000, 48)) - 1, 20).astype(np.float32)
    got = _csr(lib, Xi, Xi[:400], 10, _lib.EXCLUDE_LINEAR, precision)
    assert got[3]["precision_used"] != 0, "tensor-core tier not used"
    _assert_same(got, oracle.knn_ties(Xi, Xi[:400], 10, exclude="linear"))
    Xr = rng.normal(size=(3000, 40)).astype(np.float32)
    Xr[200:260] = Xr[3]  # duplicates: ties beyond the spare ranks
    got = _csr(lib, Xr, Xr[:300], 8, _lib.EXCLUDE_KPLUS1, precision)
    _assert_same(got, oracle.knn_ties(Xr, Xr[:300], 8, exclude="kplus1"))


def test_ties_index_queries_and_edges(gpu, lib, oracle):
    rng = np.random.default_rng(3)
    X = rng.integers(0, 4, size=(700, 5)).astype(np.float32)
    # queries NULL = the index's own rows (the precomputed-table build)
    got = _csr(lib, X, None, 12, _lib.EXCLUDE_NONE, "fp32", queries_none=True)
    _assert_same(got, oracle.knn_ties(X, X, 12))
    # k >= n: every point, sorted
    small = X[:9].copy()
    got = _csr(lib, small, small, 20, _lib.EXCLUDE_LINEAR, "fp32")
    _assert_same(got, oracle.knn_ties(small, small, 20, exclude="linear"))
    # k = 0: empty lists
    got = _csr(lib, X, X[:5], 0, _lib.EXCLUDE_NONE, "fp32")
    assert np.array_equal(got[0], np.zeros(6, np.int64))


def test_precomputed_table_serves_knn(gpu, oracle):
    rng = np.random.default_rng(8)
    X = rng.integers(0, 3, size=(1200, 7)).astype(np.float32)
    order = _lib.default_order()
    ix = fuel_gb300.SearchIndex(X, distance="sqeuclidean", tree="linear", precompute=15, order=order)
    max_k, off, idx, dist = ix._table
    assert max_k == 15
    _assert_same((off, idx, dist), oracle.knn_ties(X, X, 15, order=order))
    for k in (1, 6, 14):
        gi, gd = ix.knn(X, k)  # exclude_self: the k+1 rule of the precomputed path
        assert ix.last_stats.get("served_from") == "precomputed table"
        ci, cd = oracle.knn(X, X, k, metric="sqeuclidean", order=order, exclude="kplus1", threads=8)
        assert np.array_equal(gi, ci) and np.array_equal(f32_bits(gd), f32_bits(cd))
    gi, gd = ix.knn(X, 15, exclude_self=False)
    ci, cd = oracle.knn(X, X, 15, metric="sqeuclidean", order=order, threads=8)
    assert np.array_equal(gi, ci) and np.array_equal(f32_bits(gd), f32_bits(cd))
    # beyond max_k: the scan answers, same rule
    gi, gd = ix.knn(X, 20)
    assert ix.last_stats.get("served_from") is None
    ci, cd = oracle.knn(X, X, 20, metric="sqeuclidean", order=order, exclude="kplus1", threads=8)
    assert np.array_equal(gi, ci) and np.array_equal(f32_bits(gd), f32_bits(cd))
    # the Python tie-inclusive call
    li, ld = ix.knn_with_ties(X, 3)
    ro, ri, rd = oracle.knn_ties(X, X, 3, order=order, exclude="kplus1")
    assert all(np.array_equal(li[i], ri[ro[i]:ro[i + 1]]) for i in range(X.shape[0]))
