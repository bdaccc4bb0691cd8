"""Float64 data on the GPU: the exact FP64 scan (fuelg_*_f64).

fuel builds a float64 index for every input that is not float32
(python/fuel/_dispatch.py:8-19, build_linear_scan_f64 python/search.rs:
1371-1389) and compares f64 distances in its f64 operation order
(src/distance/squared_euclidean.rs:44-67 / :99-133).  Every result here must
equal the oracle's f64 restatement bit for bit -- indices, f64 distance bits,
tie lists, range lists, pairwise matrices -- for both summation orders, every
exclude rule, k beyond n and tie-heavy integer data; and the KNN-10 / LOF-10
scores computed from the GPU's own neighbour lists of the reference's golden
data must match the reference's golden scores.
"""
import ctypes
import json
import os

import numpy as np
import pytest

from conftest import threads
from fuel_gb300 import SearchIndex, _lib, pairwise_distances
from fuel_gb300.search import _take_csr

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MODES = {"none": _lib.EXCLUDE_NONE, "linear": _lib.EXCLUDE_LINEAR, "kplus1": _lib.EXCLUDE_KPLUS1}


def gauss(n, d, seed):
    return np.random.default_rng(seed).normal(size=(n, d)) * 3.0


def ints(n, d, seed):
    return np.random.default_rng(seed).integers(0, 3, size=(n, d)).astype(np.float64)


def bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


def gpu_knn(ix, Q, k, mode):
    """fuelg_knn_f64 through the C ABI; Q None = the index's own rows."""
    m = ix.shape[0] if Q is None else Q.shape[0]
    idx = np.empty((m, k), np.int64)
    dist = np.empty((m, k), np.float64)
    st = _lib.Stats()
    _lib.check(_lib.load().fuelg_knn_f64(ix._handle, None if Q is None else _lib.ptr(Q), m, k, mode,
                                         _lib.ptr(idx), _lib.ptr(dist), ctypes.byref(st)))
    assert st.precision_used == 5
    return idx, dist


def gpu_lists(ix, Q, m, call, *args):
    lib = _lib.load()
    res = ctypes.c_void_p()
    _lib.check(getattr(lib, call)(ix._handle, None if Q is None else _lib.ptr(Q), m, *args, ctypes.byref(res),
                                  None))
    try:
        return _take_csr(lib, res, m, True)
    finally:
        lib.fuelg_range_free(res)


@pytest.mark.parametrize("order", ["arm", "x86"])
@pytest.mark.parametrize("metric", ["sqeuclidean", "euclidean"])
@pytest.mark.parametrize("d", [1, 3, 4, 7, 8, 9, 16, 33])
def test_knn_f64_matches_oracle(gpu, oracle, order, metric, d):
    X = gauss(1500, d, d)
    Q = gauss(200, d, d + 100)
    ix = SearchIndex(X, distance=metric, tree="linear", order=order)
    for k in (1, 7, 40):
        gi, gd = ix.knn(Q, k, exclude_self=False)
        oi, od = oracle.knn(X, Q, k, metric=metric, order=order, threads=threads())
        assert gd.dtype == np.float64
        assert np.array_equal(gi, oi), f"k={k}"
        assert np.array_equal(bits(gd), bits(od)), f"k={k}"


@pytest.mark.parametrize("order", ["arm", "x86"])
@pytest.mark.parametrize("exclude", ["none", "linear", "kplus1"])
def test_knn_f64_ties_exclude_and_k_beyond_n(gpu, oracle, order, exclude):
    X = ints(600, 3, 7)  # 27 distinct points: long tie runs everywhere
    ix = SearchIndex(X, distance="euclidean", tree="linear", order=order)
    for k in (1, 5, 30, 605):
        gi, gd = gpu_knn(ix, None, k, MODES[exclude])
        oi, od = oracle.knn(X, X, k, metric="euclidean", order=order, exclude=exclude, threads=threads())
        assert np.array_equal(gi, oi), f"k={k}"
        assert np.array_equal(bits(gd), bits(od)), f"k={k}"


@pytest.mark.parametrize("order", ["arm", "x86"])
@pytest.mark.parametrize("exclude", ["none", "linear", "kplus1"])
def test_knn_ties_f64_lists(gpu, oracle, order, exclude):
    X = ints(400, 2, 9)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear", order=order)
    for k in (1, 4, 25):
        off, idx, dist = gpu_lists(ix, None, X.shape[0], "fuelg_knn_ties_f64", k, MODES[exclude])
        ooff, oidx, odist = oracle.knn_ties(X, X, k, metric="sqeuclidean", order=order, exclude=exclude)
        assert np.array_equal(off, ooff), f"k={k}"
        assert np.array_equal(idx, oidx), f"k={k}"
        assert np.array_equal(bits(dist), bits(odist)), f"k={k}"
    # explicit queries, and the Python mirror
    Q = X[::7].copy()
    li, ld = ix.knn_with_ties(Q, 6, exclude_self=False)
    ooff, oidx, odist = oracle.knn_ties(X, Q, 6, metric="sqeuclidean", order=order)
    assert np.array_equal(np.concatenate(li), oidx)
    assert np.array_equal(bits(np.concatenate(ld)), bits(odist))


@pytest.mark.parametrize("order", ["arm", "x86"])
@pytest.mark.parametrize("metric", ["sqeuclidean", "euclidean"])
def test_range_f64_matches_oracle(gpu, oracle, order, metric):
    for X in (gauss(2000, 5, 3), ints(1500, 4, 4)):
        Q = X[:120].copy()
        ix = SearchIndex(X, distance=metric, tree="linear", order=order)
        for radius in (0.0, 1.0, 2.5, 6.0):
            for excl in (0, 1):
                off, idx, dist = gpu_lists(ix, Q, Q.shape[0], "fuelg_range_f64", float(radius), excl)
                ooff, oidx, odist = oracle.range_search(X, Q, radius, metric=metric, order=order,
                                                        exclude_self=bool(excl), threads=threads())
                assert np.array_equal(off, ooff), (radius, excl)
                assert np.array_equal(idx, oidx), (radius, excl)
                assert np.array_equal(bits(dist), bits(odist)), (radius, excl)


@pytest.mark.parametrize("order", ["arm", "x86"])
@pytest.mark.parametrize("metric", ["sqeuclidean", "euclidean"])
@pytest.mark.parametrize("form", ["condensed", "square"])
def test_pairwise_f64_matches_oracle(gpu, oracle, order, metric, form):
    for n, d in ((1, 3), (2, 5), (70, 7), (45, 33)):
        P = gauss(n, d, n + d)
        got = pairwise_distances(P, distance=metric, form=form, order=order)
        assert got.dtype == np.float64
        full = np.empty((n, n))
        for i in range(n):
            for j in range(n):
                v = oracle.dist("knn", order, P[i], P[j])
                full[i, j] = np.sqrt(v) if metric == "euclidean" else v
        want = full if form == "square" else full[np.tril_indices(n, -1)]
        assert np.array_equal(bits(got), bits(want)), (n, d)


@pytest.mark.parametrize("order", ["arm", "x86"])
def test_knn10_lof10_golden_from_gpu_lists(gpu, oracle, order):
    """for_each_knn (src/outlier/common.rs:13-49: search k+1, drop self, keep k)
    on the reference's 6-gaussian-4d data, scored KNN-10 / LOF-10 from the GPU
    lists against the reference's golden scores (src/outlier/knn.rs:78-96,
    src/outlier/lof.rs:193-211)."""
    g = json.load(open(os.path.join(GOLDEN, "gaussian4d.json")))
    ref = json.load(open(os.path.join(GOLDEN, "outlier_scores.json")))
    X = np.array(g["points"], np.float64)
    ix = SearchIndex(X, distance="euclidean", tree="linear", order=order)
    idx, dist = gpu_knn(ix, None, 10, _lib.EXCLUDE_KPLUS1)
    oi, od = oracle.knn(X, X, 10, metric="euclidean", order=order, exclude="kplus1")
    assert np.array_equal(idx, oi) and np.array_equal(bits(dist), bits(od))
    assert np.max(np.abs(oracle.knn_outlier(dist) - np.array(ref["KNN-10"]))) <= 1e-6
    assert np.max(np.abs(oracle.lof(idx, dist) - np.array(ref["LOF-10"]))) <= 1e-6


def test_float64_python_mirror(gpu, oracle):
    X = gauss(800, 6, 11)
    ix = SearchIndex(X)  # euclidean, float64
    assert ix.dtype == np.float64
    i, d = ix.knn(X, 5)  # the indexed array itself: the linear-index exclude rule
    oi, od = oracle.knn(X, X, 5, metric="euclidean", order=ix.order, exclude="linear", threads=threads())
    assert np.array_equal(i, oi) and np.array_equal(bits(d), bits(od))
    assert ix.last_stats["precision_used"] == 5
    # integer input becomes a float64 index, as in fuel
    Xi = np.random.default_rng(2).integers(0, 5, size=(300, 3)).astype(np.int32)
    ii = SearchIndex(Xi, distance="sqeuclidean")
    assert ii.dtype == np.float64
    gi, gd = ii.knn(Xi[:20].astype(np.float64), 4, exclude_self=False)
    oi, od = oracle.knn(Xi.astype(np.float64), Xi[:20].astype(np.float64), 4, metric="sqeuclidean",
                        order=ii.order, threads=threads())
    assert np.array_equal(gi, oi) and np.array_equal(bits(gd), bits(od))
    # the precomputed table (tie lists of the index's own rows) and its k+1 rule
    ip = SearchIndex(X, precompute=8)
    pi, pd = ip.knn(X, 5)
    assert ip.last_stats["served_from"] == "precomputed table"
    oi, od = oracle.knn(X, X, 5, metric="euclidean", order=ip.order, exclude="kplus1", threads=threads())
    assert np.array_equal(pi, oi) and np.array_equal(bits(pd), bits(od))
    # radius search and the priority searcher in the index dtype
    li, ld = ix.radius_search(X[:30], 2.0, exclude_self=False)
    off, oidx, odist = oracle.range_search(X, X[:30], 2.0, metric="euclidean", order=ix.order)
    assert np.array_equal(np.concatenate(li), oidx) and np.array_equal(bits(np.concatenate(ld)), bits(odist))
    ps = ix.priority_searcher(X[3])
    first = ps.next()
    assert first is not None and first[1] == 3 and first[0] == 0.0
    # a float32 call on a float64 index is refused, and the reverse
    lib = _lib.load()
    q32 = X[:2].astype(np.float32)
    out_i = np.empty((2, 1), np.int64)
    out_d = np.empty((2, 1), np.float32)
    assert lib.fuelg_knn(ix._handle, _lib.ptr(q32), 2, 1, 0, 0, _lib.ptr(out_i), _lib.ptr(out_d), None) == _lib.EINVAL
    i32 = SearchIndex(X.astype(np.float32))
    out_d64 = np.empty((2, 1), np.float64)
    assert lib.fuelg_knn_f64(i32._handle, _lib.ptr(X[:2]), 2, 1, 0, _lib.ptr(out_i), _lib.ptr(out_d64),
                             None) == _lib.EINVAL
    with pytest.raises(NotImplementedError):
        SearchIndex(X, precision="split_bf16")


def test_float64_empty_and_edge_shapes(gpu, oracle):
    X = gauss(5, 3, 1)
    ix = SearchIndex(X, distance="sqeuclidean")
    i, d = ix.knn(X[:0], 3, exclude_self=False)
    assert i.shape == (0, 3)
    i, d = ix.knn(X[:2], 0, exclude_self=False)
    assert i.shape == (2, 0)
    empty = SearchIndex(np.zeros((0, 3)), distance="sqeuclidean")
    i, d = empty.knn(X[:2], 4, exclude_self=False)
    assert (i == -1).all() and np.isinf(d).all()
    li, ld = empty.radius_search(X[:2], 1.0, exclude_self=False)
    assert all(len(a) == 0 for a in li)
    off, idx, dist = gpu_lists(empty, X[:2], 2, "fuelg_knn_ties_f64", 3, 0)
    assert off.tolist() == [0, 0, 0]
