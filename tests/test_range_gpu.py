"""Parity of the GPU range search with linear_scan_range (bit-exact CSR)."""
import numpy as np
import pytest

from conftest import f32_bits, threads
from fuel_gb300 import SearchIndex, range_search

pytestmark = pytest.mark.gpu


def check(oracle, X, Q, radius, metric, order, exclude):
    ix = SearchIndex(X, distance=metric, tree="linear", order=order)
    gi, gd = ix.radius_search(Q if not exclude else X, radius, exclude_self=exclude)
    off, ci, cd = oracle.range_search(X, Q if not exclude else X, radius, metric=metric, order=order,
                                      exclude_self=exclude, threads=threads())
    m = len(gi)
    assert m == len(off) - 1
    for i in range(m):
        assert np.array_equal(gi[i], ci[off[i]:off[i + 1]]), i
        assert np.array_equal(f32_bits(gd[i]), f32_bits(cd[off[i]:off[i + 1]])), i


@pytest.mark.parametrize("metric", ["sqeuclidean", "euclidean"])
@pytest.mark.parametrize("order", ["arm", "x86"])
@pytest.mark.parametrize("d", [2, 9, 64])
def test_range_parity(gpu, oracle, metric, order, d):
    rng = np.random.default_rng(d)
    X = rng.normal(size=(1200, d)).astype(np.float32)
    Q = rng.normal(size=(97, d)).astype(np.float32)
    r = float(np.sqrt(d)) * (1.0 if metric == "euclidean" else np.sqrt(d))
    check(oracle, X, Q, r, metric, order, False)
    check(oracle, X, Q, r, metric, order, True)


def test_range_ties_and_empty(gpu, oracle):
    rng = np.random.default_rng(0)
    X = rng.integers(0, 3, size=(800, 4)).astype(np.float32)
    check(oracle, X, X[:50], 2.0, "sqeuclidean", "arm", False)
    check(oracle, X, X[:50], 0.0, "sqeuclidean", "arm", True)  # only exact duplicates
    check(oracle, X, X[:50], -1.0, "sqeuclidean", "arm", False)  # nothing


def test_range_search_function(gpu, oracle):
    X = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0]], np.float32)
    gi, gd = range_search(X, np.array([[0.5, 0.0]], np.float32), 1.0, tree="linear")
    assert gi[0].tolist() == [0, 1]  # src/search/linear_scan.rs:264-275


def _priority_reference(oracle, X, q, metric, skip, cutoff, cuts, skip_every):
    """The reference's LinearScanPrioritySearcher loop restated on the
    oracle's full (distance, index)-ordered list: filter [skip, cutoff],
    hand out in order, cutoff lowered at given steps, a point filter."""
    n = X.shape[0]
    i, d = oracle.knn(X, q[None, :], n, metric=metric)
    cand = [(float(dd), int(ii)) for dd, ii in zip(d[0], i[0]) if skip <= dd <= cutoff]
    out, pos = [], 0
    while True:
        if len(out) in cuts:
            cutoff = min(cutoff, cuts[len(out)])
        nxt = None
        while pos < len(cand):
            dd, ii = cand[pos]
            pos += 1
            if dd > np.float32(cutoff):
                break
            if dd < skip or (skip_every and ii % skip_every == 0):
                continue
            nxt = (dd, ii)
            break
        if nxt is None:
            return out
        out.append(nxt)


@pytest.mark.parametrize("metric", ["sqeuclidean", "euclidean"])
def test_priority_searcher(gpu, oracle, metric):
    rng = np.random.default_rng(13)
    X = rng.integers(0, 5, size=(700, 6)).astype(np.float32)  # ties
    q = X[17].copy()
    ix = SearchIndex(X, distance=metric, tree="linear")
    for skip, cutoff, cuts, every in ((0.0, np.inf, {}, 0), (2.0, 30.0, {5: 12.0, 40: 9.0}, 3), (1.0, 1.0, {}, 0)):
        ps = ix.priority_searcher(q)
        ps.reset_with_limits(cutoff, skip)
        got = []
        while True:
            if len(got) in cuts:
                ps.decrease_cutoff(cuts[len(got)])
            r = ps.next(skip_point=(lambda i, e=every: e and i % e == 0) if every else None)
            if r is None:
                break
            got.append(r)
        ref = _priority_reference(oracle, X, q, metric, skip, cutoff, cuts, every)
        assert [g[1] for g in got] == [r[1] for r in ref]
        assert np.array_equal(np.float32([g[0] for g in got]), np.float32([r[0] for r in ref]))
    ps = ix.priority_searcher(q)
    assert ps.all_lower_bound() == 0.0
    first = ps.next()
    assert first[0] == 0.0 and np.array_equal(X[first[1]], q)
    assert ps.all_lower_bound() >= first[0]
