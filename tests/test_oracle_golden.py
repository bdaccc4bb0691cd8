"""Pins the oracle to the reference's own known answers and golden vectors.

Sources (reference checkout paths):
  src/math/mod.rs:672-690          exact pairwise squared distances (f32 and f64)
  src/math/mod.rs (tests)          vec_row_sqdist vs the plain sum, 1e-5 relative
  src/search/linear_scan.rs:247-262  k=2 with a tie returns 3 results [1, 0, 2]
  src/search/linear_scan.rs:264-275  range search radius 1.0 returns [0, 1]
  src/search/precomputed.rs:136-165  duplicate points: kNN lists keep all ties
  src/outlier/knn.rs:78-96, src/outlier/lof.rs:193-211 with
  testdata/reference-outlier-scores.csv: KNN-10 and LOF-10 on
  testdata/6-gaussian-4d.csv, abs tol 1e-6 (fixtures in tests/golden/).
"""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ORDERS = ["arm", "x86"]


@pytest.mark.parametrize("order", ORDERS)
def test_pairwise_sqdist_f32_row_major(oracle, order):
    pts = np.array([[0.0, 1.0], [2.0, 3.0], [1.0, 4.0]], np.float32)
    got = oracle.pairwise_sqdist(pts, pts, order).ravel()
    assert got.tolist() == [0.0, 8.0, 10.0, 8.0, 0.0, 2.0, 10.0, 2.0, 0.0]


@pytest.mark.parametrize("order", ORDERS)
def test_pairwise_sqdist_f64_vectorized(oracle, order):
    pts = np.array([[1.0, 2.0, 3.0, 4.0], [4.0, 3.0, 2.0, 1.0], [0.0, 0.0, 0.0, 0.0]], np.float64)
    got = oracle.pairwise_sqdist(pts, pts, order).ravel()
    assert got.tolist() == [0.0, 20.0, 30.0, 20.0, 0.0, 30.0, 30.0, 30.0, 0.0]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("order", ORDERS)
def test_linear_scan_knn_keeps_tie(oracle, order, dtype):
    data = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0]], dtype)
    idx, dist = oracle.knn_with_ties(data, [1.0, 0.0], 2, metric="euclidean", order=order)
    assert idx.tolist() == [1, 0, 2]
    assert dist.dtype == dtype and dist[0] <= dist[1] <= dist[2]
    # and the marshalled row is truncated to k (python/search.rs:1195-1216)
    i2, d2 = oracle.knn(data, np.array([[1.0, 0.0]], dtype), 2, metric="euclidean", order=order)
    assert i2.tolist() == [[1, 0]]


@pytest.mark.parametrize("order", ORDERS)
def test_linear_scan_range(oracle, order):
    data = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0]], np.float64)
    off, idx, _ = oracle.range_search(data, np.array([[0.5, 0.0]]), 1.0, metric="euclidean", order=order)
    assert off.tolist() == [0, 2]
    assert idx.tolist() == [0, 1]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("order", ORDERS)
def test_precomputed_tie_semantics(oracle, order, dtype):
    pts = np.array([[0.0, 0.0], [0.0, 0.0], [1.0, 0.0], [1.0, 0.0], [2.0, 0.0]], dtype)
    for i in range(len(pts)):
        for k in (1, 2):
            idx, dist = oracle.knn_with_ties(pts, pts[i], k, metric="euclidean", order=order)
            assert len(idx) >= k
            kth = dist[k - 1]
            assert np.all(dist[k:] == kth)
            # every point at distance <= the k-th distance is present
            full = np.sqrt(((pts - pts[i]) ** 2).sum(1))
            assert sorted(idx.tolist()) == sorted(np.nonzero(full <= kth)[0].tolist())


@pytest.mark.parametrize("order", ORDERS)
def test_knn10_lof10_golden(oracle, order):
    g = json.load(open(os.path.join(GOLDEN, "gaussian4d.json")))
    ref = json.load(open(os.path.join(GOLDEN, "outlier_scores.json")))
    X = np.array(g["points"], np.float64)
    # for_each_knn (src/outlier/common.rs:13-49): search k+1, drop self, keep k
    idx, dist = oracle.knn(X, X, 10, metric="euclidean", order=order, exclude="kplus1")
    knn = oracle.knn_outlier(dist)
    lof = oracle.lof(idx, dist)
    assert np.max(np.abs(knn - np.array(ref["KNN-10"]))) <= 1e-6
    assert np.max(np.abs(lof - np.array(ref["LOF-10"]))) <= 1e-6


def test_knn10_golden_f32(oracle):
    """The f32 restatement on the same data stays within f32 rounding of the golden."""
    g = json.load(open(os.path.join(GOLDEN, "gaussian4d.json")))
    ref = json.load(open(os.path.join(GOLDEN, "outlier_scores.json")))
    X = np.array(g["points"], np.float32)
    idx, dist = oracle.knn(X, X, 10, metric="euclidean", exclude="kplus1")
    assert np.max(np.abs(oracle.knn_outlier(dist.astype(np.float64)) - np.array(ref["KNN-10"]))) <= 1e-6


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("order", ORDERS)
def test_row_sqdist_layout_cases(oracle, order, dtype):
    """src/math/mod.rs tests check_row_sqdist_layouts (C-order rows) and
    check_row_sqdist_strided: vec_row_sqdist -- math::sqdist per row, the
    order of Lloyd's later passes -- within 1e-5 relative (to max(expected,
    1)) of the plain sum of squared differences, on the reference's own value
    ramps and (n, d) sizes."""
    f64 = dtype == np.float64
    sizes = [(64, 32), (65, 32), (13, 7) if f64 else (9, 5), (100, 16)]
    for n, d in sizes:
        center = (np.arange(d) * 0.1 + 0.5).astype(dtype)
        pts = (np.arange(n * d) * 0.03 + 0.01).astype(dtype).reshape(n, d)
        for j in range(n):
            got = oracle.dist("sqdist", order, center, pts[j])
            diff = center - pts[j]
            want = (diff * diff).sum(dtype=dtype)
            assert abs(got - want) / max(want, 1.0) < 1e-5, (n, d, j)
    for n, d in [(17, 11), (64, 5)]:
        center = (np.arange(d) * 0.2 + 0.25).astype(dtype)
        base = (np.arange(n * d * 2) * 0.01 + 0.03).astype(dtype).reshape(n, 2 * d)
        pts = np.ascontiguousarray(base[:, ::2])
        for j in range(n):
            got = oracle.dist("sqdist", order, center, pts[j])
            diff = center - pts[j]
            want = (diff * diff).sum(dtype=dtype)
            assert abs(got - want) / max(want, 1.0) < 1e-5, (n, d, j)
