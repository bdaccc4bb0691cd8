"""FP64 accuracy report of returned kNN rows (fuelg_knn_error) and the FP32
issue-rate measurement (fuelg_fp32_rate) behind the plain tiers' roofline.

The report is checked against the same quantities computed here in numpy
float64 from the returned lists: max relative error, near-ties (adjacent f32
distances equal or one ulp apart) and order flips (adjacent neighbours that
FP64 distances rank the other way)."""
import ctypes

import numpy as np
import pytest

from fuel_gb300 import SearchIndex, _lib

pytestmark = pytest.mark.gpu


def _report(ix, Q, idx, dist):
    rep = _lib.ErrorReport()
    _lib.check(_lib.load().fuelg_knn_error(ix._handle, _lib.ptr(np.ascontiguousarray(Q)), Q.shape[0],
                                           idx.shape[1], _lib.ptr(idx), _lib.ptr(dist), ctypes.byref(rep)))
    return rep.as_dict()


def _numpy_report(X, Q, idx, dist, euclid):
    ok = idx >= 0
    Xd, Qd = X.astype(np.float64), Q.astype(np.float64)
    D = np.zeros(idx.shape)
    for r in range(idx.shape[0]):
        v = idx[r][ok[r]]
        d = ((Xd[v] - Qd[r]) ** 2).sum(axis=1)
        D[r, :len(v)] = np.sqrt(d) if euclid else d
    err = np.abs(dist.astype(np.float64) - D)
    rel = np.where(D > 0, err / np.where(D > 0, D, 1), 0)
    pair = ok[:, 1:] & ok[:, :-1]
    gap = dist[:, 1:].view(np.int32).astype(np.int64) - dist[:, :-1].view(np.int32).astype(np.int64)
    ties = int(((gap >= 0) & (gap <= 1) & pair).sum())
    flips = int((((D[:, :-1] > D[:, 1:]) | ((D[:, :-1] == D[:, 1:]) & (idx[:, :-1] > idx[:, 1:]))) & pair).sum())
    return float(err[ok].max()), float(rel[ok].max()), int(ok.sum()), ties, flips


@pytest.mark.parametrize("metric", ["sqeuclidean", "euclidean"])
def test_error_report_matches_numpy(gpu, metric):
    rng = np.random.default_rng(4)
    X = rng.normal(size=(4000, 24)).astype(np.float32)
    X[100:130] = X[5] + np.float32(1e-7)  # near-duplicates: f32 ties and one-ulp neighbours
    Q = X[:300].copy()
    ix = SearchIndex(X, distance=metric, tree="linear")
    idx, dist = ix.knn(Q, 12, exclude_self=False)
    got = _report(ix, Q, idx, dist)
    ab, rel, pairs, ties, flips = _numpy_report(X, Q, idx, dist, metric == "euclidean")
    assert got["pairs"] == pairs == 300 * 12
    assert got["near_ties"] == ties and got["order_flips"] == flips
    assert abs(got["max_rel_err"] - rel) <= 1e-12 + 1e-9 * rel
    assert got["max_rel_err"] < 2e-6  # f32 distances within a few ulps of FP64


def test_error_report_exact_on_integer_data(gpu):
    rng = np.random.default_rng(2)
    X = np.minimum(rng.geometric(0.1, size=(3000, 64)) - 1, 255).astype(np.float32)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear", precision="bf16")
    idx, dist = ix.knn(X[:500], 20, exclude_self=False)
    got = _report(ix, X[:500], idx, dist)
    assert got["max_abs_err"] == 0.0 and got["order_flips"] == 0 and got["pairs"] == 500 * 20
    # padded rows (k > n) are skipped
    small = SearchIndex(X[:7], distance="sqeuclidean", tree="linear")
    i2, d2 = small.knn(X[:3], 10, exclude_self=False)
    assert _report(small, X[:3], i2, d2)["pairs"] == 21


def test_fp32_rate_is_plausible(gpu):
    r = ctypes.c_double()
    _lib.check(_lib.load().fuelg_fp32_rate(ctypes.byref(r)))
    # GB300: 152 SMs x 128 FP32 lanes at up to 2.07 GHz = 40.3e12 FMA/s
    assert 5.0 < r.value < 60.0, r.value
