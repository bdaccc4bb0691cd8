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
