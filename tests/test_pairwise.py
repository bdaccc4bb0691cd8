"""pairwise_distances: the 'precomputed' conversions (host logic, CPU) and the
GPU kernel against the oracle's restatement of compute_pairwise_condensed /
compute_pairwise_dense (bit-exact, both summation orders and metrics)."""
import numpy as np
import pytest

from conftest import threads
from fuel_gb300 import pairwise_distances


def test_precomputed_conversions_cpu():
    rng = np.random.default_rng(0)
    P = rng.random((7, 3))
    sq = np.sqrt(((P[:, None, :] - P[None, :, :]) ** 2).sum(-1))
    ti, tj = np.tril_indices(7, -1)
    # scipy pdist order: pairs (a, b), a < b, row-major
    pd = np.array([sq[a, b] for a in range(7) for b in range(a + 1, 7)])
    internal = pairwise_distances(pd, distance="precomputed")
    np.testing.assert_array_equal(internal, sq[ti, tj])
    np.testing.assert_array_equal(pairwise_distances(pd, distance="precomputed", form="square"), sq)
    np.testing.assert_array_equal(pairwise_distances(sq, distance="precomputed"), sq[ti, tj])
    assert pairwise_distances(sq, distance="precomputed", form="square") is sq
    with pytest.raises(ValueError):
        pairwise_distances(np.zeros(5), distance="precomputed")
    with pytest.raises(ValueError):
        pairwise_distances(np.zeros((3, 4)), distance="precomputed")
    with pytest.raises(ValueError):
        pairwise_distances(P.astype(np.float32), form="triangle")
    with pytest.raises(ValueError):
        pairwise_distances(np.zeros(4, np.float32))
    with pytest.raises(NotImplementedError):
        pairwise_distances(P.astype(np.float32), distance="cosine")


@pytest.mark.gpu
@pytest.mark.parametrize("order", ["arm", "x86"])
@pytest.mark.parametrize("metric", ["euclidean", "sqeuclidean"])
@pytest.mark.parametrize("form", ["condensed", "square"])
@pytest.mark.parametrize("n,d", [(1, 5), (2, 3), (33, 1), (70, 7), (129, 64), (300, 100), (150, 128), (140, 129),
                                 (257, 784)])
def test_pairwise_matches_oracle(gpu, oracle, order, metric, form, n, d):
    rng = np.random.default_rng(n * 31 + d)
    X = rng.normal(size=(n, d)).astype(np.float32)
    g = pairwise_distances(X, distance=metric, form=form, order=order)
    c = oracle.pairwise_distances(X, metric, form, order=order, threads=threads())
    assert g.shape == c.shape and g.dtype == np.float32
    np.testing.assert_array_equal(g.view(np.uint32), c.view(np.uint32))


@pytest.mark.gpu
def test_pairwise_duplicates_and_integer_data(gpu, oracle):
    """Duplicate rows give exact zeros; integer data exact values."""
    rng = np.random.default_rng(3)
    X = rng.integers(0, 20, size=(500, 24)).astype(np.float32)
    X[10] = X[3]
    g = pairwise_distances(X, distance="sqeuclidean")
    assert g[10 * 9 // 2 + 3] == 0.0
    c = oracle.pairwise_distances(X, "sqeuclidean", "condensed", threads=threads())
    np.testing.assert_array_equal(g, c)
    s = pairwise_distances(X, distance="euclidean", form="square")
    np.testing.assert_array_equal(s, s.T)
    assert np.all(np.diag(s) == 0)
