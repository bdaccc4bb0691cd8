"""Host-side logic of the Python mirror of fuel.search / fuel.cluster.kmeans
that runs before any device call (validation, name parsing, init)."""
import numpy as np
import pytest

from fuel_gb300 import cluster, search


def test_tree_names():
    assert search._normalize_tree(None) == "auto"
    assert search._normalize_tree("brute_force") == "linear"
    assert search._normalize_tree("Brute-Force") == "linear"
    assert search._normalize_tree("balltree") == "cover"
    with pytest.raises(ValueError):
        search._normalize_tree("octree")
    with pytest.raises(TypeError):
        search._normalize_tree(3)


def test_distance_names():
    assert search._parse_distance("L2") == "euclidean"
    assert search._parse_distance("squared_euclidean") == "sqeuclidean"
    with pytest.raises(NotImplementedError):
        search._parse_distance("cosine")


def test_non_linear_trees_are_not_silently_served():
    X = np.zeros((4, 3), np.float32)
    with pytest.raises(NotImplementedError):
        search.SearchIndex(X, tree="vp")


def test_float64_is_not_silently_downcast():
    X = np.zeros((4, 3), np.float64)
    # float64 search runs the exact FP64 scan; the tensor-core tiers serve float32 data
    with pytest.raises(NotImplementedError):
        search.SearchIndex(X, tree="linear", precision="bf16")
    with pytest.raises(NotImplementedError):
        cluster.kmeans(X, k=2, variant="lloyd", init="first")


def test_batched_knn_refuses_float64_sets():
    X = np.zeros((4, 3), np.float64)
    with pytest.raises(NotImplementedError):
        search.knn_batched([(X, X, 2)])
    with pytest.raises(NotImplementedError):
        search.knn_batched([(X.astype(np.float32), X.astype(np.int32), 2)])


def test_batched_kmeans_refuses_non_float32_data():
    X = np.zeros((6, 3), np.float64)
    with pytest.raises(NotImplementedError):
        cluster.kmeans_batched([(X, X[:2])])


def test_integer_input_becomes_float64_like_reference():
    assert search._ensure_float(np.zeros((2, 2), np.int32)).dtype == np.float64


def test_kmeans_variants():
    X = np.zeros((4, 3), np.float32)
    with pytest.raises(NotImplementedError):
        cluster.kmeans(X, k=2, variant="macqueen")
    with pytest.raises(ValueError):
        cluster.kmeans(X, k=2, variant="nope")


def test_kmeans_init_parsing():
    X = np.arange(30, dtype=np.float32).reshape(10, 3)
    assert np.array_equal(cluster._init_centers(X, 3, "first", None), X[:3])
    r = cluster._init_centers(X, 4, "random", 5)
    assert r.shape == (4, 3) and len({tuple(v) for v in r}) == 4
    with pytest.raises(ValueError):
        cluster._init_centers(X, 3, np.zeros((2, 3)), None)
    with pytest.raises(NotImplementedError):
        cluster._init_centers(X, 3, "kmeans++", None)
    with pytest.raises(ValueError):
        cluster._init_centers(X, 3, "bogus", None)


def test_precision_names():
    from fuel_gb300 import _lib
    assert _lib.PRECISION["auto"] == -1 and _lib.PRECISION["fp32"] == 0
    X = np.zeros((4, 3), np.float32)
    with pytest.raises(ValueError):
        cluster.kmeans(X, k=2, variant="lloyd", init="first", precision="fp16")
    with pytest.raises(ValueError):
        cluster.kmeans(X, k=2, variant="lloyd", init="first", precision="tf32")
