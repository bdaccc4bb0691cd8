"""Self-checks of the oracle's restated heap / exclude-self / Lloyd logic
against independent brute force built from the oracle's per-pair distances."""
import numpy as np
import pytest

from conftest import threads


def brute_knn(oracle, X, Q, k, metric, order, mode):
    """Tie-inclusive KNNHeap semantics by brute force: kept = all keys with
    distance <= the k-th smallest; then exclude-self, truncate, pad."""
    m = Q.shape[0]
    idx = np.full((m, k), -1, np.int64)
    dist = np.full((m, k), np.inf, np.float32)
    for i in range(m):
        dv = np.array([oracle.dist("knn", order, Q[i], X[j]) for j in range(X.shape[0])], np.float32)
        if metric == "euclidean":
            dv = np.sqrt(dv).astype(np.float32)
        qk = k + 1 if mode == "kplus1" else k
        srt = np.lexsort((np.arange(len(dv)), dv))
        if qk == 0 or len(dv) == 0:
            kept = np.array([], np.int64)
        else:
            kth = dv[srt[min(qk, len(dv)) - 1]]
            kept = srt[dv[srt] <= kth]
        if mode != "none":
            kept = kept[kept != i]
        kept = kept[:k]
        idx[i, :len(kept)] = kept
        dist[i, :len(kept)] = dv[kept]
    return idx, dist


@pytest.mark.parametrize("mode", ["none", "linear", "kplus1"])
@pytest.mark.parametrize("metric", ["sqeuclidean", "euclidean"])
@pytest.mark.parametrize("order", ["arm", "x86"])
def test_heap_matches_bruteforce_with_ties(oracle, mode, metric, order):
    rng = np.random.default_rng(3)
    X = rng.integers(0, 3, size=(60, 5)).astype(np.float32)  # many exact ties and duplicates
    for k in (1, 2, 5, 59, 61):
        a = oracle.knn(X, X, k, metric=metric, order=order, exclude=mode)
        b = brute_knn(oracle, X, X, k, metric, order, mode)
        assert np.array_equal(a[0], b[0]), (k, mode)
        assert np.array_equal(a[1], b[1])


def test_linear_exclude_drops_to_k_minus_1_without_ties(oracle):
    X = np.array([[0.0], [1.0], [3.0], [7.0]], np.float32)
    idx, dist = oracle.knn(X, X, 2, exclude="linear")
    # self is within the 2 nearest, no tie at the 2nd distance: one real neighbour + pad
    assert idx.tolist() == [[1, -1], [0, -1], [1, -1], [2, -1]]
    assert np.isinf(dist[:, 1]).all()
    idx2, _ = oracle.knn(X, X, 2, exclude="kplus1")
    assert idx2.tolist() == [[1, 2], [0, 2], [1, 0], [2, 1]]


def test_thread_count_does_not_change_knn(oracle):
    rng = np.random.default_rng(5)
    X = rng.normal(size=(300, 9)).astype(np.float32)
    a = oracle.knn(X, X, 7, threads=1)
    b = oracle.knn(X, X, 7, threads=threads())
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("order", ["arm", "x86"])
def test_orders_agree_within_rounding(oracle, order):
    rng = np.random.default_rng(7)
    a = rng.normal(size=777).astype(np.float32)
    b = rng.normal(size=777).astype(np.float32)
    exact = float(((a.astype(np.float64) - b) ** 2).sum())
    for kind in ("knn", "sqdist", "pairwise"):
        v = float(oracle.dist(kind, order, a, b))
        assert abs(v - exact) <= 1e-5 * exact


def test_x86_and_arm_orders_differ_somewhere(oracle):
    """The two profiles are genuinely different summation orders."""
    rng = np.random.default_rng(11)
    diffs = 0
    for _ in range(200):
        a = rng.normal(size=100).astype(np.float32)
        b = rng.normal(size=100).astype(np.float32)
        diffs += oracle.dist("sqdist", "arm", a, b) != oracle.dist("sqdist", "x86", a, b)
    assert diffs > 0


def test_lloyd_reference_vs_fp64_sums(oracle):
    rng = np.random.default_rng(1)
    centers = rng.uniform(-10, 10, size=(5, 3))
    X = (centers[rng.integers(0, 5, 400)] + rng.normal(size=(400, 3))).astype(np.float32)
    init = X[:5].copy()
    c1, l1, it1, in1 = oracle.lloyd(X, 5, init, max_iter=100, threads=4)
    c2, l2, it2, in2 = oracle.lloyd(X, 5, init, max_iter=100, sums="fp64")
    assert np.array_equal(l1, l2) and it1 == it2
    assert abs(in1 - in2) <= 1e-4 * in2
    assert np.allclose(c1, c2, rtol=1e-5, atol=1e-5)
    # at convergence labels are the argmin under the reference sqdist order
    lab, _ = oracle.lloyd_assign(X, c1, initial=False)
    assert np.array_equal(lab, l1)
    assert abs(in2 - oracle.lloyd_inertia_fp64(X, c2, l2)) <= 1e-9 * in2


def test_lloyd_iteration_counting(oracle):
    X = np.array([[0.0], [0.1], [10.0], [10.1]], np.float32)
    init = np.array([[0.0], [10.0]], np.float32)
    _, lab, it, _ = oracle.lloyd(X, 2, init, max_iter=100)
    # iteration 1 assigns, iteration 2 finds no change -> stop (lloyd.rs:133-199)
    assert it == 2 and lab.tolist() == [0, 0, 1, 1]
    _, _, it1, _ = oracle.lloyd(X, 2, init, max_iter=1)
    assert it1 == 1


def test_lloyd_empty_cluster_keeps_center(oracle):
    X = np.array([[0.0], [1.0], [2.0]], np.float32)
    init = np.array([[1.0], [1.0], [50.0]], np.float32)  # duplicate centre 1 loses every tie
    c, lab, _, _ = oracle.lloyd(X, 3, init, max_iter=5, sums="fp64")
    assert (lab != 1).all()
    assert c[1, 0] == 1.0
