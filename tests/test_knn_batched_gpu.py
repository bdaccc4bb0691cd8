"""Many independent kNN query sets in one call (fuelg_knn_batched).

Each set -- its own data, n, d, k, metric and exclude rule -- must get exactly
what fuelg_knn returns on a linear index of its data (plain FP32 tier) and what
the oracle returns: indices and f32 distance bits, for sets of uneven shape in
the same call, including an empty index, k > n and the three exclude rules."""
import numpy as np
import pytest

from conftest import f32_bits, threads
import fuel_gb300
from fuel_gb300 import SearchIndex

pytestmark = pytest.mark.gpu


def _sets(rng):
    out = []
    shapes = [(3000, 16, 900, 10), (500, 3, 500, 7), (12000, 64, 300, 40), (700, 129, 700, 1),
              (2000, 8, 50, 100), (40, 5, 40, 60), (0, 12, 30, 4), (5000, 200, 64, 25), (1, 2, 9, 3)]
    metrics = ["sqeuclidean", "euclidean"]
    excludes = ["none", "linear", "kplus1"]
    for j, (n, d, m, k) in enumerate(shapes):
        if j % 3 == 1:  # tie-heavy integer data
            X = rng.integers(0, 3, size=(n, d)).astype(np.float32)
        else:
            X = rng.normal(size=(n, d)).astype(np.float32)
        ex = excludes[j % 3] if m <= n else "none"
        Q = X[:m].copy() if ex != "none" else rng.normal(size=(m, d)).astype(np.float32)
        out.append((X, Q, k, {"distance": metrics[j % 2], "exclude": ex}))
    return out


def test_batched_sets_match_single_calls_and_oracle(gpu, oracle):
    rng = np.random.default_rng(17)
    sets = _sets(rng)
    res = fuel_gb300.knn_batched(sets)
    assert len(res) == len(sets)
    for (X, Q, k, opt), (gi, gd) in zip(sets, res):
        ci, cd = oracle.knn(X, Q, k, metric=opt["distance"], exclude=opt["exclude"], threads=threads()) \
            if X.shape[0] else (np.full((Q.shape[0], k), -1, np.int64), np.full((Q.shape[0], k), np.inf, np.float32))
        assert np.array_equal(gi, ci), (X.shape, k, opt)
        assert np.array_equal(f32_bits(gd), f32_bits(cd)), (X.shape, k, opt)
        if X.shape[0] and opt["exclude"] != "kplus1":
            ix = SearchIndex(X, distance=opt["distance"], tree="linear", precision="fp32")
            si, sd = ix.knn(Q, k, exclude_self=False) if opt["exclude"] == "none" else ix.knn(X, k)
            if opt["exclude"] == "linear":
                si, sd = si[:Q.shape[0]], sd[:Q.shape[0]]
            assert np.array_equal(gi, si) and np.array_equal(f32_bits(gd), f32_bits(sd))
    assert fuel_gb300.knn_batched.last_stats["kernel_launches"] <= 4


def test_batched_rejects_bad_sets(gpu):
    X = np.zeros((10, 4), np.float32)
    with pytest.raises(ValueError):
        fuel_gb300.knn_batched([(X, X, 3, {"exclude": "sideways"})])
    with pytest.raises(ValueError):
        fuel_gb300.knn_batched([(X, np.zeros((3, 5), np.float32), 3)])
    assert fuel_gb300.knn_batched([]) == []
