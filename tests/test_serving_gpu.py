"""kNN serving loop (continuous batching): every request's result equals the
same rows answered alone (bit-identical), whatever the mix it was batched
with; requests submitted together are merged into shared GPU batches."""
import threading

import numpy as np
import pytest

from fuel_gb300 import SearchIndex, workloads
from fuel_gb300.serving import Server


def _mix(rng, d, count, max_rows=300):
    out = []
    for _ in range(count):
        m = int(np.exp(rng.uniform(0, np.log(max_rows))))
        out.append((rng.standard_normal((m, d)).astype(np.float32), int(rng.choice([1, 10, 100]))))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16", "split_bf16", "fp16"])
def test_serving_results_equal_alone(gpu, precision):
    rng = np.random.default_rng(3)
    X = workloads.unit_normal_rows(60000, 96, seed=0)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear", precision=precision)
    reqs = _mix(rng, 96, 40)
    alone = [ix.knn(Q, k, exclude_self=False) for Q, k in reqs]
    with Server(ix, precision=precision, max_batch_queries=2048, workers=2) as sv:
        handles = [sv.submit(Q, k) for Q, k in reqs]
        got = [h.result() for h in handles]
        st = sv.stats()
    for (gi, gd), (ai, ad) in zip(got, alone):
        np.testing.assert_array_equal(gi, ai)
        np.testing.assert_array_equal(gd.view(np.uint32), ad.view(np.uint32))
    assert st["queries"] == sum(Q.shape[0] for Q, _ in reqs)
    assert st["max_batch_requests"] > 1  # submitted together -> merged
    assert all(h.latency_ms is not None and h.latency_ms >= 0 for h in handles)


@pytest.mark.gpu
def test_serving_mixed_k_integer_data(gpu):
    """Integer data (exact BF16 screen, no proof margin): one tensor-core
    launch per batch with every row selecting its own k matches each request
    answered alone."""
    rng = np.random.default_rng(5)
    X = workloads.knn_geometric(n=40000, d=64, seed=3)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear", precision="bf16")
    reqs = [(X[rng.integers(0, X.shape[0], size=int(m))].copy(), int(k))
            for m, k in zip(rng.integers(1, 200, size=24), rng.choice([1, 3, 10, 57, 100], size=24))]
    alone = [ix.knn(Q, k, exclude_self=False) for Q, k in reqs]
    with Server(ix, precision="bf16", max_batch_queries=4096, workers=1) as sv:
        got = [h.result() for h in [sv.submit(Q, k) for Q, k in reqs]]
        st = sv.stats()
    for (gi, gd), (ai, ad) in zip(got, alone):
        np.testing.assert_array_equal(gi, ai)
        np.testing.assert_array_equal(gd.view(np.uint32), ad.view(np.uint32))
    assert st["max_batch_requests"] > 1


@pytest.mark.gpu
def test_serving_concurrent_submitters_and_budget(gpu):
    """Several host threads submit at once under a budget that admits only a
    few requests at a time: all complete, each equal to its lone answer."""
    rng = np.random.default_rng(9)
    X = workloads.unit_normal_rows(30000, 96, seed=1)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear", precision="bf16")
    reqs = _mix(rng, 96, 48, max_rows=200)
    alone = [ix.knn(Q, k, exclude_self=False) for Q, k in reqs]
    results = [None] * len(reqs)
    with Server(ix, precision="bf16", max_batch_queries=1024, budget_bytes=3 << 20, workers=3) as sv:
        def client(lo):
            for i in range(lo, len(reqs), 4):
                results[i] = sv.submit(*reqs[i]).result()
        ts = [threading.Thread(target=client, args=(c,)) for c in range(4)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
    for (gi, gd), (ai, ad) in zip(results, alone):
        np.testing.assert_array_equal(gi, ai)
        np.testing.assert_array_equal(gd, ad)


@pytest.mark.gpu
def test_serving_rejects_oversize(gpu):
    X = workloads.unit_normal_rows(1000, 96, seed=2)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear")
    with Server(ix, precision="fp32", max_batch_queries=64, budget_bytes=1 << 30, workers=1) as sv:
        with pytest.raises(ValueError):
            sv.submit(np.zeros((65, 96), np.float32), 5)  # more rows than a batch
    with Server(ix, precision="fp32", max_batch_queries=4096, budget_bytes=1 << 16, workers=1) as sv:
        with pytest.raises(MemoryError):
            sv.submit(np.zeros((4000, 96), np.float32), 100)  # above the memory budget
