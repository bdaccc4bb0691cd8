"""Batched k-means: every problem of one fuelg_kmeans_batched call equals
its own fuelg_kmeans_lloyd call bit for bit (centres, labels, iteration
count) and the exact-mean oracle on small problems; inertia within 1e-9
relative (FP64 sums in a different order)."""
import numpy as np
import pytest

from fuel_gb300 import kmeans, kmeans_batched, workloads


def _mixed(count, seed, n_max=20000, dims=(2, 3, 8, 17, 32, 40, 64, 100)):
    rng = np.random.default_rng(seed)
    descs = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(40), np.log(n_max))))
        d = int(rng.choice(dims))
        k = int(np.exp(rng.uniform(np.log(2), np.log(256))))
        descs.append((n, d, min(k, n), int(rng.integers(0, 2**31 - 1))))
    return [workloads.batched_kmeans_data(t) for t in descs]


def _same(a, b):
    np.testing.assert_array_equal(a.centers.view(np.uint32), b.centers.view(np.uint32))
    np.testing.assert_array_equal(a.labels, b.labels)
    assert a.n_iter == b.n_iter
    assert abs(a.inertia - b.inertia) <= 1e-9 * max(1.0, abs(b.inertia))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "split_bf16"])
@pytest.mark.parametrize("fixed", [False, True])
@pytest.mark.parametrize("order", ["arm", "x86"])
def test_batched_equals_single(gpu, fixed, order, precision):
    probs = _mixed(24, seed=5 + fixed)
    got = kmeans_batched(probs, max_iter=12, order=order, fixed_iters=fixed, precision=precision)
    for (X, init), g in zip(probs, got):
        ref = kmeans(X, k=init.shape[0], variant="lloyd", init=init, max_iter=12, order=order,
                     fixed_iters=fixed)
        _same(g, ref)


@pytest.mark.gpu
def test_batched_oracle_small(gpu, oracle):
    probs = _mixed(10, seed=11, n_max=3000, dims=(2, 8, 5, 32))
    got = kmeans_batched(probs, max_iter=15)
    for (X, init), g in zip(probs, got):
        rc, rl, rit, rinert = oracle.lloyd_exact(X, init.shape[0], init, max_iter=15)
        np.testing.assert_array_equal(g.centers.view(np.uint32), rc.view(np.uint32))
        np.testing.assert_array_equal(g.labels, rl)
        assert g.n_iter == rit
        assert abs(g.inertia - rinert) <= 1e-9 * max(1.0, abs(rinert))


@pytest.mark.gpu
@pytest.mark.parametrize("max_iter", [1, 2, 3, 7])
def test_batched_short_runs(gpu, max_iter):
    probs = _mixed(9, seed=max_iter, n_max=5000)
    got = kmeans_batched(probs, max_iter=max_iter, fixed_iters=True)
    for (X, init), g in zip(probs, got):
        ref = kmeans(X, k=init.shape[0], variant="lloyd", init=init, max_iter=max_iter, fixed_iters=True)
        _same(g, ref)


@pytest.mark.gpu
def test_batched_config_sample(gpu):
    """40 problems drawn like the 512-problem benchmark (n up to 200,000)."""
    descs = workloads.batched_kmeans_problems(count=40, seed=3)
    probs = [workloads.batched_kmeans_data(t) for t in descs]
    got = kmeans_batched(probs, max_iter=8, fixed_iters=True)
    for (X, init), g in zip(probs, got):
        ref = kmeans(X, k=init.shape[0], variant="lloyd", init=init, max_iter=8, fixed_iters=True)
        _same(g, ref)


@pytest.mark.gpu
def test_batched_change_list_overflow(gpu):
    """A pass in which most tensor-core rows change: the first update moves
    centre 0 away from the majority, which then moves to centre 1 (75% of
    the rows).  The change list holds half of the tensor-core rows, so the
    rest of the pass takes the screen epilogue's direct sums; the result must
    still equal the single-problem call and the exact-mean oracle."""
    from oracle import oracle
    rng = np.random.default_rng(21)
    n, d = 4096, 32
    X = rng.normal(scale=0.01, size=(n, d)).astype(np.float32)
    X[: 3 * n // 4, 0] += 0.0          # majority near x0 = 0
    X[3 * n // 4:, 0] += 100.0         # minority near x0 = 100
    init = np.zeros((2, d), np.float32)
    init[0, 0] = 1.0                   # pass 1: every row nearest centre 0
    init[1, 0] = -1.5                  # pass 2: centre 0 at ~25 -> the majority moves here
    small = workloads.batched_kmeans_data((300, 8, 3, 7))  # a CUDA-core problem alongside
    probs = [(X, init), small]
    got = kmeans_batched(probs, max_iter=6, fixed_iters=True, precision="split_bf16")
    ref = kmeans(X, k=2, variant="lloyd", init=init, max_iter=6, fixed_iters=True)
    _same(got[0], ref)
    rc, rl, rit, _ = oracle.lloyd_exact(X, 2, init, max_iter=6, fixed_iters=True)
    np.testing.assert_array_equal(got[0].centers.view(np.uint32), rc.view(np.uint32))
    np.testing.assert_array_equal(got[0].labels, rl)
    assert (rl == 1).sum() >= n // 2, "most rows must have moved to centre 1"
    rs = kmeans(small[0], k=small[1].shape[0], variant="lloyd", init=small[1], max_iter=6, fixed_iters=True)
    _same(got[1], rs)
