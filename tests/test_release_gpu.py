"""fuelg_release: the state the engine keeps between calls (memory pool, the
Lloyd loop's CUDA graphs kept per host thread, the cancellation word) is freed,
and the next call sets it up again with bit-identical results -- also for graphs
kept by other threads, alive or exited."""
import threading

import numpy as np
import pytest

from fuel_gb300 import SearchIndex, _lib, kmeans
from fuel_gb300.serving import Server

pytestmark = pytest.mark.gpu


def mixture(n, d, k, seed):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-10, 10, size=(k, d))
    return (c[rng.integers(0, k, n)] + rng.normal(size=(n, d))).astype(np.float32)


def lloyd(X, init, precision):
    # 30 fixed passes: the middle ones replay the kept 8-pass and 1-pass graphs
    return kmeans(X, k=init.shape[0], variant="lloyd", max_iter=30, init=init, precision=precision,
                  fixed_iters=True)


def same(a, b):
    return (a.n_iter == b.n_iter and np.array_equal(a.labels, b.labels)
            and np.array_equal(a.centers.view(np.uint32), b.centers.view(np.uint32)))


@pytest.mark.parametrize("precision", ["fp32", "split_bf16"])
def test_release_between_calls(gpu, precision):
    X = mixture(20000, 64, 32, 3)
    init = X[:32].copy()
    a = lloyd(X, init, precision)
    b = lloyd(X, init, precision)  # kept graphs updated in place
    _lib.release()
    c = lloyd(X, init, precision)  # pool, graphs and cancel word made again
    _lib.release()
    _lib.release()  # nothing kept: a no-op
    d = lloyd(X, init, precision)
    assert same(a, b) and same(a, c) and same(a, d)


def test_release_with_graphs_of_other_threads(gpu):
    X = mixture(20000, 64, 24, 4)
    init = X[:24].copy()
    ref = lloyd(X, init, "split_bf16")
    out, first_done, go = {}, threading.Event(), threading.Event()

    def alive():
        out["a"] = lloyd(X, init, "split_bf16")
        first_done.set()
        go.wait(120)
        out["b"] = lloyd(X, init, "split_bf16")  # its handles were destroyed: forgotten and made again

    t = threading.Thread(target=alive)
    t.start()
    assert first_done.wait(120)
    _lib.release()
    go.set()
    t.join(120)
    # a thread that exits destroys the graphs it keeps
    t2 = threading.Thread(target=lambda: out.__setitem__("c", lloyd(X, init, "split_bf16")))
    t2.start()
    t2.join(120)
    _lib.release()
    out["d"] = lloyd(X, init, "split_bf16")
    assert sorted(out) == ["a", "b", "c", "d"]
    for key in "abcd":
        assert same(ref, out[key]), key


def test_release_keeps_indexes_and_refuses_open_server(gpu, lib):
    X = mixture(30000, 32, 16, 5)
    Q = X[:500]
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear")
    i0, d0 = ix.knn(Q, 10, exclude_self=False)
    _lib.release()
    assert lib.fuelg_cancel() == _lib.OK  # no cancellation word until the next call: a no-op
    i1, d1 = ix.knn(Q, 10, exclude_self=False)
    assert np.array_equal(i0, i1) and np.array_equal(d0.view(np.uint32), d1.view(np.uint32))
    with Server(ix, precision="fp32", workers=1) as sv:
        with pytest.raises(ValueError, match="serving handle"):
            _lib.release()
        i2, d2 = sv.submit(Q, 10).result()
    _lib.release()
    assert np.array_equal(i0, i2) and np.array_equal(d0.view(np.uint32), d2.view(np.uint32))
    i3, d3 = ix.knn(Q, 10, exclude_self=False)
    assert np.array_equal(i0, i3) and np.array_equal(d0.view(np.uint32), d3.view(np.uint32))
