"""Parity of the GPU linear-scan kNN with the restated fuel CPU path.

Bar: bit-exact.  Indices must be identical and the f32 distances identical to
the last bit, because the GPU forms every distance in fuel's own summation
order (profile 'arm' or 'x86') and orders keys exactly as DistPair does.
"""
import ctypes
import threading
import time

import numpy as np
import pytest

from conftest import f32_bits, threads
from fuel_gb300 import SearchIndex, _lib, knn_search, workloads

pytestmark = pytest.mark.gpu


def gpu_knn(X, Q, k, metric="sqeuclidean", order="arm", mode="none", precision="fp32"):
    idx = SearchIndex(X, distance=metric, tree="linear", order=order, precision=precision)
    excl = {"none": False, "linear": True, "kplus1": True}[mode]
    if mode == "kplus1":
        idx.precompute = 1  # the k+1 exclude rule of the precomputed path
    if excl:
        return idx.knn(X, k, exclude_self=True)
    return idx.knn(Q, k, exclude_self=False)


def assert_same(a, b):
    assert a[0].shape == b[0].shape
    bad = np.nonzero((a[0] != b[0]).any(1))[0]
    assert len(bad) == 0, f"{len(bad)} rows differ, first {bad[:5]}: gpu={a[0][bad[0]]} cpu={b[0][bad[0]]}"
    assert np.array_equal(f32_bits(a[1]), f32_bits(b[1]))


DIMS = [1, 2, 3, 4, 7, 8, 9, 15, 16, 17, 31, 32, 33, 64, 100, 128, 784]


@pytest.mark.parametrize("d", DIMS)
@pytest.mark.parametrize("order", ["arm", "x86"])
def test_knn_dims_orders(gpu, oracle, d, order):
    rng = np.random.default_rng(d)
    n = 700 if d < 200 else 300
    X = rng.normal(size=(n, d)).astype(np.float32)
    Q = rng.normal(size=(129, d)).astype(np.float32)
    for k in (1, 10):
        g = gpu_knn(X, Q, k, order=order)
        c = oracle.knn(X, Q, k, order=order, threads=threads())
        assert_same(g, c)


@pytest.mark.parametrize("metric", ["sqeuclidean", "euclidean"])
@pytest.mark.parametrize("mode", ["none", "linear", "kplus1"])
def test_knn_ties_and_exclude(gpu, oracle, metric, mode):
    rng = np.random.default_rng(42)
    X = rng.integers(0, 3, size=(1500, 6)).astype(np.float32)  # many exact ties, duplicates
    for k in (1, 2, 5, 33, 100):
        if mode == "none":
            g = gpu_knn(X, X, k, metric=metric, mode=mode)
        else:
            g = gpu_knn(X, X, k, metric=metric, mode=mode)
        c = oracle.knn(X, X, k, metric=metric, exclude=mode, threads=threads())
        assert_same(g, c)


@pytest.mark.parametrize("order", ["arm", "x86"])
def test_knn_plain_config_full(gpu, oracle, order):
    """n=20,000, d=16, 6-Gaussian mixture, k=10, queries = data (self-join)."""
    X = workloads.knn_plain()
    idx = SearchIndex(X, distance="sqeuclidean", tree="linear", order=order)
    g = idx.knn(X, 10)  # same source -> exclude_self (linear-scan rule)
    c = oracle.knn(X, X, 10, metric="sqeuclidean", order=order, exclude="linear", threads=threads())
    assert_same(g, c)
    assert idx.last_stats["kernel_launches"] >= 1


def test_knn_geometric_integer_data(gpu, oracle):
    """Integer-valued geometric coordinates (d=128, k=100): exact FP32, many ties."""
    X = workloads.knn_geometric(n=3000)
    g = gpu_knn(X, X[:200], 100)
    c = oracle.knn(X, X[:200], 100, threads=threads())
    assert_same(g, c)


def test_knn_edge_shapes(gpu, oracle):
    rng = np.random.default_rng(0)
    X = rng.normal(size=(5, 3)).astype(np.float32)
    # k > n pads with -1 / inf
    g = gpu_knn(X, X[:2], 8)
    c = oracle.knn(X, X[:2], 8)
    assert_same(g, c)
    assert (g[0][:, 5:] == -1).all() and np.isinf(g[1][:, 5:]).all()
    # k = 0 and m = 0
    ix = SearchIndex(X, tree="linear")
    i0, d0 = ix.knn(X[:3], 0, exclude_self=False)
    assert i0.shape == (3, 0) and d0.shape == (3, 0)
    i1, d1 = ix.knn(np.zeros((0, 3), np.float32), 4)
    assert i1.shape == (0, 4)
    # a single point; exclude-self leaves only padding
    one = np.ones((1, 3), np.float32)
    i2, d2 = SearchIndex(one, tree="linear").knn(one, 1)
    assert i2.tolist() == [[-1]]
    # empty index
    empty = SearchIndex(np.zeros((0, 3), np.float32), tree="linear")
    i3, d3 = empty.knn(X[:2], 2, exclude_self=False)
    assert (i3 == -1).all() and np.isinf(d3).all()


def test_knn_device_pointers_match_host(gpu, oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    X = rng.normal(size=(2000, 24)).astype(np.float32)
    Q = rng.normal(size=(300, 24)).astype(np.float32)
    lib = _lib.load()
    h = ctypes.c_void_p()
    _lib.check(lib.fuelg_index_create(_lib.ptr(X), 2000, 24, 0, 0, ctypes.byref(h)))
    try:
        Qd = torch.from_numpy(Q).cuda()
        oi = torch.empty((300, 7), dtype=torch.int64, device="cuda")
        od = torch.empty((300, 7), dtype=torch.float32, device="cuda")
        st = _lib.Stats()
        _lib.check(lib.fuelg_knn(h, _lib.ptr(Qd), 300, 7, 0, 0, _lib.ptr(oi), _lib.ptr(od), ctypes.byref(st)))
        assert st.h2d_bytes == 0 and st.d2h_bytes == 0
        c = oracle.knn(X, Q, 7)
        assert_same((oi.cpu().numpy(), od.cpu().numpy()), c)
    finally:
        lib.fuelg_index_destroy(h)


def test_knn_search_function(gpu, oracle):
    rng = np.random.default_rng(1)
    X = rng.normal(size=(400, 40)).astype(np.float32)
    g = knn_search(X, X, 5, distance="euclidean", tree="linear")
    c = oracle.knn(X, X, 5, metric="euclidean", exclude="linear")
    assert_same(g, c)


def test_knn_deterministic_reruns(gpu):
    X = workloads.knn_plain(n=5000)
    ix = SearchIndex(X, tree="linear", distance="sqeuclidean")
    a = ix.knn(X, 10)
    b = ix.knn(X, 10)
    assert np.array_equal(a[0], b[0]) and np.array_equal(f32_bits(a[1]), f32_bits(b[1]))


def test_cancel_from_another_thread(gpu):
    """Host-injected cancellation: a long scan stops and raises KeyboardInterrupt."""
    rng = np.random.default_rng(2)
    X = rng.normal(size=(1_500_000, 16)).astype(np.float32)
    ix = SearchIndex(X, tree="linear", distance="sqeuclidean")
    lib = _lib.load()

    def fire():
        time.sleep(0.3)
        lib.fuelg_cancel()

    t = threading.Thread(target=fire)
    t.start()
    with pytest.raises(KeyboardInterrupt):
        ix.knn(X, 10)  # 2.25e12 distances: seconds of work, cancelled long before the end
    t.join()
    # the next call starts with a cleared cancel word and succeeds
    i, d = ix.knn(X[:10], 3, exclude_self=False)
    assert (i[:, 0] == np.arange(10)).all()


# ---------------------------------------------------------------------------
# Tensor-core tier (tcgen05 BF16 screen): same bar -- bit-exact vs the oracle.
# Integer data below 2^24 takes the exact path (no re-score); other data is
# re-scored in the reference order and proven; failures fall back to the scan.
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("d", [32, 64, 100, 128, 256])
@pytest.mark.parametrize("order", ["arm", "x86"])
@pytest.mark.parametrize("metric", ["sqeuclidean", "euclidean"])
def test_knn_tc_general_data(gpu, oracle, d, order, metric):
    rng = np.random.default_rng(d + 7)
    X = rng.normal(size=(3000, d)).astype(np.float32)
    Q = rng.normal(size=(300, d)).astype(np.float32)
    for k in (1, 10, 64):
        g = gpu_knn(X, Q, k, metric=metric, order=order, precision="bf16")
        c = oracle.knn(X, Q, k, metric=metric, order=order, threads=threads())
        assert_same(g, c)


@pytest.mark.parametrize("mode", ["none", "linear", "kplus1"])
@pytest.mark.parametrize("metric", ["sqeuclidean", "euclidean"])
def test_knn_tc_integer_ties(gpu, oracle, mode, metric):
    X = workloads.knn_geometric(n=4000, d=128)
    for k in (1, 10, 100):
        g = gpu_knn(X, X, k, metric=metric, mode=mode, precision="bf16")
        c = oracle.knn(X, X, k, metric=metric, exclude=mode, threads=threads())
        assert_same(g, c)


def test_knn_tc_geometric_config_reduced(gpu, oracle):
    """n=50,000 integer geometric rows (d=128), k=100, 2,000 query rows."""
    X = workloads.knn_geometric(n=50_000)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear", precision="bf16")
    g = ix.knn(X[:2000], 100, exclude_self=False)
    assert ix.last_stats["precision_used"] == 1
    c = oracle.knn(X, X[:2000], 100, threads=threads())
    assert_same(g, c)


def test_knn_tc_small_shapes(gpu, oracle):
    rng = np.random.default_rng(5)
    for n, m, d in ((1, 1, 32), (5, 3, 40), (257, 129, 33), (300, 1, 64)):
        X = rng.normal(size=(n, d)).astype(np.float32)
        Q = rng.normal(size=(m, d)).astype(np.float32)
        for k in (1, 3, 8):
            g = gpu_knn(X, Q, k, precision="bf16")
            c = oracle.knn(X, Q, k)
            assert_same(g, c)


@pytest.mark.parametrize("k", [100, 200, 228, 229, 600])
def test_knn_tc_large_k(gpu, oracle, k):
    """Large k: many selections per query up to the tensor-core tier's limit
    (k + max(8, k // 8) <= 256 kept keys per column half, i.e. k <= 228);
    above it the
    exact scan answers.  Same bar either way."""
    rng = np.random.default_rng(k)
    X = rng.normal(size=(6000, 48)).astype(np.float32)
    Q = rng.normal(size=(150, 48)).astype(np.float32)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear", precision="bf16")
    g = ix.knn(Q, k, exclude_self=False)
    assert ix.last_stats["precision_used"] == (1 if k <= 228 else 0)
    assert_same(g, oracle.knn(X, Q, k, threads=threads()))
    Xi = workloads.knn_geometric(n=3000, d=64)
    g = gpu_knn(Xi, Xi, k, mode="linear", precision="bf16")
    c = oracle.knn(Xi, Xi, k, exclude="linear", threads=threads())
    assert_same(g, c)


@pytest.mark.parametrize("d", [32, 64, 96, 128])
@pytest.mark.parametrize("metric", ["sqeuclidean", "euclidean"])
def test_knn_tc_split_general_data(gpu, oracle, d, metric):
    """Split-BF16 (hi + lo) screen: bit-exact like every tier."""
    rng = np.random.default_rng(d + 101)
    X = rng.normal(size=(4000, d)).astype(np.float32)
    Q = rng.normal(size=(257, d)).astype(np.float32)
    ix = SearchIndex(X, distance=metric, tree="linear", precision="split_bf16")
    for k in (1, 10, 100):
        g = ix.knn(Q, k, exclude_self=False)
        assert ix.last_stats["precision_used"] == 2
        assert_same(g, oracle.knn(X, Q, k, metric=metric, threads=threads()))


def test_knn_tc_split_unit_rows_certified(gpu, oracle):
    """Unit-norm rows (d=96, the serving data): the split screen's error bound
    is small enough that nearly every query is certified without the exact
    rescan; results bit-exact."""
    X = workloads.unit_normal_rows(60000, 96, seed=0)
    Q = workloads.unit_normal_rows(300, 96, seed=5)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear", precision="split_bf16")
    g = ix.knn(Q, 100, exclude_self=False)
    st = ix.last_stats
    assert st["precision_used"] == 2
    kk2 = 100 + 12
    redo = (st["rescored"] - 300 * kk2) / X.shape[0]
    assert redo <= 0.02 * 300, f"{redo} of 300 queries needed the exact rescan"
    assert_same(g, oracle.knn(X, Q, 100, threads=threads()))


@pytest.mark.parametrize("d", [32, 96, 128])
@pytest.mark.parametrize("metric", ["sqeuclidean", "euclidean"])
@pytest.mark.parametrize("order", ["arm", "x86"])
def test_knn_tc_fp16_general_data(gpu, oracle, d, metric, order):
    """FP16 screen (one product, wider proof margin): bit-exact like every tier."""
    rng = np.random.default_rng(d + 303)
    X = rng.normal(size=(4000, d)).astype(np.float32)
    Q = rng.normal(size=(257, d)).astype(np.float32)
    ix = SearchIndex(X, distance=metric, tree="linear", precision="fp16", order=order)
    for k in (1, 10, 100):
        g = ix.knn(Q, k, exclude_self=False)
        assert ix.last_stats["precision_used"] == 4
        assert_same(g, oracle.knn(X, Q, k, metric=metric, order=order, threads=threads()))


def test_knn_tc_fp16_unit_rows_certified(gpu, oracle):
    """Unit-norm rows (d=96): the FP16 screen with its margin certifies nearly
    every query without the exact rescan; results bit-exact."""
    X = workloads.unit_normal_rows(60000, 96, seed=0)
    Q = workloads.unit_normal_rows(300, 96, seed=5)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear", precision="fp16")
    for k, kk2 in ((1, 9), (10, 18), (100, 125)):
        g = ix.knn(Q, k, exclude_self=False)
        st = ix.last_stats
        assert st["precision_used"] == 4
        redo = (st["rescored"] - 300 * kk2) / X.shape[0]
        assert redo <= 0.02 * 300, f"k={k}: {redo} of 300 queries needed the exact rescan"
        assert_same(g, oracle.knn(X, Q, k, threads=threads()))


def test_knn_tc_fp16_tiny_and_integer_values(gpu, oracle):
    """Values in the FP16 subnormal range (absolute rounding term of the bound)
    and integer data (exact one-product screen) stay bit-exact."""
    rng = np.random.default_rng(17)
    X = (rng.normal(size=(3000, 64)) * 1e-5).astype(np.float32)
    Q = (rng.normal(size=(200, 64)) * 1e-5).astype(np.float32)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear", precision="fp16")
    for k in (1, 10):
        assert_same(ix.knn(Q, k, exclude_self=False), oracle.knn(X, Q, k, threads=threads()))
        assert ix.last_stats["precision_used"] == 4
    Xi = workloads.knn_geometric(n=5000, d=128)
    g = gpu_knn(Xi, Xi, 50, mode="linear", precision="fp16")
    assert_same(g, oracle.knn(Xi, Xi, 50, exclude="linear", threads=threads()))


def test_knn_tc_fp16_out_of_range_uses_plain_tier(gpu, oracle):
    """Values beyond the FP16 range: the plain FP32 tier answers (same bar)."""
    rng = np.random.default_rng(23)
    X = rng.normal(size=(2000, 48)).astype(np.float32)
    X[7, 3] = 1e6
    Q = rng.normal(size=(100, 48)).astype(np.float32)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear", precision="fp16")
    g = ix.knn(Q, 10, exclude_self=False)
    assert ix.last_stats["precision_used"] == 0
    assert_same(g, oracle.knn(X, Q, 10, threads=threads()))
    ix2 = SearchIndex(Q, distance="sqeuclidean", tree="linear", precision="fp16")
    Qbig = X[:20].copy()  # one query row holds 1e6
    g2 = ix2.knn(Qbig, 5, exclude_self=False)
    assert ix2.last_stats["precision_used"] == 0
    assert_same(g2, oracle.knn(Q, Qbig, 5, threads=threads()))


# ---------------------------------------------------------------------------
# Work decomposition of the tensor-core scan: whole waves of query blocks run
# one CTA per block; a batch of less than a wave cuts each block's index scan
# into equal tile ranges whose kept lists are merged.  Results must not depend
# on the cut.
# ---------------------------------------------------------------------------
def test_knn_tc_multiwave_with_split_tail(gpu, oracle):
    """40,000 queries = 313 blocks: one whole wave (304 blocks) plus a 9-block
    tail whose 32-tile scans are cut in two and merged."""
    rng = np.random.default_rng(41)
    X = rng.normal(size=(4096, 32)).astype(np.float32)
    Q = rng.normal(size=(40_000, 32)).astype(np.float32)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear", precision="bf16")
    g = ix.knn(Q, 10, exclude_self=False)
    assert ix.last_stats["precision_used"] == 1
    assert_same(g, oracle.knn(X, Q, 10, threads=threads()))


@pytest.mark.parametrize("precision", ["bf16", "fp16", "split_bf16"])
def test_knn_tc_quanta_invariance(gpu, oracle, monkeypatch, precision):
    """Forcing 1, 2, 5, 9 or 37 tile ranges per query block gives the same
    keys as the default cut and as the oracle (one piece per block, pieces
    merged across CTAs, a CTA holding pieces of several blocks)."""
    rng = np.random.default_rng(43)
    X = rng.normal(size=(20_000, 64)).astype(np.float32)
    Q = rng.normal(size=(1000, 64)).astype(np.float32)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear", precision=precision)
    want = {k: oracle.knn(X, Q, k, threads=threads()) for k in (1, 50)}
    for k in (1, 50):
        assert_same(ix.knn(Q, k, exclude_self=False), want[k])
    for s in ("1", "2", "5", "9", "37"):
        monkeypatch.setenv("FUELG_KNN_QUANTA", s)
        for k in (1, 50):
            assert_same(ix.knn(Q, k, exclude_self=False), want[k])
    monkeypatch.delenv("FUELG_KNN_QUANTA")
