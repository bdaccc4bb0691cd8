"""Sharded exchange logic (fuel_gb300.shard): kNN candidate merge with fuel's
tie and exclude-self rules, range-result merge, and Lloyd with exact integer
centroid sums all-reduced across ranks.  Single-process merges are checked
against the oracle on the unsharded data; the collectives run as two gloo
ranks on CPU."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

from fuel_gb300 import shard

HERE = os.path.dirname(os.path.abspath(__file__))
MODES = {0: "none", 1: "linear", 2: "kplus1"}


def _split_knn(oracle, X, Q, k, mode, parts, qidx):
    cuts = np.linspace(0, len(X), parts + 1).astype(int)
    lists = []
    for a, b in zip(cuts[:-1], cuts[1:]):
        i, d = oracle.knn(X[a:b], Q, k + 1)
        lists.append((np.where(i >= 0, i + a, -1), d))
    return shard.merge_knn(lists, k, mode, qidx)


@pytest.mark.parametrize("parts", [1, 2, 3, 7])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_merge_knn_matches_unsharded(oracle, parts, mode):
    rng = np.random.default_rng(parts * 10 + mode)
    X = rng.integers(0, 3, size=(97, 4)).astype(np.float32)  # heavy ties and duplicates
    qidx = np.arange(len(X))
    for k in (1, 2, 5, 13):
        gi, gd = _split_knn(oracle, X, X, k, mode, parts, qidx)
        ri, rd = oracle.knn(X, X, k, exclude=MODES[mode])
        np.testing.assert_array_equal(gi, ri)
        np.testing.assert_array_equal(gd.view(np.uint32), rd.view(np.uint32))


def test_merge_knn_padding_when_k_exceeds_points(oracle):
    X = np.arange(12, dtype=np.float32).reshape(6, 2)
    for mode in (0, 1, 2):
        gi, gd = _split_knn(oracle, X, X, 9, mode, 4, np.arange(6))
        ri, rd = oracle.knn(X, X, 9, exclude=MODES[mode])
        np.testing.assert_array_equal(gi, ri)
        np.testing.assert_array_equal(gd, rd)


def test_merge_knn_foreign_queries(oracle):
    rng = np.random.default_rng(3)
    X = rng.normal(size=(200, 6)).astype(np.float32)
    Q = rng.normal(size=(31, 6)).astype(np.float32)
    gi, gd = _split_knn(oracle, X, Q, 8, 0, 5, None)
    ri, rd = oracle.knn(X, Q, 8)
    np.testing.assert_array_equal(gi, ri)
    np.testing.assert_array_equal(gd, rd)


def test_merge_knn_rejects_bad_mode():
    i = np.zeros((1, 3), np.int64)
    d = np.zeros((1, 3), np.float32)
    with pytest.raises(ValueError):
        shard.merge_knn([(i, d)], 2, 5, np.zeros(1, np.int64))
    with pytest.raises(ValueError):
        shard.merge_knn([(i, d)], 2, 1, None)


def test_merge_range_matches_unsharded(oracle):
    rng = np.random.default_rng(5)
    X = rng.integers(0, 4, size=(150, 3)).astype(np.float32)
    cuts = [0, 40, 41, 150]
    parts = []
    for a, b in zip(cuts[:-1], cuts[1:]):
        off, ii, dd = oracle.range_search(X[a:b], X, 3.0)
        parts.append((off, ii + a, dd))
    off, ii, dd = shard.merge_range(parts)
    ro, ri, rd = oracle.range_search(X, X, 3.0)
    np.testing.assert_array_equal(off, ro)
    np.testing.assert_array_equal(ii, ri)
    np.testing.assert_array_equal(dd, rd)


def test_shard_bounds_cover_rows():
    for n in (0, 1, 5, 17):
        for w in (1, 2, 3, 8):
            b = [shard.shard_bounds(n, w, r) for r in range(w)]
            assert b[0][0] == 0 and b[-1][1] == n
            assert all(b[r][1] == b[r + 1][0] for r in range(w - 1))
            assert max(h - lo for lo, h in b) - min(h - lo for lo, h in b) <= 1


def test_exact_sums_single_process_match_oracle(oracle):
    rng = np.random.default_rng(11)
    X = (rng.normal(size=(800, 9)) * np.exp2(rng.integers(-6, 6, size=(800, 1)))).astype(np.float32)
    init = X[:5].copy()
    assign = lambda A, C, initial: oracle.lloyd_assign(A, C, initial=initial)[0]  # noqa: E731
    C, lab, it, _, inert = shard.sharded_lloyd(X, 5, init, assign, max_iter=12)
    rc, rl, rit, rinert = oracle.lloyd_exact(X, 5, init, max_iter=12)
    np.testing.assert_array_equal(C.view(np.uint32), rc.view(np.uint32))
    np.testing.assert_array_equal(lab, rl)
    assert it == rit
    assert abs(inert - rinert) <= 1e-9 * abs(rinert)


def test_rne_ratio_matches_oracle(oracle):
    rng = np.random.default_rng(2)
    for _ in range(3000):
        S = int(rng.integers(-2**50, 2**50))
        cnt = int(rng.integers(1, 1 << 20))
        e = int(rng.integers(-60, 10))
        assert shard.rne_f32_ratio(S, cnt, e) == oracle.rn_f32_ratio(S, cnt, e)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


@pytest.fixture(scope="module")
def two_ranks(tmp_path_factory):
    """Runs tests/_shard_worker.py as two gloo ranks; returns their outputs."""
    out = str(tmp_path_factory.mktemp("shard") / "res")
    port = _free_port()
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", CUDA_VISIBLE_DEVICES="")
    procs = [subprocess.Popen([sys.executable, os.path.join(HERE, "_shard_worker.py"), str(r), "2", str(port), out],
                              env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT) for r in range(2)]
    logs = []
    for p in procs:
        try:
            logs.append(p.communicate(timeout=240)[0].decode(errors="replace"))
        except subprocess.TimeoutExpired:
            for q in procs:
                q.kill()
            pytest.fail("gloo ranks did not finish")
    for p, log in zip(procs, logs):
        assert p.returncode == 0, log[-2000:]
    return [dict(np.load(f"{out}.{r}.npz")) for r in range(2)]


def test_gloo_sharded_knn(oracle, two_ranks):
    sys.path.insert(0, HERE)
    import _shard_worker
    Xk, _, _ = _shard_worker.data()
    for k in (1, 4, 9):
        for mode in (0, 1, 2):
            ri, rd = oracle.knn(Xk, Xk, k, exclude=MODES[mode])
            for res in two_ranks:
                np.testing.assert_array_equal(res[f"knn_{k}_{mode}_i"], ri)
                np.testing.assert_array_equal(res[f"knn_{k}_{mode}_d"], rd)


def test_gloo_sharded_range(oracle, two_ranks):
    sys.path.insert(0, HERE)
    import _shard_worker
    Xk, _, _ = _shard_worker.data()
    ro, ri, rd = oracle.range_search(Xk, Xk, 2.0)
    for res in two_ranks:
        np.testing.assert_array_equal(res["range_off"], ro)
        np.testing.assert_array_equal(res["range_idx"], ri)
        np.testing.assert_array_equal(res["range_dist"], rd)


@pytest.mark.parametrize("fixed", [0, 1])
def test_gloo_sharded_lloyd_bit_identical(oracle, two_ranks, fixed):
    """Exact integer sums make the sharded centres bit-identical to the
    single-process exact-mean Lloyd; labels and iteration counts match."""
    sys.path.insert(0, HERE)
    import _shard_worker
    _, Xl, init = _shard_worker.data()
    rc, rl, rit, rinert = oracle.lloyd_exact(Xl, 6, init, max_iter=25, fixed_iters=bool(fixed))
    labels = np.zeros(len(Xl), np.int64)
    for res in two_ranks:
        np.testing.assert_array_equal(res[f"lloyd_{fixed}_C"].view(np.uint32), rc.view(np.uint32))
        it, _, lo, hi = res[f"lloyd_{fixed}_meta"]
        assert it == rit
        labels[lo:hi] = res[f"lloyd_{fixed}_lab"]
        assert abs(float(res[f"lloyd_{fixed}_inertia"][0]) - rinert) <= 1e-9 * abs(rinert)
    np.testing.assert_array_equal(labels, rl)
