"""Automatic precision tier (FUELG_PREC_AUTO, the Python default).

fuel's own keyword arguments (SearchIndex(data, distance=..., tree=...),
kmeans(data, k=..., variant=...)) must reach the tensor-core tiers where they
serve the shape, and the answer must stay the exact reference answer: the
tier choice only changes speed."""
import os

import numpy as np
import pytest

from conftest import f32_bits, threads
from fuel_gb300 import SearchIndex, kmeans

pytestmark = pytest.mark.gpu


def _same(g, c):
    assert np.array_equal(g[0], c[0]) and np.array_equal(f32_bits(g[1]), f32_bits(c[1]))


def test_auto_knn_integer_data_takes_the_exact_bf16_screen(gpu, oracle):
    rng = np.random.default_rng(1)
    X = np.minimum(rng.geometric(0.2, size=(5000, 64)) - 1, 255).astype(np.float32)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear")
    g = ix.knn(X[:700], 10)  # not the same array: no exclude
    assert ix.last_stats["precision_used"] == 1
    _same(g, oracle.knn(X, X[:700], 10, threads=threads()))


def test_auto_knn_real_data_is_timed_and_cached(gpu, oracle, tmp_path, monkeypatch):
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("FUELG_TUNE_CACHE", str(cache))
    rng = np.random.default_rng(2)
    X = rng.normal(size=(6000, 72)).astype(np.float32)
    X /= np.linalg.norm(X, axis=1, keepdims=True)
    Q = rng.normal(size=(900, 72)).astype(np.float32)
    ix = SearchIndex(X, distance="euclidean", tree="linear")
    g = ix.knn(Q, 7)
    tier = ix.last_stats["precision_used"]
    assert tier in (1, 2, 4), "a tensor-core tier serves d=72"
    _same(g, oracle.knn(X, Q, 7, metric="euclidean", threads=threads()))
    lines = [ln.split() for ln in cache.read_text().splitlines()]
    assert any(ln[0] == "knn" and ln[1] == "72" for ln in lines), "the bucket decision is written to the cache"
    g2 = ix.knn(Q[:300], 6)  # same (d, n, k) bucket: the cached tier runs
    assert ix.last_stats["precision_used"] == tier
    _same(g2, oracle.knn(X, Q[:300], 6, metric="euclidean", threads=threads()))


def test_auto_knn_small_d_is_plain(gpu, oracle):
    rng = np.random.default_rng(3)
    X = rng.normal(size=(3000, 16)).astype(np.float32)
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear")
    g = ix.knn(X, 5)
    assert ix.last_stats["precision_used"] == 0
    _same(g, oracle.knn(X, X, 5, exclude="linear", threads=threads()))


def test_auto_kmeans_picks_the_screen_for_large_problems(gpu, oracle):
    rng = np.random.default_rng(4)
    X = rng.normal(size=(20000, 40)).astype(np.float32)
    init = X[:12].copy()
    r = kmeans(X, k=12, variant="lloyd", max_iter=4, init=init, fixed_iters=True)
    assert r.stats["precision_used"] in (2, 3)
    rc, rl, _, _ = oracle.lloyd_exact(X, 12, init, max_iter=4, fixed_iters=True, threads=threads())
    assert np.array_equal(r.labels, rl) and np.array_equal(f32_bits(r.centers), f32_bits(rc))
    small = kmeans(X[:3000], k=12, variant="lloyd", max_iter=4, init=init, fixed_iters=True)
    assert small.stats["precision_used"] == 0
