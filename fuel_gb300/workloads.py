"""Seeded synthetic inputs with the shapes and value distributions of the
benchmark configurations (the reference publishes no datasets for this path;
MNIST, used by examples/kmeans_mnist_runtime.py, is replaced by a sparse
0..255/255 matrix of the same size).

Each generator derives child seeds with numpy's SeedSequence so every
component (centres, memberships, noise, init rows) has its own stream.
"""
from __future__ import annotations

import numpy as np


def _children(seed: int, n: int):
    return [np.random.default_rng(s) for s in np.random.SeedSequence(seed).spawn(n)]


def gaussian_mixture(n: int, d: int, n_centers: int, box: float, sd: float, seed: int = 0) -> np.ndarray:
    """n points from an equal-weight isotropic mixture; centres ~ U[-box, box]^d."""
    r_c, r_m, r_x = _children(seed, 3)
    centers = r_c.uniform(-box, box, size=(n_centers, d))
    comp = r_m.integers(0, n_centers, size=n)
    x = centers[comp] + r_x.normal(0.0, sd, size=(n, d))
    return np.ascontiguousarray(x, dtype=np.float32)


def knn_plain(n: int = 20000, d: int = 16, seed: int = 0):
    """kNN self-join, plain: 6-component mixture, centres in [-5,5]^16, sd 0.5; k=10."""
    return gaussian_mixture(n, d, 6, 5.0, 0.5, seed)


def lloyd_sparse(n: int = 70000, d: int = 784, k: int = 64, seed: int = 0, init_seed: int = 1):
    """Lloyd k=64: coordinates 0 w.p. 0.8 else U{1..255}, scaled by 1/255; init = k distinct rows."""
    rng = np.random.default_rng(seed)
    nz = rng.random((n, d)) >= 0.8
    vals = rng.integers(1, 256, size=(n, d))
    x = np.where(nz, vals, 0).astype(np.float32) / np.float32(255.0)
    rows = np.random.default_rng(init_seed).choice(n, size=k, replace=False)
    return np.ascontiguousarray(x), np.ascontiguousarray(x[rows])


def knn_geometric(n: int = 1_000_000, d: int = 128, seed: int = 0) -> np.ndarray:
    """Integer-valued coordinates min(geometric(0.1) - 1, 255) as float32 (many exact ties)."""
    rng = np.random.default_rng(seed)
    x = np.minimum(rng.geometric(0.1, size=(n, d)) - 1, 255)
    return np.ascontiguousarray(x, dtype=np.float32)


def unit_normal_rows(n: int, d: int, seed: int = 0) -> np.ndarray:
    """Standard-normal rows normalised to unit length (serving index)."""
    x = np.random.default_rng(seed).standard_normal((n, d))
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    return np.ascontiguousarray(x, dtype=np.float32)


def batched_kmeans_problems(count: int = 512, seed: int = 0, n_range=(1000, 200000), dims=(2, 8, 32, 64),
                            k_range=(4, 256)):
    """Problem descriptors (n, d, k, seed) of the batched k-means workload."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]))))
        d = int(rng.choice(dims))
        k = int(np.exp(rng.uniform(np.log(k_range[0]), np.log(k_range[1]))))
        out.append((n, d, min(k, n), int(rng.integers(0, 2**31 - 1))))
    return out


def batched_kmeans_data(desc):
    """One problem of the batched workload: a Gaussian mixture with k centres
    uniform in [-10, 10]^d and sd 1 (equal weights), float32; init = the
    first k rows of a seeded permutation.  Returns (X [n, d], init [k, d])."""
    n, d, k, seed = desc
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-10.0, 10.0, size=(k, d))
    comp = rng.integers(0, k, size=n)
    X = (centres[comp] + rng.standard_normal((n, d))).astype(np.float32)
    init = X[rng.permutation(n)[:k]].copy()
    return np.ascontiguousarray(X), np.ascontiguousarray(init)
