"""Drop-in for ``fuel.cluster.kmeans`` (python/fuel/cluster/_kmeans.py:120-164)
running Lloyd's iteration on one GB300.

Served variants: every exact Lloyd-type variant of fuel ('lloyd',
'lloyd_naive', 'lloyd_blas' and the bound-accelerated 'elkan', 'simp_elkan',
'hamerly', 'simp_hamerly', 'exponion', 'shallot' and their aliases).  The
bound-based variants only skip distance computations that cannot change an
assignment, so they follow Lloyd's assignment sequence; on the GPU the plain
Lloyd pass is the fast path for all of them.  'hartigan_wong*', 'macqueen'
and 'kmedians' are different algorithms and raise NotImplementedError.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

_LLOYD_FAMILY = {
    "lloyd", "lloyd_blas", "lloyd_naive", "elkan", "s_elkan", "simp_elkan", "simplified_elkan", "hamerly",
    "s_hamerly", "simp_hamerly", "simplified_hamerly", "exponion", "shallot",
}
_OTHER = {"hartigan_wong", "hartigan_wong_quick", "macqueen", "kmedians"}
# variants whose reference result carries no inertia (KMeansResult::without_inertia:
# src/cluster/kmeans/elkan.rs:267, selkan.rs:223, hamerly.rs:270, shamerly.rs:234,
# exponion.rs:230, shallot.rs:297)
_WITHOUT_INERTIA = {
    "elkan", "s_elkan", "simp_elkan", "simplified_elkan", "hamerly", "s_hamerly", "simp_hamerly",
    "simplified_hamerly", "exponion", "shallot",
}


class KMeansResult:
    """python/fuel/cluster/_kmeans.py:5-34."""

    def __init__(self, centers, labels, n_iter, inertia, inertia_bound):
        self.centers = centers
        self.labels = labels
        self.n_iter = n_iter
        self.inertia = inertia
        self.inertia_bound = inertia_bound
        self.stats = None

    def __repr__(self):
        return (f"KMeansResult(centers={self.centers}, labels={self.labels}, n_iter={self.n_iter}, "
                f"inertia={self.inertia}, inertia_bound={self.inertia_bound})")


def _init_centers(data: np.ndarray, k: int, init, seed):
    """InitMethod::parse (python/kmeans.rs:101-134) for the methods served here."""
    n, d = data.shape
    if init is None:
        init = "random"
    if isinstance(init, str):
        if init == "first":
            if k > n:
                raise ValueError(f"k={k} exceeds the number of points n={n}")
            return np.ascontiguousarray(data[:k], np.float32)  # FirstK, init/first.rs:36-44
        if init == "random":
            # RandomSample draws k distinct rows (init/random.rs:33-41) from a Pcg32
            # stream; this engine draws them with numpy's default_rng(seed).
            if k > n:
                raise ValueError(f"k={k} exceeds the number of points n={n}")
            rows = np.random.default_rng(0 if seed is None else seed).choice(n, size=k, replace=False)
            return np.ascontiguousarray(data[rows], np.float32)
        if init in ("kmeans++", "kgeometric++"):
            raise NotImplementedError(f"init '{init}' seeding is not served by the GB300 engine; pass an array")
        raise ValueError(f"unknown initialization method '{init}', valid options are 'random', 'first', "
                         "'kmeans++', 'kgeometric++'")
    arr = np.asarray(init)
    if arr.ndim != 2:
        raise ValueError("init must be a string or a 2D numpy array")
    if arr.shape != (k, d):
        raise ValueError(f"init array must have shape (k, d) = ({k}, {d}), got ({arr.shape[0]}, {arr.shape[1]})")
    return np.ascontiguousarray(arr, np.float32)


def kmeans(data, *, k, variant="simp_elkan", max_iter=300, tol=0, seed=None, init=None, precision=None,
           order=None, fixed_iters=False):
    """K-means clustering (Euclidean space) on the GPU.

    Returns ``KMeansResult(centers float32[k, d], labels int64[n], n_iter,
    inertia, inertia_bound=None)``.  ``n_iter`` counts the initial assignment
    as iteration 1 (src/cluster/kmeans/util.rs:40).  ``inertia`` is the FP64
    sum of squared distances of the final pass, or None for the bound-based
    variants, whose reference results carry none (``stats["inertia_fp64"]``
    has it for every variant).  ``fixed_iters=True`` runs
    exactly ``max_iter`` iterations (benchmark mode).  ``precision`` (None /
    'auto' | 'fp32' | 'bf16' | 'split_bf16') picks the assignment tier; every
    tier gives the same result, and the default runs the split-BF16 tensor-core
    screen where it serves the shape (d >= 32, n >= 16384), the plain FP32
    scan otherwise.
    """
    v = str(variant).lower()
    if v in _OTHER:
        raise NotImplementedError(f"kmeans variant '{variant}' is not served by the GB300 engine")
    if v not in _LLOYD_FAMILY:
        raise ValueError(f"unknown kmeans variant '{variant}'. Valid: {sorted(_LLOYD_FAMILY | _OTHER)}")
    data = np.asarray(data)
    if data.dtype not in (np.float32, np.float64):
        data = data.astype(np.float64)
    if data.dtype != np.float32:
        raise NotImplementedError(
            f"data has dtype {data.dtype}; the GB300 engine serves float32 (cast with .astype(np.float32))")
    if data.ndim != 2:
        raise ValueError("data must be a 2D array")
    k = int(k)
    if k <= 0:
        raise ValueError("k must be positive")
    max_iter = int(max_iter)
    if tol is None:
        tol = 0.0
    order = order or _lib.default_order()
    X = np.ascontiguousarray(data)
    n, d = X.shape
    C0 = _init_centers(X, k, init, seed)
    precision = "auto" if precision is None else precision
    if precision not in _lib.PRECISION or precision == "fp16":
        raise ValueError("precision must be one of 'auto', 'fp32', 'bf16', 'split_bf16'")
    centers = np.empty((k, d), np.float32)
    labels = np.empty(n, np.int64)
    iters = ctypes.c_int32(0)
    inertia = ctypes.c_double(0.0)
    st = _lib.Stats()
    _lib.check(_lib.load().fuelg_kmeans_lloyd(
        _lib.ptr(X), n, d, k, _lib.ptr(C0), max(1, max_iter), float(tol), _lib.PRECISION[precision],
        _lib.ORDER[order], _lib.LLOYD_FIXED_ITERS if fixed_iters else 0, _lib.ptr(centers), _lib.ptr(labels),
        ctypes.byref(iters), ctypes.byref(inertia), ctypes.byref(st)))
    res = KMeansResult(centers, labels, int(iters.value),
                       None if v in _WITHOUT_INERTIA else float(inertia.value), None)
    res.stats = st.as_dict()
    res.stats["inertia_fp64"] = float(inertia.value)
    return res


def lloyd_assign(data, centers, *, initial=False, order=None):
    """One Lloyd assignment pass on the GPU: (labels int64[n], best float32[n]).

    Nearest centre per point with fuel's arithmetic (``initial=True``: the
    initial pass, src/cluster/kmeans/lloyd.rs:12-112; otherwise the
    iteration loop's math::sqdist, lloyd.rs:140-158), first index on ties.
    This is the local step of ``fuel_gb300.shard.sharded_lloyd``.
    """
    X = np.ascontiguousarray(data, np.float32)
    C = np.ascontiguousarray(centers, np.float32)
    if X.ndim != 2 or C.ndim != 2 or X.shape[1] != C.shape[1]:
        raise ValueError("data [n, d] and centers [k, d] must share d")
    n, d = X.shape
    labels = np.empty(n, np.int64)
    best = np.empty(n, np.float32)
    _lib.check(_lib.load().fuelg_lloyd_assign(_lib.ptr(X), n, d, _lib.ptr(C), C.shape[0], int(bool(initial)),
                                              _lib.ORDER[order or _lib.default_order()], _lib.ptr(labels),
                                              _lib.ptr(best), None))
    return labels, best


def kmeans_batched(problems, *, max_iter=300, order=None, fixed_iters=False, precision="auto"):
    """Many independent Lloyd k-means problems in one engine call.

    ``problems``: iterable of ``(data float32[n, d], init float32[k, d])``.
    Returns a list of ``KMeansResult`` -- each exactly what
    ``kmeans(data, k=k, variant="lloyd", init=init, max_iter=max_iter,
    fixed_iters=fixed_iters)`` returns for that problem.  All problems'
    points are assigned by one persistent kernel per iteration and the
    middle iterations run as one replayed CUDA graph.  ``precision``
    other than "fp32" screens problems with 32 <= d <= 64 and k <= 256 on
    the tensor cores (exact re-score where undecided; same results).
    """
    order = order or _lib.default_order()
    keep, descs, outs = [], [], []
    for data, init in problems:
        data = np.asarray(data)
        if data.dtype != np.float32:
            # kmeans() serves float32 data too; a silent cast would change the answer
            raise NotImplementedError(
                f"data has dtype {data.dtype}; the GB300 engine serves float32 (cast with .astype(np.float32))")
        X = np.ascontiguousarray(data, np.float32)
        C0 = np.ascontiguousarray(init, np.float32)
        if X.ndim != 2 or C0.ndim != 2 or X.shape[1] != C0.shape[1]:
            raise ValueError("each problem needs data [n, d] and init [k, d]")
        n, d = X.shape
        k = C0.shape[0]
        centers = np.empty((k, d), np.float32)
        labels = np.empty(n, np.int64)
        keep += [X, C0, centers, labels]
        descs.append(_lib.KMeansProblem(X.ctypes.data, n, d, k, C0.ctypes.data, centers.ctypes.data,
                                        labels.ctypes.data, 0, 0, 0.0))
        outs.append((centers, labels))
    arr = (_lib.KMeansProblem * len(descs))(*descs)
    st = _lib.Stats()
    _lib.check(_lib.load().fuelg_kmeans_batched(ctypes.cast(arr, ctypes.c_void_p), len(descs), max(1, int(max_iter)),
                                                _lib.ORDER[order], _lib.PRECISION[precision],
                                                _lib.LLOYD_FIXED_ITERS if fixed_iters else 0, ctypes.byref(st)))
    res = []
    for desc, (centers, labels) in zip(arr, outs):
        if desc.status != _lib.OK:
            raise NotImplementedError("a problem's data cannot be summed exactly (non-finite values or an exponent "
                                      "range beyond 128 bits)")
        r = KMeansResult(centers, labels, int(desc.out_iters), float(desc.out_inertia), None)
        res.append(r)
    kmeans_batched.last_stats = st.as_dict()
    return res
