"""Drop-in for fuel's linear-scan search API on one GB300.

Mirrors ``fuel.search`` (python/fuel/search.py:205-408): ``SearchIndex``,
``knn_search`` and ``range_search`` keep their names, keyword arguments,
validation, return types and exclude-self rules.  The scan itself runs in
libfuelg.so; distances are bit-identical to fuel's f32 distances for the
chosen summation profile (``order``).

What is served: float32 data and float64 data (every other input dtype
becomes float64, as in fuel; float64 runs the exact FP64 scan with fuel's f64
distances), distances ``euclidean``/``l2`` and ``sqeuclidean``/
``squared_euclidean``, the linear scan (``tree`` = ``None``, ``'auto'``,
``'linear'``, ``'brute'``, ``'bruteforce'``).  Anything else raises
``NotImplementedError`` rather than silently running elsewhere.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

_DISTANCE = {
    "euclidean": "euclidean", "l2": "euclidean",
    "sqeuclidean": "sqeuclidean", "squared_euclidean": "sqeuclidean",
}
# python/fuel/search.py:12-26
_TREE_NAME_MAP = {
    "auto": "auto", "vp": "vp", "vptree": "vp", "cover": "cover", "covertree": "cover", "ct": "cover",
    "ball": "cover", "balltree": "cover", "kd": "kd", "kdtree": "kd", "linear": "linear", "brute": "linear",
    "bruteforce": "linear",
}


def _ensure_float(data):
    """python/fuel/_dispatch.py:8-12: non-float input becomes float64."""
    data = np.asarray(data)
    if data.dtype not in (np.float32, np.float64):
        return data.astype(np.float64)
    return data


def _normalize_tree(tree):
    """python/fuel/search.py:37-47."""
    if tree is None:
        return "auto"
    if not isinstance(tree, str):
        raise TypeError("tree must be a string or None")
    key = tree.lower().replace("_", "").replace("-", "")
    if key in _TREE_NAME_MAP:
        return _TREE_NAME_MAP[key]
    raise ValueError(
        f"unknown tree '{tree}', valid values are 'auto', 'vp', 'kd', 'cover', 'linear', 'vptree', 'ct', "
        "'covertree', 'brute', or 'brute_force'")


def _parse_distance(distance: str) -> str:
    """python/mod.rs:42-71 for the two metrics this engine serves."""
    key = str(distance).lower()
    if key in _DISTANCE:
        return _DISTANCE[key]
    raise NotImplementedError(
        f"distance '{distance}' is not served by the GB300 linear scan (served: euclidean, l2, sqeuclidean, "
        "squared_euclidean)")


class SearchIndex:
    """Persistent linear-scan index held in GB300 memory.

    Parameters mirror ``fuel.search.SearchIndex`` (python/fuel/search.py:230).
    ``precision`` (None / 'auto' | 'fp32' | 'bf16' | 'split_bf16' | 'fp16')
    picks the tier (every tier returns the exact reference answer; the
    tensor-core tiers screen in BF16, hi+lo BF16 or FP16 and re-score); the
    default lets the engine choose per (d, n, k, value class) bucket, timing
    the eligible tiers the first time a bucket is seen, and
    ``order`` ('arm' | 'x86') the summation profile to reproduce (default: the
    profile fuel compiles on this host).  ``precompute=K`` builds, on the GPU,
    the tie-inclusive kNN table of every indexed point to ``min(K, n)``
    neighbours, as PrecomputedKnnSearcher::new does (src/search/precomputed.rs:
    36-55, python/search.rs:1362-1366); self-join queries with ``k + 1 <=
    max_k`` (exclude_self) or ``k <= max_k`` are then served from the table
    with subset_with_ties (precomputed.rs:60-89) and the k+1 exclude rule of
    the precomputed path (python/search.rs:1154-1173); other queries are
    computed by the scan.  (The reference serves every external query from
    row 0 of its table, python/search.rs:578-585 with precomputed.rs:81-85;
    that is not reproduced.)
    """

    def __init__(self, data, *, distance="euclidean", tree=None, seed=None, precompute=None, precision=None,
                 order=None):
        data = _ensure_float(data)
        if data.ndim != 2:
            raise ValueError("data must be a 2D array of observations")
        self.data = data
        self.distance = distance
        self.seed = seed
        self.precompute = precompute
        self.dtype = data.dtype
        self.shape = data.shape
        self.tree = _normalize_tree(tree)
        if self.tree == "auto":
            self.tree = "linear"
        if self.tree != "linear":
            raise NotImplementedError(
                f"tree '{tree}' is not served by the GB300 engine; only the exact linear scan is accelerated")
        self._metric = _parse_distance(distance)
        self._f64 = data.dtype == np.float64
        precision = "auto" if precision is None else precision
        if precision not in _lib.PRECISION:
            raise ValueError(f"precision must be one of {sorted(_lib.PRECISION)}")
        if self._f64 and precision not in ("auto", "fp32"):
            raise NotImplementedError(
                f"precision '{precision}' applies to float32 data; float64 data runs the exact FP64 scan")
        self.precision = precision
        self.order = order or _lib.default_order()
        if self.order not in _lib.ORDER:
            raise ValueError(f"order must be one of {sorted(_lib.ORDER)}")
        self._source_shape = data.shape
        self._source_strides = data.strides
        self._source_ptr = data.__array_interface__["data"][0]
        lib = _lib.load()
        host = np.ascontiguousarray(data)
        handle = ctypes.c_void_p()
        create = lib.fuelg_index_create_f64 if self._f64 else lib.fuelg_index_create
        _lib.check(create(_lib.ptr(host), host.shape[0], host.shape[1], _lib.METRIC[self._metric],
                          _lib.ORDER[self.order], ctypes.byref(handle)))
        self._handle = handle
        self.index = self
        self.last_stats = None
        self._table = None
        if precompute is not None:
            max_k = min(int(precompute), host.shape[0])
            if max_k > 0:
                self._table = (max_k,) + self._ties_csr(None, host.shape[0], max_k, _lib.EXCLUDE_NONE)

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                _lib.load().fuelg_index_destroy(h)
            except Exception:
                pass
            self._handle = None

    def _same_source(self, query):
        """python/fuel/search.py:270-275."""
        return (query.shape == self._source_shape and query.strides == self._source_strides
                and query.__array_interface__["data"][0] == self._source_ptr)

    def _prepare_query(self, query, exclude_self):
        query = _ensure_float(query)
        if query.dtype != self.dtype:
            query = query.astype(self.dtype)
        if query.ndim != 2 or query.shape[1] != self.shape[1]:
            raise ValueError(f"query shape {query.shape} is not compatible with index data shape {self.shape}")
        if exclude_self is None:
            exclude_self = self._same_source(query)
        elif exclude_self and not self._same_source(query):
            raise ValueError(
                "exclude_self=True is only supported when query refers to the same underlying array as data")
        return query, bool(exclude_self)

    def knn(self, query, k, *, exclude_self=None):
        """(int64[m, k] indices, [m, k] distances of the index dtype), -1 / inf padded."""
        query, exclude_self = self._prepare_query(query, exclude_self)
        k = int(k)
        if k < 0:
            raise OverflowError("can't convert negative int to unsigned")
        m = query.shape[0]
        if (self._table is not None and k > 0 and self._same_source(query)
                and (k + 1 if exclude_self else k) <= self._table[0]):
            self.last_stats = {"served_from": "precomputed table", "max_k": self._table[0]}
            return self._knn_from_table(m, k, exclude_self)
        q = np.ascontiguousarray(query)
        idx = np.empty((m, k), np.int64)
        dist = np.empty((m, k), self.dtype)
        if exclude_self:
            mode = _lib.EXCLUDE_KPLUS1 if self.precompute is not None else _lib.EXCLUDE_LINEAR
        else:
            mode = _lib.EXCLUDE_NONE
        st = _lib.Stats()
        lib = _lib.load()
        if self._f64:
            _lib.check(lib.fuelg_knn_f64(self._handle, _lib.ptr(q), m, k, mode, _lib.ptr(idx), _lib.ptr(dist),
                                         ctypes.byref(st)))
        else:
            _lib.check(lib.fuelg_knn(self._handle, _lib.ptr(q), m, k, mode, _lib.PRECISION[self.precision],
                                     _lib.ptr(idx), _lib.ptr(dist), ctypes.byref(st)))
        self.last_stats = st.as_dict()
        return idx, dist

    def _ties_csr(self, q, m, k, mode):
        """fuelg_knn_ties -> (offsets int64[m+1], idx int64[], dist[] of the index
        dtype); q None: the index's own rows are the queries."""
        lib = _lib.load()
        res = ctypes.c_void_p()
        st = _lib.Stats()
        qp = None if q is None else _lib.ptr(q)
        if self._f64:
            _lib.check(lib.fuelg_knn_ties_f64(self._handle, qp, m, k, mode, ctypes.byref(res), ctypes.byref(st)))
        else:
            _lib.check(lib.fuelg_knn_ties(self._handle, qp, m, k, mode, _lib.PRECISION[self.precision],
                                          ctypes.byref(res), ctypes.byref(st)))
        try:
            off, idx, dist = _take_csr(lib, res, m, self._f64)
        finally:
            lib.fuelg_range_free(res)
        self.last_stats = st.as_dict()
        return off, idx, dist

    def knn_with_ties(self, query, k, *, exclude_self=None):
        """Tie-inclusive kNN lists: ([int64 arrays], [distance arrays]) per
        query row -- the k nearest points plus every point tied with the k-th
        distance, sorted by (distance, index), as KNNHeap::into_vec returns
        them (src/api/search.rs:80-151); exclude_self drops index i from row i
        after the search (the linear-index rule, python/search.rs:485-488, or
        the k+1 rule of a precomputed index, :1163-1170)."""
        query, exclude_self = self._prepare_query(query, exclude_self)
        k = int(k)
        if k < 0:
            raise OverflowError("can't convert negative int to unsigned")
        q = np.ascontiguousarray(query)
        m = q.shape[0]
        if exclude_self:
            mode = _lib.EXCLUDE_KPLUS1 if self.precompute is not None else _lib.EXCLUDE_LINEAR
        else:
            mode = _lib.EXCLUDE_NONE
        off, idx, dist = self._ties_csr(q, m, k, mode)
        return ([idx[off[i]:off[i + 1]].copy() for i in range(m)],
                [dist[off[i]:off[i + 1]].copy() for i in range(m)])

    def _knn_from_table(self, m, k, exclude_self):
        """subset_with_ties of every row's table entry (src/search/precomputed.rs:
        60-67), self dropped, truncated to k (python/search.rs:1154-1173, 1195-1216).
        Every row holds at least max_k >= kq entries, so the first kq columns of
        each row decide the answer."""
        max_k, off, idx, dist = self._table
        kq = k + 1 if exclude_self else k
        cols = off[:-1, None] + np.arange(kq)[None, :]
        gi = idx[cols]
        gd = dist[cols]
        if exclude_self:
            is_self = gi == np.arange(m)[:, None]
            has = is_self.any(axis=1)
            p = np.where(has, np.argmax(is_self, axis=1), kq)
            j = np.arange(k)[None, :]
            src = j + (j >= p[:, None])
            gi = np.take_along_axis(gi, src, axis=1)
            gd = np.take_along_axis(gd, src, axis=1)
        return np.ascontiguousarray(gi[:, :k]), np.ascontiguousarray(gd[:, :k])

    def radius_search(self, query, radius, *, exclude_self=None):
        """([int64 arrays], [distance arrays]) per query row, sorted by (distance, index)."""
        query, exclude_self = self._prepare_query(query, exclude_self)
        q = np.ascontiguousarray(query)
        m = q.shape[0]
        lib = _lib.load()
        res = ctypes.c_void_p()
        st = _lib.Stats()
        call = lib.fuelg_range_f64 if self._f64 else lib.fuelg_range
        _lib.check(call(self._handle, _lib.ptr(q), m, float(radius), int(exclude_self), ctypes.byref(res),
                        ctypes.byref(st)))
        try:
            off, idx, dist = _take_csr(lib, res, m, self._f64)
        finally:
            lib.fuelg_range_free(res)
        self.last_stats = st.as_dict()
        idx_list = [idx[off[i]:off[i + 1]].copy() for i in range(m)]
        dist_list = [dist[off[i]:off[i + 1]].copy() for i in range(m)]
        return idx_list, dist_list

    def priority_searcher(self, query):
        """Priority search for one coordinate query row: candidates in
        ascending (distance, index) order between a skip distance and a
        cutoff (src/search/linear_scan.rs:70-235)."""
        return PrioritySearcher(self, query)

    def __repr__(self):
        return f"<SearchIndex tree={self.tree!r} dtype={self.dtype!r} shape={self.shape!r}>"


def _take_csr(lib, res, m, f64=False):
    """Copy a fuelg_range_result to host arrays (offsets[m+1], idx[], dist[])."""
    mm, tot = ctypes.c_int64(), ctypes.c_int64()
    _lib.check(lib.fuelg_range_size(res, ctypes.byref(mm), ctypes.byref(tot)))
    off = np.empty(m + 1, np.int64)
    idx = np.empty(max(1, tot.value), np.int64)
    dist = np.empty(max(1, tot.value), np.float64 if f64 else np.float32)
    copy = lib.fuelg_range_copy_f64 if f64 else lib.fuelg_range_copy
    _lib.check(copy(res, _lib.ptr(off), _lib.ptr(idx), _lib.ptr(dist)))
    return off, idx[:tot.value], dist[:tot.value]


class PrioritySearcher:
    """LinearScanPrioritySearcher (src/search/linear_scan.rs:70-235) over the
    GPU range scan.  On first use the candidates with skip <= distance <=
    cutoff are computed (one fuelg_range call with the cutoff as radius, the
    skip applied to its (distance, index)-ordered hits) and then handed out
    in order; ``decrease_cutoff`` only ever lowers the cutoff, and candidates
    past it end the iteration, as in the reference."""

    def __init__(self, index: SearchIndex, query):
        q = np.ascontiguousarray(np.asarray(query, dtype=index.dtype).reshape(1, -1))
        if q.shape[1] != index.shape[1]:
            raise ValueError(f"query must have {index.shape[1]} coordinates")
        self._index = index
        self._query = q
        self._ft = index.dtype.type  # cutoff and skip compare in the index dtype
        self.reset()

    def reset(self):
        self._cand = None
        self._pos = 0
        self.cutoff = self._ft(np.inf)
        self.skip = self._ft(0.0)

    def reset_with_limits(self, cutoff, skip):
        if not skip >= 0 or not cutoff >= skip:
            raise ValueError("need 0 <= skip <= cutoff")
        self.reset()
        self.cutoff = self._ft(cutoff)
        self.skip = self._ft(skip)

    def _ensure(self):
        if self._cand is not None:
            return
        idx, dist = self._index.radius_search(self._query, float(self.cutoff), exclude_self=False)
        keep = dist[0] >= self.skip
        self._cand = (idx[0][keep], dist[0][keep])
        self._pos = 0

    def next(self, skip_point=None):
        """Next (distance, index) or None; skip_point(index) -> True skips a
        point (SearchFilter)."""
        self._ensure()
        idx, dist = self._cand
        while self._pos < len(idx):
            i, d = int(idx[self._pos]), dist[self._pos]
            self._pos += 1
            if d > self.cutoff:
                return None
            if d < self.skip:
                continue
            if skip_point is not None and skip_point(i):
                continue
            return float(d), i
        return None

    def all_lower_bound(self):
        if self._cand is None:
            return 0.0
        idx, dist = self._cand
        for j in range(self._pos, len(idx)):
            d = dist[j]
            if d > self.cutoff:
                break
            if d >= self.skip:
                return float(d)
        return float("inf")

    def decrease_cutoff(self, threshold):
        if threshold > self.cutoff:
            raise ValueError("thresholds must only decrease")
        self.cutoff = self._ft(threshold)


def knn_search(data, query, k, *, exclude_self=None, distance="euclidean", tree="auto", seed=None, **kw):
    """python/fuel/search.py:315-368."""
    data = _ensure_float(data)
    query = _ensure_float(query)
    index = SearchIndex(data, distance=distance, tree=tree, seed=seed, **kw)
    return index.knn(query, k, exclude_self=exclude_self)


def range_search(data, query, radius, *, exclude_self=None, distance="euclidean", tree="auto", seed=None, **kw):
    """python/fuel/search.py:371-408."""
    data = _ensure_float(data)
    query = _ensure_float(query)
    index = SearchIndex(data, distance=distance, tree=tree, seed=seed, **kw)
    return index.radius_search(query, radius, exclude_self=exclude_self)


def knn_batched(sets, *, order=None):
    """Many independent exact kNN query sets in one engine call.

    ``sets``: iterable of ``(data float32[n, d], queries float32[m, d], k)`` or
    ``(data, queries, k, options)`` with ``options`` a dict of ``distance``
    ('euclidean' default, or 'sqeuclidean') and ``exclude`` ('none' default,
    'linear' -- the linear index's exclude-self rule, python/search.rs:485-488
    -- or 'kplus1', the precomputed / tree rule, :1163-1170; query row i is
    matched against point i of the same set).  Returns a list of
    ``(int64[m, k], float32[m, k])`` -- for each set exactly what
    ``SearchIndex(data, distance=..., tree='linear', precision='fp32').knn``
    returns -- computed by one scan launch over all sets (each with its own n,
    d and k) and one merge launch.  No reference counterpart: fuel answers one
    call at a time.
    """
    order = order or _lib.default_order()
    if order not in _lib.ORDER:
        raise ValueError(f"order must be one of {sorted(_lib.ORDER)}")
    modes = {"none": _lib.EXCLUDE_NONE, "linear": _lib.EXCLUDE_LINEAR, "kplus1": _lib.EXCLUDE_KPLUS1}
    keep, descs, outs = [], [], []
    for item in sets:
        data, queries, k = item[0], item[1], int(item[2])
        opts = item[3] if len(item) > 3 else {}
        if _ensure_float(data).dtype != np.float32 or _ensure_float(queries).dtype != np.float32:
            # a silent cast would change the answer: fuel searches such data in float64
            raise NotImplementedError("knn_batched serves float32 sets; search float64 data with SearchIndex "
                                      "(the exact FP64 scan)")
        X = np.ascontiguousarray(data, np.float32)
        Q = np.ascontiguousarray(queries, np.float32)
        if X.ndim != 2 or Q.ndim != 2 or X.shape[1] != Q.shape[1]:
            raise ValueError("each set needs data [n, d] and queries [m, d]")
        if k < 0:
            raise ValueError("k must be non-negative")
        metric = _parse_distance(opts.get("distance", "euclidean"))
        exclude = opts.get("exclude", "none")
        if exclude not in modes:
            raise ValueError(f"exclude must be one of {sorted(modes)}")
        idx = np.empty((Q.shape[0], k), np.int64)
        dist = np.empty((Q.shape[0], k), np.float32)
        keep += [X, Q]
        descs.append(_lib.KnnSet(X.ctypes.data if X.size else None, X.shape[0], X.shape[1], _lib.METRIC[metric],
                                 Q.ctypes.data if Q.size else None, Q.shape[0], k, modes[exclude],
                                 idx.ctypes.data, dist.ctypes.data, 0, 0))
        outs.append((idx, dist))
    if not descs:
        return []
    arr = (_lib.KnnSet * len(descs))(*descs)
    st = _lib.Stats()
    _lib.check(_lib.load().fuelg_knn_batched(ctypes.cast(arr, ctypes.c_void_p), len(descs), _lib.ORDER[order],
                                             _lib.PRECISION["fp32"], ctypes.byref(st)))
    knn_batched.last_stats = st.as_dict()
    return outs


def _condensed_n(length: int) -> int:
    """n with n*(n-1)/2 == length (python/fuel/search.py:50-57)."""
    import math
    if length < 0:
        raise ValueError("condensed distance vector length must be non-negative")
    n = (1 + math.isqrt(1 + 8 * length)) // 2
    if n * (n - 1) // 2 != length:
        raise ValueError("condensed distance vector length must be n*(n-1)/2 for some integer n")
    return n


def pairwise_distances(data, distance="euclidean", form="condensed", *, order=None):
    """All pairwise distances of a point set (python/fuel/search.py:92-150).

    ``form='condensed'``: the lower triangle as one vector, pair (i, j) with
    j < i at ``i*(i-1)//2 + j``; ``form='square'``: the symmetric matrix.
    Raw float32 or float64 points with distance ``euclidean``/``l2`` or
    ``sqeuclidean``/``squared_euclidean`` run on the GPU (fuelg_pairwise /
    fuelg_pairwise_f64), bit-identical to fuel's distance of that dtype in the
    chosen summation ``order``;
    ``distance='precomputed'`` converts between the forms as fuel does (a 1-D
    input is a scipy ``pdist`` vector, pairs (a, b) with a < b).
    """
    data = _ensure_float(data)
    distance = str(distance).lower()
    form = str(form).lower()
    if form not in ("condensed", "square"):
        raise ValueError("form must be 'condensed' or 'square'")
    if distance == "precomputed":
        if data.ndim == 1:
            n = _condensed_n(data.shape[0])
            ti, tj = np.tril_indices(n, -1)  # i > j
            internal = data[tj * (2 * n - tj - 1) // 2 + (ti - tj - 1)]
            if form == "condensed":
                return internal
            sq = np.zeros((n, n), dtype=data.dtype)
            sq[ti, tj] = internal
            sq[tj, ti] = internal
            return sq
        if data.ndim == 2:
            if data.shape[0] != data.shape[1]:
                raise ValueError("precomputed distance matrix must be square")
            if form == "square":
                return data
            return data[np.tril_indices(data.shape[0], -1)].copy()
        raise ValueError("precomputed data must be a square matrix or condensed distance vector")
    if data.ndim != 2:
        raise ValueError("data must be a 2D array of observations when distance is not 'precomputed'")
    metric = _parse_distance(distance)
    order = order or _lib.default_order()
    if order not in _lib.ORDER:
        raise ValueError(f"order must be one of {sorted(_lib.ORDER)}")
    X = np.ascontiguousarray(data)
    n, d = X.shape
    square = form == "square"
    if d == 0:  # every distance between empty rows is 0
        return np.zeros((n, n) if square else n * (n - 1) // 2, dtype=X.dtype)
    out = np.empty(n * n if square else n * (n - 1) // 2, dtype=X.dtype)
    st = _lib.Stats()
    lib = _lib.load()
    call = lib.fuelg_pairwise_f64 if X.dtype == np.float64 else lib.fuelg_pairwise
    _lib.check(call(_lib.ptr(X), n, d, _lib.METRIC[metric], _lib.ORDER[order], 1 if square else 0, _lib.ptr(out),
                    ctypes.byref(st)))
    pairwise_distances.last_stats = st.as_dict()
    return out.reshape(n, n) if square else out
