"""Test-side oracle for fuel's linear-scan kNN / range search and Lloyd k-means.

This module is TEST INFRASTRUCTURE.  Only the tests, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` import it, and only as the checker
(or, for the baseline, as the thing timed on the host cores).  The product
library (``fuel_gb300``) never imports it.

Two oracles live here:

* ``libfuel_oracle.so`` (``fuel_oracle.c``): a C restatement of fuel's CPU
  code in fuel's own operation order, for both summation profiles that fuel
  compiles (``'arm'``: src/math/unroll.rs + the portable distance fallback;
  ``'x86'``: src/math/avx2.rs + the AVX2/FMA distance kernel).  Its results
  are bit-identical to what fuel returns on that ISA.
* an FP64 oracle (numpy): distances formed and summed in double, ordered by
  (distance, index) exactly like ``DistPair`` (src/api/search.rs:23-30).

Pinned against the reference's own known answers in tests/test_oracle_golden.py.
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libfuel_oracle.so")
_lib = None

ORDERS = {"arm": 0, "x86": 1}
KINDS = {"knn": 0, "sqdist": 1, "pairwise": 2, "dot": 3}
METRICS = {"sqeuclidean": 0, "euclidean": 1}
EXCLUDE = {"none": 0, "linear": 1, "kplus1": 2}


def host_order() -> str:
    """The summation profile fuel itself compiles on this machine."""
    m = platform.machine().lower()
    return "x86" if m in ("x86_64", "amd64") else "arm"


def build() -> str:
    """Compile libfuel_oracle.so in place (gcc, no cmake)."""
    src = os.path.join(_HERE, "fuel_oracle.c")
    if (not os.path.exists(_LIB_PATH)) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return _LIB_PATH


def load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = ctypes.CDLL(_LIB_PATH)
    i64, i32, dbl = ctypes.c_int64, ctypes.c_int, ctypes.c_double
    vp = ctypes.c_void_p
    lib.fo_dist_f32.restype = ctypes.c_float
    lib.fo_dist_f32.argtypes = [i32, i32, vp, vp, i64]
    lib.fo_dist_f64.restype = ctypes.c_double
    lib.fo_dist_f64.argtypes = [i32, i32, vp, vp, i64]
    for nm in ("fo_pairwise_sqdist_f32", "fo_pairwise_sqdist_f64"):
        getattr(lib, nm).restype = None
        getattr(lib, nm).argtypes = [i32, vp, i64, vp, i64, i64, vp]
    for nm in ("fo_knn_f32", "fo_knn_f64"):
        getattr(lib, nm).restype = i32
        getattr(lib, nm).argtypes = [vp, i64, i64, vp, i64, i64, i32, i32, i32, i32, vp, vp]
    for nm in ("fo_range_f32", "fo_range_f64"):
        getattr(lib, nm).restype = i32
        getattr(lib, nm).argtypes = [vp, i64, i64, vp, i64, dbl, i32, i32, i32, i32,
                                     ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp)]
    lib.fo_free.restype = None
    lib.fo_free.argtypes = [vp]
    lib.fo_pairwise_dist_f32.restype = i32
    lib.fo_pairwise_dist_f32.argtypes = [vp, i64, i64, i32, i32, i32, i32, vp]
    lib.fo_lloyd_f32.restype = i32
    lib.fo_lloyd_f32.argtypes = [vp, i64, i64, i64, vp, i64, dbl, i32, i32, i32, vp, vp,
                                 ctypes.POINTER(i64), ctypes.POINTER(dbl), ctypes.POINTER(i64)]
    lib.fo_lloyd_assign_f32.restype = i32
    lib.fo_lloyd_assign_f32.argtypes = [vp, i64, i64, i64, vp, i32, i32, i32, vp, vp]
    _lib = lib
    return lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _f(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def dist(kind: str, order: str, a, b) -> float:
    """One per-pair distance in the reference's operation order."""
    lib = load()
    a = np.asarray(a)
    if a.dtype == np.float64:
        a, b = _f(a, np.float64), _f(b, np.float64)
        return float(lib.fo_dist_f64(KINDS[kind], ORDERS[order], _p(a), _p(b), a.shape[0]))
    a, b = _f(a, np.float32), _f(b, np.float32)
    return np.float32(lib.fo_dist_f32(KINDS[kind], ORDERS[order], _p(a), _p(b), a.shape[0]))


def pairwise_sqdist(p1, p2, order: str | None = None) -> np.ndarray:
    """math::pairwise_sqdist (src/math/mod.rs) as an [n1, n2] matrix."""
    lib = load()
    order = order or host_order()
    p1 = np.asarray(p1)
    is64 = p1.dtype == np.float64
    dt = np.float64 if is64 else np.float32
    p1, p2 = _f(p1, dt), _f(p2, dt)
    out = np.empty((p1.shape[0], p2.shape[0]), dtype=dt)
    fn = lib.fo_pairwise_sqdist_f64 if is64 else lib.fo_pairwise_sqdist_f32
    fn(ORDERS[order], _p(p1), p1.shape[0], _p(p2), p2.shape[0], p1.shape[1], _p(out))
    return out


def pairwise_distances(X, metric: str = "euclidean", form: str = "condensed", order: str | None = None,
                       threads: int = 1) -> np.ndarray:
    """fuel.search.pairwise_distances for raw f32 points (python/fuel/search.py:92-150):
    the condensed lower triangle (pair (i, j), j < i, at i*(i-1)/2 + j) or the
    square matrix, each value distance(X[i], X[j]) in the reference's order."""
    lib = load()
    order = order or host_order()
    X = _f(X, np.float32)
    n, d = X.shape
    square = form == "square"
    out = np.empty(n * n if square else n * (n - 1) // 2, dtype=np.float32)
    rc = lib.fo_pairwise_dist_f32(_p(X), n, d, METRICS[metric], ORDERS[order], int(square), threads, _p(out))
    if rc:
        raise ValueError("pairwise_distances: invalid arguments")
    return out.reshape(n, n) if square else out


def knn(X, Q, k: int, metric: str = "sqeuclidean", order: str | None = None, exclude: str = "none",
        threads: int = 1):
    """SearchIndex(tree='linear').knn: (int64[m,k], float[m,k]) with -1/+inf padding."""
    lib = load()
    order = order or host_order()
    X = np.asarray(X)
    is64 = X.dtype == np.float64
    dt = np.float64 if is64 else np.float32
    X, Q = _f(X, dt), _f(Q, dt)
    m, d = Q.shape
    idx = np.empty((m, k), dtype=np.int64)
    dd = np.empty((m, k), dtype=dt)
    fn = lib.fo_knn_f64 if is64 else lib.fo_knn_f32
    rc = fn(_p(X), X.shape[0], d, _p(Q), m, k, METRICS[metric], ORDERS[order], EXCLUDE[exclude], threads,
            _p(idx), _p(dd))
    if rc != 0:
        raise ValueError("oracle knn: bad arguments")
    return idx, dd


def range_search(X, Q, radius: float, metric: str = "sqeuclidean", order: str | None = None,
                 exclude_self: bool = False, threads: int = 1):
    """linear_scan_range per query row -> CSR (offsets[m+1], idx[], dist[])."""
    lib = load()
    order = order or host_order()
    X = np.asarray(X)
    is64 = X.dtype == np.float64
    dt = np.float64 if is64 else np.float32
    X, Q = _f(X, dt), _f(Q, dt)
    m, d = Q.shape
    po, pi, pd = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    fn = lib.fo_range_f64 if is64 else lib.fo_range_f32
    fn(_p(X), X.shape[0], d, _p(Q), m, float(radius), METRICS[metric], ORDERS[order], int(exclude_self),
       threads, ctypes.byref(po), ctypes.byref(pi), ctypes.byref(pd))
    off = np.ctypeslib.as_array(ctypes.cast(po, ctypes.POINTER(ctypes.c_int64)), shape=(m + 1,)).copy()
    tot = int(off[-1])
    if tot:
        idx = np.ctypeslib.as_array(ctypes.cast(pi, ctypes.POINTER(ctypes.c_int64)), shape=(tot,)).copy()
        ctyp = ctypes.c_double if is64 else ctypes.c_float
        dist_ = np.ctypeslib.as_array(ctypes.cast(pd, ctypes.POINTER(ctyp)), shape=(tot,)).copy()
    else:
        idx = np.empty(0, np.int64)
        dist_ = np.empty(0, dt)
    for p in (po, pi, pd):
        lib.fo_free(p)
    return off, idx, dist_


def lloyd(X, k: int, init, max_iter: int = 300, tol: float = 0.0, order: str | None = None,
          threads: int = 1, sums: str = "reference"):
    """lloyd() with a fixed init array.  sums='reference' reproduces fuel's f32
    running sums (result depends on `threads`, the rayon thread count);
    sums='fp64' uses fp64 cluster sums and returns the fp64 inertia."""
    lib = load()
    order = order or host_order()
    X = _f(X, np.float32)
    init = _f(init, np.float32)
    n, d = X.shape
    cent = np.empty((k, d), np.float32)
    lab = np.empty(n, np.int64)
    it = ctypes.c_int64()
    inert = ctypes.c_double()
    chg = ctypes.c_int64()
    rc = lib.fo_lloyd_f32(_p(X), n, d, k, _p(init), max_iter, float(tol), ORDERS[order], threads,
                          0 if sums == "reference" else 1, _p(cent), _p(lab), ctypes.byref(it),
                          ctypes.byref(inert), ctypes.byref(chg))
    if rc != 0:
        raise ValueError("oracle lloyd: bad arguments")
    return cent, lab, int(it.value), float(inert.value)


def lloyd_assign(X, centers, initial: bool = False, order: str | None = None, threads: int = 1):
    """One assignment pass against fixed centres: (labels int64[n], best f32[n])."""
    lib = load()
    order = order or host_order()
    X = _f(X, np.float32)
    C = _f(centers, np.float32)
    n, d = X.shape
    lab = np.empty(n, np.int64)
    best = np.empty(n, np.float32)
    lib.fo_lloyd_assign_f32(_p(X), n, d, C.shape[0], _p(C), int(initial), ORDERS[order], threads, _p(lab),
                            _p(best))
    return lab, best


# --------------------------------------------------------------------------
# FP64 oracle
# --------------------------------------------------------------------------

def sqdist_fp64(X, Q) -> np.ndarray:
    """Exact-in-double squared distances [m, n]: differences and sums in fp64."""
    X = np.asarray(X, np.float64)
    Q = np.asarray(Q, np.float64)
    out = np.empty((Q.shape[0], X.shape[0]), np.float64)
    step = max(1, int(2e7 // max(1, X.shape[0] * X.shape[1])))
    for s in range(0, Q.shape[0], step):
        diff = Q[s:s + step, None, :] - X[None, :, :]
        out[s:s + step] = np.einsum("mnd,mnd->mn", diff, diff)
    return out


def knn_fp64(X, Q, k: int, metric: str = "sqeuclidean", exclude_self: bool = False):
    """Top-k by (fp64 distance, index); exclude_self drops index i for query i
    after selecting k+1 (the tree-path semantics)."""
    D = sqdist_fp64(X, Q)
    if metric == "euclidean":
        D = np.sqrt(D)
    m, n = D.shape
    idx = np.full((m, k), -1, np.int64)
    dist_ = np.full((m, k), np.inf)
    ar = np.arange(n)
    for i in range(m):
        order_ = np.lexsort((ar, D[i]))
        if exclude_self:
            order_ = order_[order_ != i]
        order_ = order_[:k]
        idx[i, :len(order_)] = order_
        dist_[i, :len(order_)] = D[i, order_]
    return idx, dist_


def lloyd_inertia_fp64(X, centers, labels) -> float:
    X = np.asarray(X, np.float64)
    C = np.asarray(centers, np.float64)
    diff = X - C[np.asarray(labels)]
    return float(np.einsum("nd,nd->", diff, diff))


# --------------------------------------------------------------------------
# Outlier scores from kNN lists (for the ELKI golden vectors)
# --------------------------------------------------------------------------

def knn_outlier(dist_k: np.ndarray) -> np.ndarray:
    """kNN outlier score: distance to the k-th neighbour (src/outlier/knn.rs:14-36)."""
    return np.array([row[np.isfinite(row)][-1] if np.isfinite(row).any() else 0.0 for row in dist_k])


def lof(idx: np.ndarray, dist_: np.ndarray) -> np.ndarray:
    """Local outlier factor from exclusive k-NN lists (src/outlier/lof.rs:38-80)."""
    n = idx.shape[0]
    neigh = [[(int(j), float(dv)) for j, dv in zip(idx[i], dist_[i]) if j >= 0] for i in range(n)]
    kdist = np.array([nb[-1][1] if nb else 0.0 for nb in neigh])
    lrd = np.empty(n)
    for i in range(n):
        if not neigh[i]:
            lrd[i] = np.inf
            continue
        s = 0.0
        for j, dv in neigh[i]:
            s += max(kdist[j], dv)
        lrd[i] = len(neigh[i]) / s if s > 0 else np.inf
    out = np.empty(n)
    for i in range(n):
        if not neigh[i] or np.isinf(lrd[i]):
            out[i] = 1.0
        else:
            s = 0.0
            for j, _ in neigh[i]:
                s += lrd[j]
            out[i] = s / (lrd[i] * len(neigh[i]))
    return out


def knn_with_ties(X, q, k: int, metric: str = "sqeuclidean", order: str | None = None):
    """The full tie-inclusive linear_scan_knn list for one query (no truncation)."""
    lib = load()
    order = order or host_order()
    dt = np.float64 if np.asarray(X).dtype == np.float64 else np.float32
    X = _f(X, dt)
    q = _f(q, dt).ravel()
    fn = lib.fo_knn_ties_f64 if dt == np.float64 else lib.fo_knn_ties_f32
    fn.restype = ctypes.c_int64
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                   ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
    cap = X.shape[0]
    idx = np.empty(cap, np.int64)
    dd = np.empty(cap, dt)
    cnt = fn(_p(X), X.shape[0], X.shape[1], _p(q), k, METRICS[metric], ORDERS[order], cap, _p(idx), _p(dd))
    return idx[:cnt].copy(), dd[:cnt].copy()


def knn_ties(X, Q, k: int, metric: str = "sqeuclidean", order: str | None = None, exclude: str = "none"):
    """Tie-inclusive lists of every query row as CSR (offsets, idx, dist):
    linear_scan_knn's KNNHeap::into_vec list (k, or k+1 for exclude='kplus1'),
    then index i dropped from row i for exclude 'linear' / 'kplus1'
    (python/search.rs:485-488, 1163-1170)."""
    dt = np.float64 if np.asarray(X).dtype == np.float64 else np.float32
    Q = _f(Q, dt)
    kq = k + 1 if exclude == "kplus1" else k
    offs, ids, ds = [0], [], []
    for i in range(Q.shape[0]):
        ii, dd = knn_with_ties(X, Q[i], kq, metric=metric, order=order)
        if exclude != "none":
            keep = ii != i
            ii, dd = ii[keep], dd[keep]
        ids.append(ii)
        ds.append(dd)
        offs.append(offs[-1] + len(ii))
    cat = (lambda parts, dt: np.concatenate(parts).astype(dt) if parts else np.empty(0, dt))
    return np.array(offs, np.int64), cat(ids, np.int64), cat(ds, dt)


# --------------------------------------------------------------------------
# Exact-mean Lloyd: fuel's assignment order, centres = correctly rounded f32
# of the exact mean of each cluster's member rows.
# --------------------------------------------------------------------------

def rn_f32_ratio(S: int, cnt: int, e_lo: int) -> np.float32:
    """Round-to-nearest-even f32 of S * 2**e_lo / cnt (S, cnt Python ints)."""
    import math
    if S == 0:
        return np.float32(0.0)
    neg = S < 0
    A = -S if neg else S
    sh = max(0, 27 - (A.bit_length() - cnt.bit_length()))
    q, r = divmod(A << sh, cnt)
    drop = q.bit_length() - 24
    mant = q >> drop
    rem = q & ((1 << drop) - 1)
    half = 1 << (drop - 1)
    if rem > half or (rem == half and (r != 0 or (mant & 1))):
        mant += 1
    v = np.float32(math.ldexp(float(mant), drop + e_lo - sh))
    return -v if neg else v


def fixed_point(X: np.ndarray):
    """Exact integer form of f32 data: X == I * 2**e_lo.  Returns (I, e_lo)
    with I int64 when the sums of up to len(X) rows fit, else Python ints.
    Only the non-zero entries are decoded."""
    X = np.ascontiguousarray(X, np.float32)
    flat = X.view(np.uint32).ravel()
    pos = np.flatnonzero(flat & 0x7FFFFFFF)
    if pos.size == 0:
        return np.zeros(X.shape, np.int64), 0
    bits = flat[pos].astype(np.int64)
    eb = (bits >> 23) & 0xFF
    mant = (bits & 0x7FFFFF) | np.where(eb != 0, 1 << 23, 0)
    unit = np.where(eb == 0, -149, eb - 150)
    # trailing zeros from the lowest set bit (a power of two below 2**24: exact in float64)
    ctz = np.log2((mant & -mant).astype(np.float64)).astype(np.int64)
    mm = mant >> ctz
    # mant = mm * 2**ctz with mm odd, so X = mm * 2**(unit + ctz)
    low = unit + ctz
    e_lo = int(low.min())
    e_hi = int((unit + np.floor(np.log2(mant)).astype(np.int64)).max())
    sign = np.where((bits >> 31) & 1, -1, 1)
    width = e_hi - e_lo + 1 + int(np.ceil(np.log2(X.shape[0] + 1))) + 1
    if width <= 62:
        I = np.zeros(flat.size, np.int64)
        I[pos] = sign * (mm << (low - e_lo))
        return I.reshape(X.shape), e_lo
    obj = np.zeros(flat.size, dtype=object)
    for t, p_ in enumerate(pos):
        obj[p_] = int(sign[t]) * (int(mm[t]) << int(low[t] - e_lo))
    return obj.reshape(X.shape), e_lo


def exact_means(I, e_lo, labels, k, prev, If64=None):
    """Correctly rounded f32 means of every cluster's member rows (I * 2**e_lo);
    empty clusters keep their previous centre.  With If64 (the float64 copy of
    an int64 I whose column sums of |I| stay below 2**53) the sums are one
    exact float64 matrix product and the rounding is vectorised
    (_rn_f32_ratio_vec); otherwise exact Python integers per coordinate."""
    C = np.array(prev, np.float32, copy=True)
    labels = np.asarray(labels)
    cnt = np.bincount(labels, minlength=k)[:k]
    if If64 is not None and labels.shape[0] < (1 << 26):
        onehot = np.zeros((k, labels.shape[0]), np.float64)
        onehot[labels, np.arange(labels.shape[0])] = 1.0
        S = onehot @ If64  # every partial sum is an integer below 2**53: exact in any order
        live = cnt > 0
        C[live] = _rn_f32_ratio_vec(S[live], cnt[live], e_lo)
        return C
    for j in range(k):
        rows = np.nonzero(labels == j)[0]
        if len(rows) == 0:
            continue
        S = I[rows].sum(axis=0)
        C[j] = [rn_f32_ratio(int(v), len(rows), e_lo) for v in S]
    return C


def _rn_f32_ratio_vec(S, cnt, e_lo):
    """Vectorised rn_f32_ratio for exact integer sums S (float64 [r, d],
    |S| < 2**53) and counts cnt (< 2**26): the float64 quotient rounded to f32,
    then corrected against the exact rounding boundaries of that f32 (the
    midpoints to its neighbours, times cnt, are exact float64 products), so
    double rounding cannot slip through.  Results that are zero or subnormal
    for a non-zero sum are recomputed with rn_f32_ratio."""
    cnt = np.asarray(cnt, np.float64)[:, None]
    neg = S < 0
    T = np.ldexp(np.abs(S), e_lo)
    c = (T / cnt).astype(np.float32)
    up = np.nextafter(c, np.float32(np.inf))
    dn = np.nextafter(c, np.float32(0.0))
    c64 = c.astype(np.float64)
    m_hi = (c64 + up.astype(np.float64)) * 0.5 * cnt
    m_lo = (c64 + dn.astype(np.float64)) * 0.5 * cnt
    c_even = (c.view(np.uint32) & 1) == 0
    out = c.copy()
    out = np.where(T > m_hi, up, out)
    out = np.where(T == m_hi, np.where(c_even, c, up), out)
    out = np.where(T < m_lo, dn, out)
    out = np.where((T == m_lo) & (T > 0), np.where(c_even, c, dn), out)
    out = np.where(neg, -out, out).astype(np.float32)
    bad = (np.abs(S) > 0) & (np.abs(out) < np.float32(1.1754944e-38))
    for r, j in zip(*np.nonzero(bad)):
        e = int(round(float(np.abs(S[r, j]))))
        out[r, j] = rn_f32_ratio(-e if neg[r, j] else e, int(cnt[r, 0]), e_lo)
    return out


def lloyd_exact(X, k: int, init, max_iter: int = 300, order: str | None = None, threads: int = 1,
                fixed_iters: bool = False):
    """Lloyd with fuel's assignment arithmetic (iteration 1: pairwise order;
    later: math::sqdist order; first index wins ties) and exact-mean centres;
    the loop and iteration count follow src/cluster/kmeans/lloyd.rs:118-202
    (fixed_iters ignores the changed == 0 stop).  Returns (centres, labels,
    iterations, fp64 inertia)."""
    X = np.ascontiguousarray(X, np.float32)
    C = np.ascontiguousarray(init, np.float32).copy()
    I, e_lo = fixed_point(X)
    If64 = None
    if I.dtype == np.int64 and float(np.abs(I).sum(axis=0, dtype=np.float64).max(initial=0.0)) < 2.0 ** 52:
        If64 = I.astype(np.float64)
    labels, _ = lloyd_assign(X, C, initial=True, order=order, threads=threads)
    if max_iter > 1:
        C = exact_means(I, e_lo, labels, k, C, If64)
    it = 1
    while it < max_iter:
        it += 1
        new, _ = lloyd_assign(X, C, initial=False, order=order, threads=threads)
        changed = int((new != labels).sum())
        labels = new
        if it < max_iter:
            C = exact_means(I, e_lo, labels, k, C, If64)
        if not fixed_iters and changed == 0:
            break
    return C, labels, it, lloyd_inertia_fp64(X, C, labels)
