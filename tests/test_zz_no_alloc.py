"""The allocation-free kNN entry point (fuelg_knn_noalloc).

It is for callers that cannot allocate device memory -- hosts whose GPU memory
belongs to another allocator or is budgeted up front, embedded users with a
fixed footprint -- and keeps every temporary in a static device array.  It must
return exactly what fuelg_knn and the oracle return on the same inputs (indices
and f32 distance bits; the bar of every kNN parity test here), call after call:
the static array keeps the previous call's contents, so a second call with
different inputs must not see stale state.  The cases cover the paths that are
specific to the in-array driver: an empty index, the k+1 exclude rule, and
k = 4095, where the split count of the scan has to be cut down until the lists
fit the array.  This file sorts last so that a -x run reaches it only after
every other test has passed.
"""
import ctypes

import numpy as np
import pytest

from fuel_gb300 import _lib

pytestmark = pytest.mark.gpu

_EXCLUDE_NAMES = {0: "none", 1: "linear", 2: "kplus1"}
_METRIC_NAMES = {0: "sqeuclidean", 1: "euclidean"}
_ORDER_NAMES = {0: "arm", 1: "x86"}


def knn_reference_entry(lib, X, Q, k, metric, order, mode):
    """fuelg_knn through an index handle, host buffers."""
    h = ctypes.c_void_p()
    _lib.check(lib.fuelg_index_create(_lib.ptr(X), X.shape[0], X.shape[1], metric, order, ctypes.byref(h)))
    try:
        idx = np.empty((Q.shape[0], k), np.int64)
        dist = np.empty((Q.shape[0], k), np.float32)
        _lib.check(lib.fuelg_knn(h, _lib.ptr(Q), Q.shape[0], k, mode, 0, _lib.ptr(idx), _lib.ptr(dist), None))
        return idx, dist
    finally:
        lib.fuelg_index_destroy(h)


def knn_noalloc(lib, torch, X, Q, k, metric, order, mode):
    # an empty index still passes a (never read) device pointer
    Xd = torch.from_numpy(X).cuda() if X.size else torch.zeros(1, dtype=torch.float32, device="cuda")
    Qd = torch.from_numpy(Q).cuda()
    oi = torch.full((Q.shape[0], k), 7, dtype=torch.int64, device="cuda")
    od = torch.full((Q.shape[0], k), 7.0, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.fuelg_knn_noalloc(_lib.ptr(Xd), X.shape[0], Q.shape[1], _lib.ptr(Qd), Q.shape[0], k, metric,
                                     order, mode, _lib.ptr(oi), _lib.ptr(od), ctypes.c_void_p(stream)))
    torch.cuda.synchronize()
    return oi.cpu().numpy(), od.cpu().numpy()


def _case_data(rng, n, d, m, mode):
    if mode:  # self-join on tie-heavy integer data
        X = rng.integers(0, 4, size=(n, d)).astype(np.float32)
        Q = X[:m].copy() if m <= n else X.copy()
    else:
        X = rng.normal(size=(n, d)).astype(np.float32)
        Q = rng.normal(size=(m, d)).astype(np.float32)
    return X, Q


def test_noalloc_matches_fuelg_knn_and_oracle_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    from oracle import oracle
    lib = _lib.load()
    assert _lib.device_count() >= 1, "needs a GPU"
    rng = np.random.default_rng(123)
    cases = [
        # (n, d, m, k, metric, order, exclude)
        (5000, 16, 3000, 10, 0, 0, 1),      # self-join-like, ties possible, linear exclude rule
        (2500, 33, 40000, 100, 1, 1, 0),    # more queries than one scratch batch holds
        (3000, 12, 2000, 7, 0, 0, 2),       # k+1 exclude rule
        (0, 6, 300, 5, 0, 0, 0),            # empty index: every row padded
        (60000, 8, 64, 4095, 0, 0, 2),      # largest k: the scan's splits are cut to fit the array
    ]
    for n, d, m, k, metric, order, mode in cases:
        X, Q = _case_data(rng, n, d, m, mode) if n else (np.zeros((0, d), np.float32),
                                                         rng.normal(size=(m, d)).astype(np.float32))
        ri, rd = knn_reference_entry(lib, X, Q, k, metric, order, mode)
        gi, gd = knn_noalloc(lib, torch, X, Q, k, metric, order, mode)
        case = (n, d, m, k, metric, order, mode)
        assert np.array_equal(gi, ri), f"indices differ from fuelg_knn for {case}"
        assert np.array_equal(gd.view(np.uint32), rd.view(np.uint32)), f"distances differ from fuelg_knn for {case}"
        if n:
            ci, cd = oracle.knn(X, Q, k, metric=_METRIC_NAMES[metric], order=_ORDER_NAMES[order],
                                exclude=_EXCLUDE_NAMES[mode], threads=8)
        else:
            ci, cd = np.full((m, k), -1, np.int64), np.full((m, k), np.inf, np.float32)
        assert np.array_equal(gi, ci), f"indices differ from the oracle for {case}"
        assert np.array_equal(gd.view(np.uint32), cd.view(np.uint32)), f"distances differ from the oracle for {case}"


def test_noalloc_rejects_host_buffers_and_oversize_k():
    lib = _lib.load()
    X = np.zeros((4, 3), np.float32)
    oi = np.zeros((4, 2), np.int64)
    od = np.zeros((4, 2), np.float32)
    rc = lib.fuelg_knn_noalloc(_lib.ptr(X), 4, 3, _lib.ptr(X), 4, 2, 0, 0, 0, _lib.ptr(oi), _lib.ptr(od), None)
    assert rc == _lib.EINVAL and "cannot stage host buffers" in _lib.last_error()
    rc = lib.fuelg_knn_noalloc(_lib.ptr(X), 4, 3, _lib.ptr(X), 4, 5000, 0, 0, 0, _lib.ptr(oi), _lib.ptr(od), None)
    assert rc == _lib.ENOTSUP and "4095" in _lib.last_error()
