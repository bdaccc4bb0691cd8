"""The allocation-free kNN entry point (fuelg_knn_noalloc).

It is for callers that cannot allocate device memory -- a CUDA graph being
captured, hosts whose GPU memory belongs to another allocator, embedded users
with a fixed footprint -- and keeps every temporary in a static device array.
It must return exactly what fuelg_knn returns on the same inputs (indices and
f32 distance bits; the bar of every kNN parity test here), call after call:
the static array keeps the previous call's contents, so a second call with
different inputs must not see stale state.  This file sorts last so that a
-x run reaches it only after every other test has passed.
"""
import ctypes

import numpy as np
import pytest

from fuel_gb300 import _lib

pytestmark = pytest.mark.gpu


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
    Xd = torch.from_numpy(X).cuda()
    Qd = torch.from_numpy(Q).cuda()
    oi = torch.full((Q.shape[0], k), 7, dtype=torch.int64, device="cuda")
    od = torch.full((Q.shape[0], k), 7.0, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.fuelg_knn_noalloc(_lib.ptr(Xd), X.shape[0], X.shape[1], _lib.ptr(Qd), Q.shape[0], k, metric,
                                     order, mode, _lib.ptr(oi), _lib.ptr(od), ctypes.c_void_p(stream)))
    torch.cuda.synchronize()
    return oi.cpu().numpy(), od.cpu().numpy()


def test_noalloc_matches_fuelg_knn_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    assert _lib.device_count() >= 1, "needs a GPU"
    rng = np.random.default_rng(123)
    cases = [
        # (n, d, m, k, metric, order, exclude)
        (5000, 16, 3000, 10, 0, 0, 1),      # self-join-like, ties possible, linear exclude rule
        (2500, 33, 40000, 100, 1, 1, 0),    # more queries than one scratch batch holds
    ]
    for n, d, m, k, metric, order, mode in cases:
        X = rng.integers(0, 4, size=(n, d)).astype(np.float32) if mode else rng.normal(size=(n, d)).astype(np.float32)
        Q = X[:m].copy() if m <= n else rng.normal(size=(m, d)).astype(np.float32)
        if mode and m > n:
            Q = X.copy()
        ri, rd = knn_reference_entry(lib, X, Q, k, metric, order, mode)
        gi, gd = knn_noalloc(lib, torch, X, Q, k, metric, order, mode)
        assert np.array_equal(gi, ri)
        assert np.array_equal(gd.view(np.uint32), rd.view(np.uint32))


def test_noalloc_rejects_host_buffers_and_oversize_k():
    lib = _lib.load()
    X = np.zeros((4, 3), np.float32)
    oi = np.zeros((4, 2), np.int64)
    od = np.zeros((4, 2), np.float32)
    rc = lib.fuelg_knn_noalloc(_lib.ptr(X), 4, 3, _lib.ptr(X), 4, 2, 0, 0, 0, _lib.ptr(oi), _lib.ptr(od), None)
    assert rc == _lib.EINVAL and "device-accessible" in _lib.last_error()
    rc = lib.fuelg_knn_noalloc(_lib.ptr(X), 4, 3, _lib.ptr(X), 4, 5000, 0, 0, 0, _lib.ptr(oi), _lib.ptr(od), None)
    assert rc == _lib.ENOTSUP and "4095" in _lib.last_error()
