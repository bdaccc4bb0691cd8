"""kNN serving over a resident index (continuous batching).

``Server(index, ...)`` keeps the index (and its tensor-core form) on the
device; ``submit(queries, k)`` queues a request and returns a ``Request``
whose ``result()`` blocks for ``(idx int64[m, k], dist float32[m, k])`` --
exactly what ``index.knn(queries, k, exclude_self=False)`` returns.  Free
workers merge every queued request that fits their batch and the device
memory budget into one GPU batch, so requests that arrive while others run
are admitted as memory frees up.  No reference counterpart: fuel answers one
call at a time.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .search import SearchIndex


class Request:
    def __init__(self, server, rid, idx, dist):
        self._server = server
        self.id = rid
        self._idx, self._dist = idx, dist
        self.latency_ms = None
        self._done = False

    def result(self, timeout_ms: int = -1):
        if not self._done:
            lat = ctypes.c_double()
            _lib.check(self._server._lib.fuelg_server_wait(self._server._h, self.id, int(timeout_ms),
                                                           ctypes.byref(lat)))
            self.latency_ms = lat.value
            self._done = True
        return self._idx, self._dist


class Server:
    def __init__(self, index: SearchIndex, *, precision: str = "auto", max_batch_queries: int = 8192,
                 budget_bytes: int = 8 << 30, workers: int = 2):
        if not isinstance(index, SearchIndex):
            raise TypeError("index must be a fuel_gb300.SearchIndex")
        self._index = index  # keeps the index alive while the server runs
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self._lib.fuelg_server_create(index._handle, _lib.PRECISION[precision], int(max_batch_queries),
                                                 int(budget_bytes), int(workers), ctypes.byref(h)))
        self._h = h
        self.d = int(index.shape[1])

    def submit(self, queries, k: int) -> Request:
        Q = np.ascontiguousarray(queries, dtype=np.float32)
        if Q.ndim != 2 or Q.shape[1] != self.d:
            raise ValueError(f"queries must have shape [m, {self.d}]")
        m = Q.shape[0]
        idx = np.empty((m, int(k)), np.int64)
        dist = np.empty((m, int(k)), np.float32)
        rid = ctypes.c_int64()
        _lib.check(self._lib.fuelg_server_submit(self._h, _lib.ptr(Q), m, int(k), _lib.ptr(idx), _lib.ptr(dist),
                                                 ctypes.byref(rid)))
        return Request(self, rid.value, idx, dist)

    def stats(self) -> dict:
        b, q, r, n = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        ms = ctypes.c_double()
        _lib.check(self._lib.fuelg_server_stats(self._h, ctypes.byref(b), ctypes.byref(q), ctypes.byref(r),
                                                ctypes.byref(n), ctypes.byref(ms)))
        return {"batches": b.value, "queries": q.value, "max_batch_rows": r.value, "max_batch_requests": n.value,
                "device_ms": ms.value}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fuelg_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
