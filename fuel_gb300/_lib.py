"""ctypes binding of libfuelg.so (include/fuelg.h).

The engine has no CPU fallback: if the shared library is missing or no CUDA
device is visible, calls raise instead of computing anything on the host.
ctypes releases the GIL for the duration of every foreign call, as fuel's
py_interruptible does for its rayon work (src/api/parallel.rs:145-173).
"""
from __future__ import annotations

import ctypes
import os
import platform

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfuelg.so")

OK, EINVAL, ENOMEM, ECUDA, ECANCELLED, ENOTSUP, ENODEV, ETIMEOUT = range(8)
METRIC = {"sqeuclidean": 0, "euclidean": 1}
ORDER = {"arm": 0, "x86": 1}
EXCLUDE_NONE, EXCLUDE_LINEAR, EXCLUDE_KPLUS1 = 0, 1, 2
# fp16: kNN / serving only (tcgen05 FP16 screen; values within the FP16 range)
PRECISION = {"auto": -1, "fp32": 0, "bf16": 1, "split_bf16": 2, "fp16": 4}
# stats["precision_used"] may also be 3: split_bf16 on scaled-integer data
# and 5: the exact FP64 scan of float64 data (the _f64 calls)
PRECISION_NAMES = {0: "fp32", 1: "bf16", 2: "split_bf16", 3: "split_bf16_scaled", 4: "fp16", 5: "fp64"}
LLOYD_FIXED_ITERS = 1


class Stats(ctypes.Structure):
    _fields_ = [
        ("device_ms", ctypes.c_double),
        ("h2d_bytes", ctypes.c_int64),
        ("d2h_bytes", ctypes.c_int64),
        ("distance_evals", ctypes.c_int64),
        ("rescored", ctypes.c_int64),
        ("iterations", ctypes.c_int32),
        ("precision_used", ctypes.c_int32),
        ("hot_kernel_ms", ctypes.c_double),
        ("hot_kernel_launches", ctypes.c_int32),
        ("kernel_launches", ctypes.c_int32),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ErrorReport(ctypes.Structure):
    """fuelg_error_report (include/fuelg.h)."""
    _fields_ = [("max_abs_err", ctypes.c_double), ("max_rel_err", ctypes.c_double), ("pairs", ctypes.c_int64),
                ("near_ties", ctypes.c_int64), ("order_flips", ctypes.c_int64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class KnnSet(ctypes.Structure):
    """fuelg_knn_set (include/fuelg.h)."""
    _fields_ = [("data", ctypes.c_void_p), ("n", ctypes.c_int64), ("d", ctypes.c_int32), ("metric", ctypes.c_int32),
                ("queries", ctypes.c_void_p), ("m", ctypes.c_int64), ("k", ctypes.c_int32),
                ("exclude_mode", ctypes.c_int32), ("out_idx", ctypes.c_void_p), ("out_dist", ctypes.c_void_p),
                ("status", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class KMeansProblem(ctypes.Structure):
    """fuelg_kmeans_problem (include/fuelg.h)."""
    _fields_ = [("data", ctypes.c_void_p), ("n", ctypes.c_int64), ("d", ctypes.c_int32), ("k", ctypes.c_int32),
                ("init", ctypes.c_void_p), ("out_centers", ctypes.c_void_p), ("out_labels", ctypes.c_void_p),
                ("out_iters", ctypes.c_int32), ("status", ctypes.c_int32), ("out_inertia", ctypes.c_double)]


_lib = None

# name -> (restype, argtypes); kept in step with include/fuelg.h
_vp, _i32, _i64, _dbl = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
_pp = ctypes.POINTER(ctypes.c_void_p)
SIGNATURES = {
    "fuelg_last_error": (ctypes.c_char_p, []),
    "fuelg_version": (ctypes.c_char_p, []),
    "fuelg_device_count": (ctypes.c_int, [ctypes.POINTER(_i32)]),
    "fuelg_index_create": (ctypes.c_int, [_vp, _i64, _i32, _i32, _i32, _pp]),
    "fuelg_index_destroy": (ctypes.c_int, [_vp]),
    "fuelg_index_info": (ctypes.c_int, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i32), ctypes.POINTER(_i32),
                                        ctypes.POINTER(_i32)]),
    "fuelg_knn": (ctypes.c_int, [_vp, _vp, _i64, _i32, _i32, _i32, _vp, _vp, ctypes.POINTER(Stats)]),
    "fuelg_knn_ties": (ctypes.c_int, [_vp, _vp, _i64, _i32, _i32, _i32, _pp, ctypes.POINTER(Stats)]),
    "fuelg_knn_batched": (ctypes.c_int, [_vp, _i32, _i32, _i32, ctypes.POINTER(Stats)]),
    "fuelg_knn_error": (ctypes.c_int, [_vp, _vp, _i64, _i32, _vp, _vp, ctypes.POINTER(ErrorReport)]),
    "fuelg_fp32_rate": (ctypes.c_int, [ctypes.POINTER(_dbl)]),
    "fuelg_range": (ctypes.c_int, [_vp, _vp, _i64, _dbl, _i32, _pp, ctypes.POINTER(Stats)]),
    "fuelg_range_size": (ctypes.c_int, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "fuelg_range_copy": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "fuelg_range_free": (ctypes.c_int, [_vp]),
    "fuelg_pairwise": (ctypes.c_int, [_vp, _i64, _i32, _i32, _i32, _i32, _vp, ctypes.POINTER(Stats)]),
    "fuelg_kmeans_lloyd": (ctypes.c_int, [_vp, _i64, _i32, _i32, _vp, _i32, _dbl, _i32, _i32, _i32, _vp, _vp,
                                          ctypes.POINTER(_i32), ctypes.POINTER(_dbl), ctypes.POINTER(Stats)]),
    "fuelg_lloyd_assign": (ctypes.c_int, [_vp, _i64, _i32, _vp, _i32, _i32, _i32, _vp, _vp, ctypes.POINTER(Stats)]),
    "fuelg_kmeans_batched": (ctypes.c_int, [_vp, _i32, _i32, _i32, _i32, _i32, ctypes.POINTER(Stats)]),
    "fuelg_server_create": (ctypes.c_int, [_vp, _i32, _i64, _i64, _i32, ctypes.POINTER(_vp)]),
    "fuelg_server_submit": (ctypes.c_int, [_vp, _vp, _i64, _i32, _vp, _vp, ctypes.POINTER(_i64)]),
    "fuelg_server_wait": (ctypes.c_int, [_vp, _i64, _i32, ctypes.POINTER(_dbl)]),
    "fuelg_server_stats": (ctypes.c_int, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64), ctypes.POINTER(_i64),
                                          ctypes.POINTER(_i64), ctypes.POINTER(_dbl)]),
    "fuelg_server_destroy": (ctypes.c_int, [_vp]),
    "fuelg_knn_noalloc": (ctypes.c_int, [_vp, _i64, _i32, _vp, _i64, _i32, _i32, _i32, _i32, _vp, _vp, _vp]),
    "fuelg_cancel": (ctypes.c_int, []),
    "fuelg_reset_cancel": (ctypes.c_int, []),
    "fuelg_release": (ctypes.c_int, []),
    "fuelg_index_create_f64": (ctypes.c_int, [_vp, _i64, _i32, _i32, _i32, _pp]),
    "fuelg_knn_f64": (ctypes.c_int, [_vp, _vp, _i64, _i32, _i32, _vp, _vp, ctypes.POINTER(Stats)]),
    "fuelg_knn_ties_f64": (ctypes.c_int, [_vp, _vp, _i64, _i32, _i32, _pp, ctypes.POINTER(Stats)]),
    "fuelg_range_f64": (ctypes.c_int, [_vp, _vp, _i64, _dbl, _i32, _pp, ctypes.POINTER(Stats)]),
    "fuelg_range_copy_f64": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "fuelg_pairwise_f64": (ctypes.c_int, [_vp, _i64, _i32, _i32, _i32, _i32, _vp, ctypes.POINTER(Stats)]),
}


def default_order() -> str:
    """Summation profile to reproduce: FUEL_GB300_ORDER, else the one fuel
    compiles for this host's ISA (x86_64 -> 'x86', anything else -> 'arm')."""
    env = os.environ.get("FUEL_GB300_ORDER")
    if env:
        if env not in ORDER:
            raise ValueError(f"FUEL_GB300_ORDER must be one of {sorted(ORDER)}, got {env!r}")
        return env
    return "x86" if platform.machine().lower() in ("x86_64", "amd64") else "arm"


def load():
    """Load libfuelg.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build the CUDA engine first (python -m fuel_gb300.build); "
            "there is no CPU fallback")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    msg = load().fuelg_last_error()
    return msg.decode() if msg else ""


def check(rc: int):
    if rc == OK:
        return
    msg = last_error()
    if rc == EINVAL:
        raise ValueError(msg)
    if rc == ECANCELLED:
        raise KeyboardInterrupt(msg)
    if rc == ENOTSUP:
        raise NotImplementedError(msg)
    if rc == ENOMEM:
        raise MemoryError(msg)
    raise RuntimeError(f"fuelg error {rc}: {msg}")


def device_count() -> int:
    n = ctypes.c_int32(0)
    check(load().fuelg_device_count(ctypes.byref(n)))
    return int(n.value)


def release():
    """Free what the engine keeps between calls (fuelg_release): its memory
    pool, the Lloyd loop's kept CUDA graphs, the cancellation word.  Call it
    with no call in flight and every index and server closed, e.g. before
    resetting the device; ValueError while a server is open."""
    check(load().fuelg_release())


def ptr(a) -> ctypes.c_void_p:
    """Address of a numpy array or torch tensor (host or CUDA)."""
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)
