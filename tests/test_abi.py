"""The C-ABI library: it loads, exports every symbol include/fuelg.h declares,
and fails loudly (no CPU fallback) where no GPU is visible.  No compute calls."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "fuelg.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fuelg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_api():
    names = declared_functions()
    for must in ("fuelg_index_create", "fuelg_knn", "fuelg_range", "fuelg_kmeans_lloyd", "fuelg_cancel",
                 "fuelg_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} declared in include/fuelg.h but not exported"


def test_python_binding_covers_header():
    from fuel_gb300 import _lib
    assert set(_lib.SIGNATURES) == set(declared_functions())


def test_stats_struct_layout_matches_header():
    from fuel_gb300 import _lib
    text = open(HEADER).read()
    body = text[text.index("typedef struct {"):text.index("} fuelg_stats;")]
    fields = re.findall(r"(double|int64_t|int32_t)\s+([a-z_0-9]+);", body)
    assert [f for _, f in fields] == [f for f, _ in _lib.Stats._fields_]


def test_version_and_device_count(lib):
    from fuel_gb300 import _lib
    assert b"sm_103a" in lib.fuelg_version()
    assert _lib.device_count() >= 0


def test_no_cpu_fallback_without_gpu(lib):
    from fuel_gb300 import _lib
    if _lib.device_count() > 0:
        pytest.skip("a GPU is visible; the no-GPU error path is not reachable")
    h = ctypes.c_void_p()
    X = np.zeros((4, 3), np.float32)
    rc = lib.fuelg_index_create(_lib.ptr(X), 4, 3, 0, 0, ctypes.byref(h))
    assert rc == _lib.ENODEV
    assert "no CUDA device" in _lib.last_error()
    X64 = X.astype(np.float64)
    assert lib.fuelg_index_create_f64(_lib.ptr(X64), 4, 3, 0, 0, ctypes.byref(h)) == _lib.ENODEV
    import fuel_gb300
    with pytest.raises(RuntimeError):
        fuel_gb300.SearchIndex(X, tree="linear")
    with pytest.raises(RuntimeError):
        fuel_gb300.SearchIndex(X64, tree="linear")
    with pytest.raises(RuntimeError):
        fuel_gb300.kmeans(X, k=2, variant="lloyd", init="first")


def test_argument_validation_before_any_device_work(lib):
    from fuel_gb300 import _lib
    h = ctypes.c_void_p()
    assert lib.fuelg_index_create(None, 4, 3, 0, 0, ctypes.byref(h)) == _lib.EINVAL
    assert lib.fuelg_index_create(None, 0, 3, 7, 0, ctypes.byref(h)) == _lib.EINVAL
    assert lib.fuelg_knn(None, None, 0, 1, 0, 0, None, None, None) == _lib.EINVAL
    assert lib.fuelg_kmeans_lloyd(None, 0, 1, 1, None, 1, 0.0, 0, 0, 0, None, None, None, None, None) == _lib.EINVAL
    assert lib.fuelg_lloyd_assign(None, 0, 1, None, 1, 0, 0, None, None, None) == _lib.EINVAL
    assert lib.fuelg_range_free(None) == _lib.OK
    assert lib.fuelg_index_destroy(None) == _lib.OK
    assert lib.fuelg_release() == _lib.OK  # nothing kept yet: a no-op
    assert lib.fuelg_index_create_f64(None, 4, 3, 0, 0, ctypes.byref(h)) == _lib.EINVAL
    assert lib.fuelg_knn_f64(None, None, 0, 1, 0, None, None, None) == _lib.EINVAL
    assert lib.fuelg_knn_ties_f64(None, None, 0, 1, 0, None, None) == _lib.EINVAL
    assert lib.fuelg_range_f64(None, None, 0, 1.0, 0, None, None) == _lib.EINVAL
    assert lib.fuelg_range_copy_f64(None, None, None, None) == _lib.EINVAL
    assert lib.fuelg_pairwise_f64(None, 3, 0, 0, 0, 0, None, None) == _lib.EINVAL


def test_rust_bindings_declare_every_header_function():
    """rust/fuel-gb300-sys declares exactly the functions of include/fuelg.h."""
    import re
    src = open(os.path.join(ROOT, "rust", "fuel-gb300-sys", "src", "lib.rs")).read()
    rust = set(re.findall(r"pub fn (fuelg_\w+)\(", src))
    assert rust == set(declared_functions())
