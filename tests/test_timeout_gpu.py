"""A bounded device wait that runs out.

Every mbarrier wait of the tensor-core kernels is bounded; on expiry the
kernel records a timeout in the call's status word, stops all its roles,
waits (with the full 4 s bound) for its own copies and MMAs, frees its tensor
memory and returns, and the call reports FUELG_ETIMEOUT.  FUELG_WAIT_LIMIT_NS
shortens the pipeline waits of one launch (the drain waits keep their bound)
so that they run out on an ordinary call: nothing is faulted, and the next
call on the same index must return the exact answer."""
import numpy as np
import pytest

from conftest import f32_bits, threads
from fuel_gb300 import SearchIndex, _lib

pytestmark = pytest.mark.gpu


def test_pipeline_wait_runs_out_and_the_next_call_is_clean(gpu, oracle, monkeypatch):
    rng = np.random.default_rng(6)
    # integer data: the exact BF16 screen, whose follow-up kernels only move keys
    X = np.minimum(rng.geometric(0.15, size=(200000, 64)) - 1, 255).astype(np.float32)
    Q = X[:4096].copy()
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear", precision="bf16")
    monkeypatch.setenv("FUELG_WAIT_LIMIT_NS", "1")
    with pytest.raises(RuntimeError, match="timed out"):
        ix.knn(Q, 10, exclude_self=False)
    monkeypatch.delenv("FUELG_WAIT_LIMIT_NS")
    gi, gd = ix.knn(Q, 10, exclude_self=False)
    assert ix.last_stats["precision_used"] == 1
    ci, cd = oracle.knn(X, Q, 10, threads=threads())
    assert np.array_equal(gi, ci) and np.array_equal(f32_bits(gd), f32_bits(cd))
    # and the library's other paths still run on this context
    assert _lib.device_count() >= 1
