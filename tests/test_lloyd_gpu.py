"""Parity of GPU Lloyd k-means with the restated fuel CPU path.

Per iteration (the primary bar): given the same centres, the GPU assignment is
bit-identical to fuel's (iteration 1 in the vec_pairwise_sqdist order,
later iterations in the math::sqdist order, strict '<' so the lowest index
wins ties).  Whole runs: the GPU keeps exact integer centroid sums and sets
every centre to the correctly rounded f32 of the exact mean, so it is compared
bit-for-bit (labels, iteration count, centre bits) with the exact-mean Lloyd
oracle, with inertia within 1e-7 relative of the FP64 value; fuel's own
f32-sums Lloyd is checked to land on the same partition.
"""
import numpy as np
import pytest

from conftest import threads
from fuel_gb300 import kmeans, workloads

pytestmark = pytest.mark.gpu


def ulp_diff(a, b):
    ai = np.ascontiguousarray(a, np.float32).view(np.int32).astype(np.int64)
    bi = np.ascontiguousarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(ai - bi).max() if a.size else 0


def mixture(n, d, k, seed):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-10, 10, size=(k, d))
    return (c[rng.integers(0, k, n)] + rng.normal(size=(n, d))).astype(np.float32)


@pytest.mark.parametrize("order", ["arm", "x86"])
@pytest.mark.parametrize("d,k", [(2, 4), (3, 7), (8, 16), (32, 10), (64, 33), (784, 64)])
def test_per_iteration_assignment_bit_exact(gpu, oracle, order, d, k):
    n = 3000 if d < 784 else 1500
    X = mixture(n, d, k, d * 100 + k)
    init = X[np.random.default_rng(1).choice(n, k, replace=False)]
    for t in (1, 2, 3, 6):
        r = kmeans(X, k=k, variant="lloyd", max_iter=t, init=init, order=order, fixed_iters=True)
        lab, _ = oracle.lloyd_assign(X, r.centers, initial=(t == 1), order=order, threads=threads())
        assert np.array_equal(r.labels, lab), f"iteration {t}: {np.sum(r.labels != lab)} labels differ"


@pytest.mark.parametrize("order", ["arm", "x86"])
def test_full_run_vs_exact_oracle(gpu, oracle, order):
    X = mixture(4000, 16, 12, 5)
    init = X[:12].copy()
    r = kmeans(X, k=12, variant="lloyd", max_iter=100, init=init, order=order)
    c, lab, it, inert = oracle.lloyd_exact(X, 12, init, max_iter=100, order=order, threads=threads())
    assert r.n_iter == it
    assert np.array_equal(r.labels, lab)
    assert np.array_equal(r.centers.view(np.uint32), c.view(np.uint32))
    assert abs(r.inertia - inert) <= 1e-7 * inert
    # fuel's own f32-sums trajectory lands on the same partition here
    c2, lab2, it2, _ = oracle.lloyd(X, 12, init, max_iter=100, order=order, threads=8)
    assert np.array_equal(r.labels, lab2)


@pytest.mark.parametrize("precision", ["fp32", "split_bf16"])
def test_lloyd_sparse_config_reduced(gpu, oracle, precision):
    """The k=64, d=784 sparse 0..255/255 workload at n=7,000, 10 iterations."""
    X, init = workloads.lloyd_sparse(n=7000)
    r = kmeans(X, k=64, variant="lloyd", max_iter=10, init=init, fixed_iters=True, precision=precision)
    # 8-bit values / 255: the split tier runs on the exact scaled-integer copy
    assert r.stats["precision_used"] == {"fp32": 0, "split_bf16": 3}[precision]
    c, lab, it, inert = oracle.lloyd_exact(X, 64, init, max_iter=10, threads=threads(), fixed_iters=True)
    assert r.n_iter == 10 == it
    assert np.array_equal(r.labels, lab)
    assert np.array_equal(r.centers.view(np.uint32), c.view(np.uint32))
    assert abs(r.inertia - inert) <= 1e-7 * inert


def test_wide_exponent_range_uses_fp64_sums(gpu, oracle):
    """Data spanning more than 128 bits of exponent falls back to FP64 sums;
    assignments stay bit-exact per iteration."""
    X = mixture(1500, 6, 5, 3)
    X[::7, 0] *= np.float32(1e-30)
    X[::11, 1] *= np.float32(1e25)
    init = X[np.random.default_rng(0).choice(1500, 5, replace=False)]
    for t in (1, 2, 4):
        r = kmeans(X, k=5, variant="lloyd", max_iter=t, init=init, fixed_iters=True)
        lab, _ = oracle.lloyd_assign(X, r.centers, initial=(t == 1), threads=threads())
        assert np.array_equal(r.labels, lab)


@pytest.mark.parametrize("scale_bits", [(-20, 20), (-45, 30)])
def test_multi_limb_exact_sums(gpu, oracle, scale_bits):
    """Exponent ranges that need 2-3 limbs of exact sums (quotients beyond 64
    bits in the mean rounding): centres and labels bit-exact against the
    exact-mean oracle, plain and tensor-core tiers."""
    lo, hi = scale_bits
    X = mixture(2000, 40, 6, 11)
    rng = np.random.default_rng(12)
    X *= np.exp2(rng.integers(lo, hi, size=X.shape)).astype(np.float32)
    init = X[:6].copy()
    c, lab, it, _ = oracle.lloyd_exact(X, 6, init, max_iter=5, threads=threads(), fixed_iters=True)
    for prec in ("fp32", "split_bf16"):
        r = kmeans(X, k=6, variant="lloyd", max_iter=5, init=init, fixed_iters=True, precision=prec)
        assert np.array_equal(r.labels, lab)
        assert np.array_equal(r.centers.view(np.uint32), c.view(np.uint32))


def test_fixed_iters_and_stop_rule(gpu):
    X = mixture(2000, 4, 3, 9)
    r1 = kmeans(X, k=3, variant="lloyd", max_iter=50, init="first")
    assert r1.n_iter < 50
    r2 = kmeans(X, k=3, variant="lloyd", max_iter=50, init="first", fixed_iters=True)
    assert r2.n_iter == 50
    assert np.array_equal(r1.labels, r2.labels)
    r3 = kmeans(X, k=3, variant="lloyd", max_iter=50, init="first", tol=1e-3)
    assert r3.n_iter <= r1.n_iter


def test_edge_cases(gpu, oracle):
    X = np.array([[0.0], [1.0], [2.0], [10.0]], np.float32)
    # duplicate initial centre: centre 1 loses every tie and stays empty
    init = np.array([[1.0], [1.0], [10.0]], np.float32)
    r = kmeans(X, k=3, variant="lloyd", max_iter=5, init=init)
    c, lab, it, _ = oracle.lloyd_exact(X, 3, init, max_iter=5)
    assert np.array_equal(r.labels, lab) and r.n_iter == it
    assert r.centers[1, 0] == 1.0
    # k = 1 and k = n
    r1 = kmeans(X, k=1, variant="lloyd", init="first")
    assert (r1.labels == 0).all() and np.isclose(r1.centers[0, 0], 3.25)
    rn = kmeans(X, k=4, variant="lloyd", init="first")
    assert rn.labels.tolist() == [0, 1, 2, 3] and rn.inertia == 0.0
    # max_iter = 1: only the initial assignment, centres are the init
    r0 = kmeans(X, k=2, variant="lloyd", max_iter=1, init="first")
    assert r0.n_iter == 1 and np.array_equal(r0.centers, X[:2])


def test_deterministic(gpu):
    X, init = workloads.lloyd_sparse(n=5000)
    a = kmeans(X, k=64, variant="lloyd", max_iter=5, init=init)
    b = kmeans(X, k=64, variant="lloyd", max_iter=5, init=init)
    assert np.array_equal(a.labels, b.labels)
    assert np.array_equal(a.centers.view(np.uint32), b.centers.view(np.uint32))
    assert a.inertia == b.inertia


# ---------------------------------------------------------------------------
# Tensor-core tiers: BF16 / split-BF16 screen + exact re-score must give the
# same assignment as the exact path, iteration by iteration.
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("precision", ["bf16", "split_bf16"])
@pytest.mark.parametrize("order", ["arm", "x86"])
@pytest.mark.parametrize("d,k", [(32, 10), (64, 33), (100, 64), (784, 64), (128, 256), (40, 17)])
def test_tc_tier_per_iteration_bit_exact(gpu, oracle, precision, order, d, k):
    n = 3000 if d < 784 else 2000
    X = mixture(n, d, k, d * 7 + k)
    init = X[np.random.default_rng(2).choice(n, k, replace=False)]
    for t in (1, 2, 4):
        r = kmeans(X, k=k, variant="lloyd", max_iter=t, init=init, order=order, fixed_iters=True,
                   precision=precision)
        assert r.stats["precision_used"] == {"bf16": 1, "split_bf16": 2}[precision]
        lab, _ = oracle.lloyd_assign(X, r.centers, initial=(t == 1), order=order, threads=threads())
        assert np.array_equal(r.labels, lab), f"iteration {t}: {np.sum(r.labels != lab)} labels differ"


@pytest.mark.parametrize("precision", ["bf16", "split_bf16"])
def test_tc_tier_matches_exact_run(gpu, precision):
    X, init = workloads.lloyd_sparse(n=9000)
    a = kmeans(X, k=64, variant="lloyd", max_iter=12, init=init, fixed_iters=True)
    b = kmeans(X, k=64, variant="lloyd", max_iter=12, init=init, fixed_iters=True, precision=precision)
    assert np.array_equal(a.labels, b.labels)
    assert np.array_equal(a.centers.view(np.uint32), b.centers.view(np.uint32))
    assert a.inertia == b.inertia
    # the hi+lo screen decides almost every point without re-scoring
    if precision == "split_bf16":
        assert b.stats["rescored"] < 0.2 * 9000 * 12


def quantised(n, d, k, seed, scale=np.float32(0.37), top=200):
    """Integers in [-top, top] (cluster centres + noise, clipped) times one f32 scale."""
    rng = np.random.default_rng(seed)
    c = rng.integers(-top // 2, top // 2, size=(k, d))
    q = np.clip(c[rng.integers(0, k, n)] + rng.integers(-20, 21, size=(n, d)), -top, top)
    return (q.astype(np.float32) * scale).astype(np.float32)


@pytest.mark.parametrize("order", ["arm", "x86"])
@pytest.mark.parametrize("d,k", [(100, 20), (784, 64), (48, 130)])
def test_tc_scaled_integer_data_per_iteration(gpu, oracle, order, d, k, monkeypatch):
    """Split tier on integer-times-scale data: the point operand is exact in
    BF16 (one copy, two products); assignments stay bit-identical.  The same
    data forced through the plain split form agrees."""
    n = 2500
    X = quantised(n, d, k, d + k)
    init = X[np.random.default_rng(3).choice(n, k, replace=False)]
    for t in (1, 2, 4):
        r = kmeans(X, k=k, variant="lloyd", max_iter=t, init=init, order=order, fixed_iters=True,
                   precision="split_bf16")
        assert r.stats["precision_used"] == 3
        lab, _ = oracle.lloyd_assign(X, r.centers, initial=(t == 1), order=order, threads=threads())
        assert np.array_equal(r.labels, lab), f"iteration {t}: {np.sum(r.labels != lab)} labels differ"
    monkeypatch.setenv("FUELG_TC_NO_SCALED", "1")
    r2 = kmeans(X, k=k, variant="lloyd", max_iter=4, init=init, order=order, fixed_iters=True, precision="split_bf16")
    assert r2.stats["precision_used"] == 2
    assert np.array_equal(r2.labels, r.labels)
    assert np.array_equal(r2.centers.view(np.uint32), r.centers.view(np.uint32))


def test_tc_scaled_detection_rejects_off_grid_values(gpu, oracle):
    """One value off the integer grid: the plain split form is used, same result."""
    X = quantised(2000, 64, 10, 4)
    X[17, 5] += np.float32(0.001)
    init = X[:10].copy()
    r = kmeans(X, k=10, variant="lloyd", max_iter=5, init=init, fixed_iters=True, precision="split_bf16")
    assert r.stats["precision_used"] == 2
    c, lab, it, _ = oracle.lloyd_exact(X, 10, init, max_iter=5, threads=threads(), fixed_iters=True)
    assert np.array_equal(r.labels, lab)
    assert np.array_equal(r.centers.view(np.uint32), c.view(np.uint32))


def test_tc_tier_small_d_falls_back_to_exact(gpu):
    X = mixture(500, 8, 4, 1)
    r = kmeans(X, k=4, variant="lloyd", init="first", precision="bf16")
    assert r.stats["precision_used"] == 0


@pytest.mark.gpu
@pytest.mark.parametrize("initial", [True, False])
@pytest.mark.parametrize("n,d,k", [(1000, 3, 7), (3000, 40, 17), (513, 784, 64)])
def test_lloyd_assign_entry_point(oracle, gpu, initial, n, d, k):
    """fuelg_lloyd_assign: labels bit-exact and best distances bit-exact vs the
    oracle's assignment pass, in both the initial and the loop arithmetic."""
    from fuel_gb300 import lloyd_assign
    rng = np.random.default_rng(n + d + k)
    X = rng.normal(size=(n, d)).astype(np.float32)
    C = X[rng.choice(n, k, replace=False)].copy()
    C[1] = C[0]  # duplicate centre: the first index must win
    for order in ("arm", "x86"):
        lab, best = lloyd_assign(X, C, initial=initial, order=order)
        rl, rb = oracle.lloyd_assign(X, C, initial=initial, order=order)
        np.testing.assert_array_equal(lab, rl)
        np.testing.assert_array_equal(best.view(np.uint32), np.asarray(rb, np.float32).view(np.uint32))


@pytest.mark.gpu
def test_sharded_lloyd_with_engine_assign(oracle, gpu):
    """The sharded exchange driven by the GPU assignment reproduces the exact
    single-process Lloyd bit for bit (one process, world size 1)."""
    from fuel_gb300 import lloyd_assign, shard
    rng = np.random.default_rng(4)
    X = (rng.normal(size=(4000, 33)) + rng.integers(0, 4, size=(4000, 1)) * 3).astype(np.float32)
    init = X[rng.choice(4000, 9, replace=False)].copy()
    assign = lambda A, C, initial: lloyd_assign(A, C, initial=initial)[0]  # noqa: E731
    C, lab, it, _, inert = shard.sharded_lloyd(X, 9, init, assign, max_iter=20)
    rc, rl, rit, rinert = oracle.lloyd_exact(X, 9, init, max_iter=20)
    np.testing.assert_array_equal(C.view(np.uint32), rc.view(np.uint32))
    np.testing.assert_array_equal(lab, rl)
    assert it == rit
    assert abs(inert - rinert) <= 1e-9 * abs(rinert)


@pytest.mark.gpu
def test_pinned_host_inputs_match_device_inputs(gpu):
    """fuelg_kmeans_lloyd through the C ABI: pinned host inputs (aligned, and
    4 bytes off a 16-byte boundary) give the same centres, labels and inertia
    bits as device-resident inputs, and report their staged bytes."""
    torch = pytest.importorskip("torch")
    import ctypes
    from fuel_gb300 import _lib
    lib = _lib.load()
    n, d, k, iters = 6000, 64, 16, 12
    X, init = workloads.lloyd_sparse(n, d, k)
    assert X.nbytes >= 1 << 20

    def run(xp, cp):
        oc = np.empty((k, d), np.float32)
        ol = np.empty(n, np.int64)
        it, inert, st = ctypes.c_int32(), ctypes.c_double(), _lib.Stats()
        _lib.check(lib.fuelg_kmeans_lloyd(xp, n, d, k, cp, iters, 0.0, _lib.PRECISION["split_bf16"],
                                          _lib.ORDER["arm"], _lib.LLOYD_FIXED_ITERS, _lib.ptr(oc), _lib.ptr(ol),
                                          ctypes.byref(it), ctypes.byref(inert), ctypes.byref(st)))
        return oc, ol, inert.value, st.h2d_bytes

    Xd = torch.from_numpy(X).cuda()
    Cd = torch.from_numpy(init).cuda()
    ref = run(_lib.ptr(Xd), _lib.ptr(Cd))
    assert ref[3] == 0
    # aligned pinned buffers
    Xh = torch.empty((n, d), dtype=torch.float32, pin_memory=True)
    Xh.copy_(torch.from_numpy(X))
    Ch = torch.empty((k, d), dtype=torch.float32, pin_memory=True)
    Ch.copy_(torch.from_numpy(init))
    # a pinned buffer 4 bytes off a 16-byte boundary
    flat = torch.empty(n * d + 1, dtype=torch.float32, pin_memory=True)
    flat[1:].copy_(torch.from_numpy(X.ravel()))
    for xp in (_lib.ptr(Xh), ctypes.c_void_p(flat.data_ptr() + 4)):
        got = run(xp, _lib.ptr(Ch))
        assert got[3] == X.nbytes + init.nbytes
        np.testing.assert_array_equal(got[0].view(np.uint32), ref[0].view(np.uint32))
        np.testing.assert_array_equal(got[1], ref[1])
        assert got[2] == ref[2]
