"""Sharded kNN, range search and Lloyd k-means across ranks (one process per
GPU): the exchange step between shards.

fuel itself is single-process (rayon threads over one shared array); this
module is the host-side logic a multi-GPU deployment of the engine needs.
Every rank holds a contiguous slice of the index rows (or of the k-means
points); the results are identical to the single-shard ones:

* kNN: each shard returns its local top-(k+1) by (distance, index) with
  global indices; merging those lists and applying fuel's KNNHeap tie rule
  and exclude-self rule reproduces the unsharded answer exactly
  (src/api/search.rs:80-151, python/search.rs:485-488, 1195-1216).
* range search: disjoint per-shard hit lists, concatenated and ordered by
  (distance, index) (src/api/search.rs:154-166).
* Lloyd: the centroid update uses exact integer sums (every f32 coordinate
  is an integer multiple of 2**e_lo), so the all-reduce of the per-shard
  sums is exact and order-independent and the correctly rounded means are
  bit-identical to the single-device ones; counts and the changed-point
  count are integers; the FP64 inertia is the only order-dependent value.

The collectives go through torch.distributed (gloo on CPU, NCCL on GPUs);
`group=None` with world size 1 runs without a process group.  The local
compute is a callable, so the same exchange logic serves the GPU engine and
a CPU implementation.
"""
from __future__ import annotations

import math
from typing import Callable, Sequence

import numpy as np

INF32 = np.float32(np.inf)
_BIG = np.iinfo(np.int64).max


# --------------------------------------------------------------------------
# process-group helpers
# --------------------------------------------------------------------------

def _world(group=None):
    try:
        import torch.distributed as dist
        if dist.is_available() and dist.is_initialized():
            return dist.get_world_size(group), dist.get_rank(group)
    except ImportError:
        pass
    return 1, 0


def _all_gather_np(a: np.ndarray, group=None) -> list[np.ndarray]:
    """All-gather of equally shaped arrays (int64 / float32 / float64)."""
    world, _ = _world(group)
    if world == 1:
        return [a]
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(a))
    out = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(out, t, group=group)
    return [o.numpy() for o in out]


def _all_gather_var(a: np.ndarray, group=None) -> list[np.ndarray]:
    """All-gather of 1-D arrays whose lengths differ between ranks."""
    world, _ = _world(group)
    if world == 1:
        return [a]
    lens = _all_gather_np(np.array([a.shape[0]], np.int64), group)
    mx = int(max(int(x[0]) for x in lens))
    pad = np.zeros((mx,), a.dtype)
    pad[: a.shape[0]] = a
    parts = _all_gather_np(pad, group)
    return [p[: int(n[0])] for p, n in zip(parts, lens)]


def _all_reduce_np(a: np.ndarray, op: str = "sum", group=None) -> np.ndarray:
    world, _ = _world(group)
    if world == 1:
        return a
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(a).copy())
    dist.all_reduce(t, op={"sum": dist.ReduceOp.SUM, "min": dist.ReduceOp.MIN, "max": dist.ReduceOp.MAX}[op],
                    group=group)
    return t.numpy()


# --------------------------------------------------------------------------
# kNN
# --------------------------------------------------------------------------

def shard_bounds(n: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous row range [lo, hi) of shard `rank` (sizes differ by <= 1)."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def _sort_rows(idx: np.ndarray, dist: np.ndarray):
    """Sort every row by (distance, index); padding (-1, +inf) last."""
    key_i = np.where(idx < 0, _BIG, idx)
    d = dist + np.float32(0.0)  # -0.0 -> +0.0: fuel compares with partial_cmp
    order = np.lexsort((key_i, d), axis=-1)
    return np.take_along_axis(idx, order, -1), np.take_along_axis(d, order, -1)


def merge_knn(parts: Sequence[tuple[np.ndarray, np.ndarray]], k: int, exclude_mode: int = 0,
              query_index: np.ndarray | None = None) -> tuple[np.ndarray, np.ndarray]:
    """Merge per-shard candidate lists into fuel's kNN result.

    parts: per shard (idx int64 [m, c], dist float32 [m, c]) with GLOBAL
    indices, each row the shard's top-c by (distance, index) with -1 / +inf
    padding, c >= k + 1 (exactly k + 1 suffices).  exclude_mode: 0 none;
    1 = fuel's linear path (search k, drop the query's own index, ties at the
    k-th distance fill in: python/search.rs:485-488 with KNNHeap's tie list);
    2 = the precomputed path (search k + 1, drop self, truncate:
    python/search.rs:1163-1170).  query_index: global index of each query row
    (required for modes 1 and 2).  Returns (int64 [m, k], float32 [m, k])
    padded like knn_results_to_arrays (python/search.rs:1195-1216)."""
    if not parts:
        raise ValueError("merge_knn: no shards")
    idx = np.concatenate([np.asarray(p[0], np.int64) for p in parts], axis=1)
    dist = np.concatenate([np.asarray(p[1], np.float32) for p in parts], axis=1)
    m = idx.shape[0]
    need = k + 1
    if idx.shape[1] < need:
        pi = np.full((m, need - idx.shape[1]), -1, np.int64)
        pdd = np.full((m, need - idx.shape[1]), INF32, np.float32)
        idx, dist = np.concatenate([idx, pi], 1), np.concatenate([dist, pdd], 1)
    idx, dist = _sort_rows(idx, dist)
    idx, dist = idx[:, :need], dist[:, :need]
    out_i = np.full((m, k), -1, np.int64)
    out_d = np.full((m, k), INF32, np.float32)
    if k == 0:
        return out_i, out_d
    if exclude_mode == 0:
        out_i[:], out_d[:] = idx[:, :k], dist[:, :k]
        return out_i, out_d
    if query_index is None:
        raise ValueError("merge_knn: exclude_mode needs query_index")
    qi = np.asarray(query_index, np.int64).reshape(m, 1)
    real = idx >= 0
    if exclude_mode == 1:
        # KNNHeap(k) result = the k best plus every later entry tied with the k-th
        kth = dist[:, k - 1:k]
        keep = real.copy()
        keep[:, k] &= (dist[:, k] == kth[:, 0]) & real[:, k - 1]
    elif exclude_mode == 2:
        keep = real.copy()
    else:
        raise ValueError(f"merge_knn: bad exclude_mode {exclude_mode}")
    keep &= idx != qi
    for r in range(m):
        sel = np.nonzero(keep[r])[0][:k]
        out_i[r, : sel.size] = idx[r, sel]
        out_d[r, : sel.size] = dist[r, sel]
    return out_i, out_d


def sharded_knn(local_knn: Callable[[np.ndarray, int], tuple[np.ndarray, np.ndarray]], row_offset: int,
                queries: np.ndarray, k: int, exclude_mode: int = 0, query_index: np.ndarray | None = None,
                group=None) -> tuple[np.ndarray, np.ndarray]:
    """kNN over an index split across ranks.  local_knn(queries, c) searches
    this rank's shard (local indices, -1/+inf padding, no self exclusion) and
    returns c columns; row_offset is the shard's first global row.  Every
    rank passes the same queries and gets the full result."""
    li, ld = local_knn(queries, k + 1)
    li = np.asarray(li, np.int64)
    gi = np.where(li >= 0, li + row_offset, -1)
    gi_all = _all_gather_np(gi, group)
    gd_all = _all_gather_np(np.asarray(ld, np.float32), group)
    return merge_knn(list(zip(gi_all, gd_all)), k, exclude_mode, query_index)


def merge_range(parts: Sequence[tuple[np.ndarray, np.ndarray, np.ndarray]]):
    """Per-shard CSR range results (offsets [m+1], idx, dist) with global
    indices -> one CSR result, each query's hits ordered by (distance, index)."""
    m = len(parts[0][0]) - 1
    offs = np.zeros(m + 1, np.int64)
    idx_out, dist_out = [], []
    for q in range(m):
        ii = np.concatenate([np.asarray(p[1][p[0][q]:p[0][q + 1]], np.int64) for p in parts])
        dd = np.concatenate([np.asarray(p[2][p[0][q]:p[0][q + 1]], np.float32) for p in parts])
        o = np.lexsort((ii, dd + np.float32(0.0)))
        idx_out.append(ii[o])
        dist_out.append(dd[o])
        offs[q + 1] = offs[q] + ii.size
    return offs, (np.concatenate(idx_out) if idx_out else np.zeros(0, np.int64)), \
        (np.concatenate(dist_out) if dist_out else np.zeros(0, np.float32))


def sharded_range(local_range, row_offset: int, queries: np.ndarray, radius: float, group=None):
    """Range search over an index split across ranks; local_range(queries,
    radius) -> (offsets, idx, dist) in local indices (no self exclusion)."""
    off, ii, dd = local_range(queries, radius)
    off = np.asarray(off, np.int64)
    gi = np.asarray(ii, np.int64) + row_offset
    offs = _all_gather_np(off, group)
    idxs = _all_gather_var(gi, group)
    dists = _all_gather_var(np.asarray(dd, np.float32), group)
    return merge_range(list(zip(offs, idxs, dists)))


# --------------------------------------------------------------------------
# Lloyd: exact integer centroid sums
# --------------------------------------------------------------------------

LIMB = 24  # bits per limb; a 24-bit mantissa shifted by < 24 spans two limbs


def _decompose(X: np.ndarray):
    """f32 -> (sign, 24-bit mantissa, unit exponent): x = sign * mant * 2**unit."""
    bits = np.ascontiguousarray(X, np.float32).view(np.uint32).astype(np.int64)
    eb = (bits >> 23) & 0xFF
    if np.any(eb == 0xFF):
        raise ValueError("sharded Lloyd: non-finite input")
    mant = (bits & 0x7FFFFF) | np.where(eb != 0, 1 << 23, 0)
    unit = np.where(eb == 0, -149, eb - 150)
    sign = np.where((bits >> 31) & 1, -1, 1)
    return sign, mant, unit


class ExactSums:
    """Exact per-cluster coordinate sums of a shard, as int64 limbs of LIMB
    bits at the common scale 2**e_lo (agreed by all ranks)."""

    def __init__(self, X: np.ndarray, group=None):
        self.X = np.ascontiguousarray(X, np.float32)
        self.group = group
        sign, mant, unit = _decompose(self.X)
        nz = mant != 0
        lo = np.array([int(unit[nz].min()) if nz.any() else 1 << 20], np.int64)
        hi = np.array([int(unit[nz].max()) if nz.any() else -(1 << 20)], np.int64)
        self.e_lo = int(_all_reduce_np(lo, "min", group)[0])
        e_hi = int(_all_reduce_np(hi, "max", group)[0])
        if self.e_lo > e_hi:  # all data zero
            self.e_lo, e_hi = 0, 0
        shift = np.where(nz, unit - self.e_lo, 0)
        self.L = (e_hi - self.e_lo) // LIMB + 2
        limb = shift // LIMB
        v = mant << (shift % LIMB)  # < 2**47
        self.lo_part = (sign * (v & ((1 << LIMB) - 1))).astype(np.float64)
        self.hi_part = (sign * (v >> LIMB)).astype(np.float64)
        self.limb = limb

    def local(self, labels: np.ndarray, k: int):
        """(sums int64 [k, d, L], counts int64 [k]) of this shard.  The float64
        bin sums are exact: addends < 2**24 in magnitude, < 2**29 of them."""
        n, d = self.X.shape
        if n >= (1 << 29):
            raise ValueError("sharded Lloyd: shard too large for exact float64 bin sums")
        lab = np.asarray(labels, np.int64)
        cell = (lab[:, None] * d + np.arange(d)[None, :]) * self.L
        nb = k * d * self.L
        s = np.bincount((cell + self.limb).ravel(), weights=self.lo_part.ravel(), minlength=nb)
        s += np.bincount((cell + self.limb + 1).ravel(), weights=self.hi_part.ravel(), minlength=nb)
        cnt = np.bincount(lab, minlength=k).astype(np.int64)
        return s.astype(np.int64).reshape(k, d, self.L), cnt

    def means(self, sums: np.ndarray, counts: np.ndarray, prev: np.ndarray) -> np.ndarray:
        """Correctly rounded (RNE) f32 means; empty clusters keep their centre
        (src/cluster/kmeans/lloyd.rs:160-176)."""
        k, d, L = sums.shape
        C = np.array(prev, np.float32, copy=True)
        w = [1 << (LIMB * j) for j in range(L)]
        for c in range(k):
            cnt = int(counts[c])
            if cnt == 0:
                continue
            row = sums[c]
            for j in range(d):
                S = 0
                for t in range(L):
                    lv = int(row[j, t])
                    if lv:
                        S += lv * w[t]
                C[c, j] = rne_f32_ratio(S, cnt, self.e_lo)
        return C


def rne_f32_ratio(S: int, cnt: int, e: int) -> np.float32:
    """S * 2**e / cnt rounded to nearest-even f32 (S, cnt integers, cnt > 0):
    27+ quotient bits plus the remainder decide the rounding; the result is
    a normal or subnormal f32 (the data are f32, so the mean is in range)."""
    if S == 0:
        return np.float32(0.0)
    neg = S < 0
    A = -S if neg else S
    # scale so that the quotient has at least 26 significant bits
    sh = max(0, 26 - (A.bit_length() - cnt.bit_length()))
    q, r = divmod(A << sh, cnt)
    exp = q.bit_length() - 1 + e - sh  # floor(log2(value)) (q >= 2**25)
    if exp < -150:  # below half the smallest subnormal
        return np.float32(-0.0 if neg else 0.0)
    keep = 24 if exp >= -126 else exp + 150  # subnormals: bits down to 2**-149
    drop = q.bit_length() - keep
    mant, rem = q >> drop, q & ((1 << drop) - 1)
    half = 1 << (drop - 1)
    if rem > half or (rem == half and (r != 0 or (mant & 1))):
        mant += 1
    v = np.float32(math.ldexp(float(mant), drop + e - sh))
    return -v if neg else v


def sharded_lloyd(X_local: np.ndarray, k: int, init: np.ndarray,
                  assign: Callable[[np.ndarray, np.ndarray, bool], np.ndarray], max_iter: int = 300,
                  fixed_iters: bool = False, group=None):
    """Lloyd k-means over points split across ranks, following
    src/cluster/kmeans/lloyd.rs:118-202 (iteration 1 = initial assignment,
    stop when no label changed, or after max_iter; centres updated between
    assignments, empty clusters keep their centre).  assign(X, centres,
    initial) -> labels of this shard (fuel's arithmetic: pairwise order on
    the initial pass, math::sqdist order later, first index wins ties).
    Returns (centres f32 [k, d], local labels int64, iterations, changed in
    the last iteration, FP64 inertia over all shards)."""
    X = np.ascontiguousarray(X_local, np.float32)
    C = np.ascontiguousarray(init, np.float32).copy()
    es = ExactSums(X, group)

    def update(labels, prev):
        s, c = es.local(labels, k)
        s = _all_reduce_np(s, "sum", group)
        c = _all_reduce_np(c, "sum", group)
        return es.means(s, c, prev)

    labels = np.asarray(assign(X, C, True), np.int64)
    if max_iter > 1:
        C = update(labels, C)
    it, changed = 1, 0
    while it < max_iter:
        it += 1
        new = np.asarray(assign(X, C, False), np.int64)
        changed = int(_all_reduce_np(np.array([(new != labels).sum()], np.int64), "sum", group)[0])
        labels = new
        if it < max_iter:
            C = update(labels, C)
        if not fixed_iters and changed == 0:
            break
    diff = X.astype(np.float64) - C.astype(np.float64)[labels]
    inertia = float(_all_reduce_np(np.array([np.einsum("ij,ij->", diff, diff)]), "sum", group)[0])
    return C, labels, it, changed, inertia
