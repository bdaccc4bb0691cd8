"""One rank of the sharded-exchange tests (gloo, CPU).  Run as
python tests/_shard_worker.py RANK WORLD PORT OUT_PREFIX; writes
OUT_PREFIX.RANK.npz.  The local search / assignment of each shard is the
CPU oracle; the exchange is fuel_gb300.shard."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402
import torch.distributed as dist  # noqa: E402

from fuel_gb300 import shard  # noqa: E402
from oracle import oracle  # noqa: E402


def data():
    """Shared inputs (every rank builds the same arrays)."""
    rng = np.random.default_rng(7)
    # small integers: many exact distance ties and duplicate points
    Xk = rng.integers(0, 4, size=(301, 5)).astype(np.float32)
    Xl = (rng.normal(size=(1500, 12)) + rng.integers(0, 3, size=(1500, 1)) * 4).astype(np.float32)
    init = Xl[rng.choice(1500, 6, replace=False)].copy()
    return Xk, Xl, init


def main():
    rank, world, port, out = int(sys.argv[1]), int(sys.argv[2]), int(sys.argv[3]), sys.argv[4]
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    Xk, Xl, init = data()
    res = {}
    lo, hi = shard.shard_bounds(len(Xk), world, rank)
    Xs = Xk[lo:hi]
    qidx = np.arange(len(Xk))
    for k in (1, 4, 9):
        for mode in (0, 1, 2):
            i, d = shard.sharded_knn(lambda Q, c: oracle.knn(Xs, Q, c), lo, Xk, k, mode, qidx)
            res[f"knn_{k}_{mode}_i"], res[f"knn_{k}_{mode}_d"] = i, d
    off, ii, dd = shard.sharded_range(lambda Q, r: oracle.range_search(Xs, Q, r), lo, Xk, 2.0)
    res["range_off"], res["range_idx"], res["range_dist"] = off, ii, dd
    lo, hi = shard.shard_bounds(len(Xl), world, rank)
    assign = lambda X, C, initial: oracle.lloyd_assign(X, C, initial=initial)[0]  # noqa: E731
    for fixed in (False, True):
        C, lab, it, chg, inert = shard.sharded_lloyd(Xl[lo:hi], 6, init, assign, max_iter=25, fixed_iters=fixed)
        res[f"lloyd_{int(fixed)}_C"], res[f"lloyd_{int(fixed)}_lab"] = C, lab
        res[f"lloyd_{int(fixed)}_meta"] = np.array([it, chg, lo, hi], np.int64)
        res[f"lloyd_{int(fixed)}_inertia"] = np.array([inert])
    dist.barrier()
    dist.destroy_process_group()
    np.savez(f"{out}.{rank}.npz", **res)


if __name__ == "__main__":
    main()
