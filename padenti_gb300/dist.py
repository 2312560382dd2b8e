"""Host logic of candidate-sharded training across ranks (one GPU per rank).

Every rank evaluates a contiguous range of the F candidates of every frontier
node (candidates are MD5-derived from (tree, node, f), so any rank can rebuild
any of them without an exchange).  The only exchange per depth is the argmax of
the per-rank best splits: the exact FP64 gain is identical on every rank for the
same counts, so the global winner is the largest gain, ties going to the lowest
global index t*F + f -- the same rule as the single-GPU split.  Two all-reduces
of one int64 per node do it: MAX over order-preserving keys of the gains, then
MIN over the indices of the ranks that hold the maximum.
"""
from __future__ import annotations

import numpy as np


def shard_range(n_features: int, rank: int, world: int) -> tuple[int, int]:
    """Candidates [f0, f1) evaluated by `rank`."""
    per = (n_features + world - 1) // world
    f0 = min(n_features, rank * per)
    return f0, min(n_features, f0 + per)


def gain_key(gain: np.ndarray) -> np.ndarray:
    """int64 keys whose order is the order of the float64 gains (NaN-free)."""
    b = np.ascontiguousarray(gain, np.float64).view(np.int64)
    return np.where(b < 0, np.int64(-0x8000000000000000) - b - 1, b)


def global_index(t: np.ndarray, f_local: np.ndarray, f0: int, n_features: int) -> np.ndarray:
    """t*F + f of a shard's winners (-1 for nodes without a candidate)."""
    t = np.asarray(t, np.int64)
    return np.where(t < 0, np.int64(-1), t * n_features + (np.asarray(f_local, np.int64) + f0))


def reduce_best_splits(gain: np.ndarray, idx: np.ndarray, group=None) -> tuple[np.ndarray, np.ndarray]:
    """Global (gain, index) of the best split of every node across the ranks of
    `group` (torch.distributed).  Nodes without a candidate on a rank carry
    idx = -1 there; a node without a candidate anywhere returns idx = -1."""
    import torch
    import torch.distributed as dist

    gain = np.ascontiguousarray(gain, np.float64)
    idx = np.ascontiguousarray(idx, np.int64)
    none = idx < 0
    key = gain_key(gain)
    key[none] = np.iinfo(np.int64).min
    k = torch.from_numpy(key.copy())
    dist.all_reduce(k, op=dist.ReduceOp.MAX, group=group)
    kmax = k.numpy()
    cand = np.where((key == kmax) & ~none, idx, np.iinfo(np.int64).max)
    c = torch.from_numpy(cand.copy())
    dist.all_reduce(c, op=dist.ReduceOp.MIN, group=group)
    best_idx = c.numpy().copy()
    best_idx[best_idx == np.iinfo(np.int64).max] = -1
    # the gain of the winner, from its key
    b = np.where(kmax < 0, np.int64(-0x8000000000000000) - kmax - 1, kmax)
    best_gain = b.view(np.float64).copy()
    best_gain[best_idx < 0] = 0.0
    return best_gain, best_idx


def global_winners(keys: list, idxs: list, counts: list) -> tuple[np.ndarray, np.ndarray]:
    """The global best split of every node from all ranks' best splits (lists over ranks):
    the largest key, ties to the lowest index, with that rank's left class counts."""
    key = np.stack(keys)
    idx = np.stack(idxs)
    kmax = key.max(axis=0)
    cand = np.where((key == kmax) & (idx >= 0), idx, np.iinfo(np.int64).max)
    best = cand.min(axis=0)
    owner = np.argmin(cand, axis=0)
    best = np.where(best == np.iinfo(np.int64).max, -1, best)
    cnt = np.stack(counts)[owner, np.arange(key.shape[1])]
    cnt[best < 0] = 0
    return best, cnt


def torch_exchange(group=None):
    """An exchange for pd_train_tree_sharded over torch.distributed: all-reduces MAX of the gain
    keys, MIN of the indices of the ranks holding the maximum, and SUM of the owner's left
    class counts (three collectives per frontier slice)."""

    def run(key: np.ndarray, idx: np.ndarray, counts: np.ndarray):
        import torch
        import torch.distributed as dist

        k = torch.from_numpy(key.copy())
        dist.all_reduce(k, op=dist.ReduceOp.MAX, group=group)
        kmax = k.numpy()
        cand = np.where((key == kmax) & (idx >= 0), idx, np.iinfo(np.int64).max)
        c = torch.from_numpy(cand.copy())
        dist.all_reduce(c, op=dist.ReduceOp.MIN, group=group)
        best = c.numpy().copy()
        mine = (best == idx) & (idx >= 0)
        cnt = torch.from_numpy(np.where(mine[:, None], counts, 0).astype(np.int64))
        dist.all_reduce(cnt, op=dist.ReduceOp.SUM, group=group)
        best[best == np.iinfo(np.int64).max] = -1
        return best, cnt.numpy().astype(np.uint32)

    return run


class LocalExchange:
    """An exchange among `world` ranks that are threads of one process (for example several
    contexts on one GPU): each rank deposits its best splits, waits at a barrier (with a
    timeout, so a missing rank ends in an error, not a hang) and computes the same global
    winners from all deposits."""

    def __init__(self, world: int, timeout: float = 120.0):
        import threading

        self.world = world
        self.barrier = threading.Barrier(world, timeout=timeout)
        self.slots = [None] * world

    def rank(self, r: int):
        def run(key, idx, counts):
            self.slots[r] = (key.copy(), idx.copy(), counts.copy())
            self.barrier.wait()
            best, cnt = global_winners([s[0] for s in self.slots], [s[1] for s in self.slots],
                                       [s[2] for s in self.slots])
            self.barrier.wait()  # every rank has read the deposits before the next slice overwrites them
            return best, cnt

        return run


def c_exchange(fn):
    """A pd_exchange_fn calling fn(key [n] int64, idx [n] int64, counts [n, K] uint32) ->
    (idx, counts) of the global winners; a Python exception returns -1 (the training call then
    fails with an error)."""
    import ctypes as C

    from padenti_gb300 import _native as N

    def cb(user, n, k, key_p, idx_p, cnt_p):
        try:
            key = np.ctypeslib.as_array(key_p, shape=(n,))
            idx = np.ctypeslib.as_array(idx_p, shape=(n,))
            cnt = np.ctypeslib.as_array(cnt_p, shape=(n, k))
            best, c = fn(key.copy(), idx.copy(), cnt.copy())
            idx[:] = best
            cnt[:] = c
            return 0
        except Exception:  # noqa: BLE001 - reported to the library as a failed exchange
            import traceback

            traceback.print_exc()
            return -1

    return N.EXCHANGE_FN(cb)
