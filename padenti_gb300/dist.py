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
