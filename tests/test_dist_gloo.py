"""Candidate-sharded split selection across two ranks (gloo on CPU): each rank
runs the oracle split on its candidate range, the argmax all-reduce of
padenti_gb300.dist must give the unsharded split exactly."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case():
    rng = np.random.default_rng(7)
    n, K, T, F = 12, 3, 6, 40
    tot = rng.integers(5, 60, size=(n, K)).astype(np.uint32)
    hist = (rng.random((n, K, T, F)) * tot[:, :, None, None]).astype(np.uint32)
    hist[0] = (tot[0] // 2)[:, None, None]  # every candidate of node 0 ties
    hist[1, :, 3, 17] = tot[1]              # a split putting everything left (no information)
    return hist, tot


def _worker(rank, world, port, out):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    sys.path.insert(0, os.path.dirname(here))
    import oracle_bind as ob
    import padenti_gb300 as pg
    from padenti_gb300 import dist as pdist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    hist, tot = _case()
    n, K, T, F = hist.shape
    f0, f1 = pdist.shard_range(F, rank, world)
    cfg = pg.ForestConfig("depth_diff2", K)
    tp = pg.TreeTrainerParameters(f1 - f0, T, [0] * 4, [1] * 4, 0, 1)
    t, f, g, _, _ = ob.split(ob.params(cfg, tp), np.ascontiguousarray(hist[..., f0:f1]), tot)
    gain, idx = pdist.reduce_best_splits(g, pdist.global_index(t, f, f0, F))
    out[rank] = (gain, idx)
    dist.destroy_process_group()


def test_sharded_argmax_equals_unsharded_split():
    import oracle_bind as ob
    import padenti_gb300 as pg

    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    hist, tot = _case()
    n, K, T, F = hist.shape
    cfg = pg.ForestConfig("depth_diff2", K)
    tp = pg.TreeTrainerParameters(F, T, [0] * 4, [1] * 4, 0, 1)
    t, f, g, _, _ = ob.split(ob.params(cfg, tp), hist, tot)
    exp_idx = np.where(t < 0, -1, t.astype(np.int64) * F + f)
    for r in range(world):
        gain, idx = out[r]
        assert np.array_equal(idx, exp_idx)
        assert np.array_equal(gain.view(np.uint64), g.view(np.uint64))
    assert exp_idx[0] == 0  # all tied: the lowest index wins


def test_gain_keys_preserve_order():
    from padenti_gb300 import dist as pdist

    g = np.array([-3.5, -0.0, 0.0, 1e-300, 0.25, 1.0, 2.0, -1e-9])
    k = pdist.gain_key(g)
    assert np.array_equal(np.argsort(k, kind="stable"), np.argsort(g, kind="stable"))
    assert pdist.shard_range(2000, 1, 3) == (667, 1334) and pdist.shard_range(10, 3, 4) == (9, 10)


def _tree_worker(rank, world, port, out):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    sys.path.insert(0, os.path.dirname(here))
    import oracle_bind as ob
    from cases import depth_case
    from padenti_gb300 import dist as pdist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfg, ts, tp, _ = depth_case(n_images=8, n_features=96, n_thresholds=20, parts=1)
    f0, f1 = pdist.shard_range(tp.n_features, rank, world)
    o = ob.train_tree_sharded(ob.params(cfg, tp), ob.OracleSet(ts, cfg), 3, 7, ts.priors, f0, f1,
                              pdist.torch_exchange(), threads=1)
    out[rank] = {k: o[k] for k in ("left_child", "features", "thresholds", "posteriors", "sample_leaf")}
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_whole_tree_equals_unsharded(world):
    """Candidate-sharded training of a whole tree over gloo ranks (each evaluates its range of the
    96 candidates; uneven ranges with 3 ranks), the per-slice exchange of padenti_gb300.dist, on
    the oracle: every rank ends with the unsharded tree, bit for bit."""
    import oracle_bind as ob
    from cases import depth_case

    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_tree_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    cfg, ts, tp, _ = depth_case(n_images=8, n_features=96, n_thresholds=20, parts=1)
    ref = ob.train_tree(ob.params(cfg, tp), ob.OracleSet(ts, cfg), 3, 7, ts.priors)
    assert ref["nodes_split"] >= 10
    for r in range(world):
        for k in ("left_child", "features", "thresholds", "sample_leaf"):
            assert np.array_equal(out[r][k], ref[k]), (r, k)
        assert np.array_equal(out[r]["posteriors"].view(np.uint32), ref["posteriors"].view(np.uint32))


def test_local_exchange_picks_the_global_winner():
    from padenti_gb300 import dist as pdist

    keys = [np.array([5, 7, np.iinfo(np.int64).min], np.int64), np.array([5, 3, np.iinfo(np.int64).min], np.int64)]
    idxs = [np.array([40, 2, -1], np.int64), np.array([12, 9, -1], np.int64)]
    cnts = [np.array([[1, 2], [3, 4], [0, 0]], np.uint32), np.array([[5, 6], [7, 8], [0, 0]], np.uint32)]
    best, cnt = pdist.global_winners(keys, idxs, cnts)
    assert best.tolist() == [12, 2, -1]  # tie on node 0 -> lowest index (rank 1); node 1 -> rank 0
    assert cnt.tolist() == [[5, 6], [3, 4], [0, 0]]
