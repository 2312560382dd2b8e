"""Candidate-sharded training on the GPU (pd_train_tree_sharded).  One GPU here, so the ranks
are threads of this process, each with its own context (and stream) on GPU 0, exchanging their
best splits on the host between depths (padenti_gb300.dist.LocalExchange: a barrier with a
timeout, no kernel waits on another).  Every rank must end with the unsharded tree, bit for
bit, which the oracle pins."""
import threading

import numpy as np
import pytest

import oracle_bind as ob
import padenti_gb300 as pg
from cases import actx_case, depth_case, rgb_case
from padenti_gb300 import dist as pdist

pytestmark = pytest.mark.gpu


def _run_ranks(cfg, ts, tp, world, tree_id, depth):
    ex = pdist.LocalExchange(world)
    trees = [pg.Tree(cfg, tree_id, depth) for _ in range(world)]
    errors = []

    def rank(r):
        try:
            tr = pg.TreeTrainer(cfg)
            f0, f1 = pdist.shard_range(tp.n_features, r, world)
            tr.train_sharded(trees[r], ts, tp, f0, f1, ex.rank(r))
        except Exception as e:  # noqa: BLE001
            errors.append((r, e))
            ex.barrier.abort()

    th = [threading.Thread(target=rank, args=(r,)) for r in range(world)]
    for t in th:
        t.start()
    for t in th:
        t.join(timeout=600)
    assert not errors, errors
    return trees


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_tree_equals_unsharded(world):
    cfg, ts, tp, _ = depth_case(n_images=12, n_features=200, n_thresholds=20, parts=1)
    ref = pg.Tree(cfg, 4, 9)
    pg.TreeTrainer(cfg).train(ref, ts, tp)
    o = ob.train_tree(ob.params(cfg, tp), ob.OracleSet(ts, cfg), 4, 9, ts.priors)
    assert np.array_equal(ref.left_child, o["left_child"])
    for t in _run_ranks(cfg, ts, tp, world, 4, 9):
        for f in ("left_child", "features", "thresholds"):
            assert np.array_equal(getattr(t, f), getattr(ref, f)), f
        assert np.array_equal(t.posteriors.view(np.uint32), ref.posteriors.view(np.uint32))


def test_sharded_rgb_tree_equals_unsharded():
    cfg, ts, tp, _ = rgb_case(n_images=6, n_features=120, n_thresholds=12)
    ref = pg.Tree(cfg, 2, 8)
    pg.TreeTrainer(cfg).train(ref, ts, tp)
    for t in _run_ranks(cfg, ts, tp, 2, 2, 8):
        for f in ("left_child", "features", "thresholds"):
            assert np.array_equal(getattr(t, f), getattr(ref, f)), f
        assert np.array_equal(t.posteriors.view(np.uint32), ref.posteriors.view(np.uint32))


def test_sharded_auto_context_tree_equals_the_oracle():
    """A feature that reads the tree: every rank keeps its own node maps and trains the
    oracle's tree."""
    cfg, ts, tp, _ = actx_case(n_features=96)
    o = ob.train_tree(ob.params(cfg, tp, "auto_context"), ob.OracleSet(ts, cfg), 3, 7, ts.priors)
    for t in _run_ranks(cfg, ts, tp, 2, 3, 7):
        assert np.array_equal(t.left_child, o["left_child"])
        assert np.array_equal(np.asarray(t.features, np.int32), o["features"])
        assert np.array_equal(t.posteriors.view(np.uint32), o["posteriors"].view(np.uint32))


def test_failed_exchange_is_an_error():
    cfg, ts, tp, _ = depth_case(n_images=4, n_features=64, n_thresholds=10)

    def broken(key, idx, counts):
        raise RuntimeError("rank lost")

    with pytest.raises(pg.PadentiError, match="exchange"):
        pg.TreeTrainer(cfg).train_sharded(pg.Tree(cfg, 0, 6), ts, tp, 0, 32, broken)
