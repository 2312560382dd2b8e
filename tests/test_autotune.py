"""The launch-shape autotuner (pd_autotune): it picks settings from its search space, never
changes the tree, and a second call with the same cache file applies the cached setting
without timing."""
import numpy as np
import pytest

import padenti_gb300 as pg
from cases import depth_case


def test_autotune_needs_a_training_set():
    from padenti_gb300 import _native as N
    import ctypes as C

    out = N.Tuning()
    tp = pg.TreeTrainerParameters(8, 4, [0] * 4, [1] * 4, 0, 1)
    assert N.lib().pd_autotune(None, C.byref(tp.c()), 5, 0, None, C.byref(out)) == -1


@pytest.mark.gpu
def test_autotune_keeps_the_tree_and_caches(tmp_path):
    cfg, ts, tp, _ = depth_case(n_images=12, n_features=128, n_thresholds=20, parts=1)
    ref = pg.Tree(cfg, 3, 9)
    pg.TreeTrainer(cfg).train(ref, ts, tp)
    cache = tmp_path / "tune.txt"
    tr = pg.TreeTrainer(cfg)
    r = tr.autotune(ts, tp, 9, cache=cache, max_trials=8)
    assert r["from_cache"] == 0 and 1 <= r["trials"] <= 8
    assert r["chunk"] in (4096, 8192, 16384, 32768) and r["hist_spi"] in (4, 8)
    assert r["fuse_max"] in (1024, 2048, 4096, 8192) and r["cand_order"] in (0, 1) and r["persist"] in (0, 1)
    assert r["ms_best"] <= r["ms_start"] * 1.0001
    tree = pg.Tree(cfg, 3, 9)
    tr.train(tree, ts, tp)  # with the tuned settings
    for f in ("left_child", "features", "thresholds"):
        assert np.array_equal(getattr(tree, f), getattr(ref, f)), f
    assert np.array_equal(tree.posteriors.view(np.uint32), ref.posteriors.view(np.uint32))
    again = pg.TreeTrainer(cfg).autotune(ts, tp, 9, cache=cache)
    assert again["from_cache"] == 1 and again["trials"] == 0
    assert [again[k] for k in ("chunk", "hist_spi", "fuse_max", "cand_order", "persist")] == \
        [r[k] for k in ("chunk", "hist_spi", "fuse_max", "cand_order", "persist")]
    assert len(cache.read_text().splitlines()) == 1
