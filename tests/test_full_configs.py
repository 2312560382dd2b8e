"""The benchmark configurations at their stated candidate parameters, bit for bit
against the oracle on an image subset (the oracle runs on all host cores).

- 640x480 depth maps, 9 classes (8 angular parts + background), 2000 samples per
  image, F=2000 candidates x T=50 thresholds, depth 16, min 20 samples per leaf:
  the whole tree and every sample's final node on the first 100 of the 2000
  benchmark images; the root histogram and root split on all 2000.
- 320x240 RGB Voronoi images, 21 classes, channel-difference feature, F=1000 x
  T=30, depth 18 (2000 samples per image, min 20 per leaf): the whole tree on 40
  images.
"""
import os

import numpy as np
import pytest

import oracle_bind as ob
import padenti_gb300 as pg
from cases import sample_labels

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1


def _depth_config(n_images):
    px, lb, sm = pg.synth_depth(0, n_images, 640, 480, parts=1, min_ellipses=2, max_ellipses=5,
                                samples_per_image=2000, bg_permille=100)
    cfg = pg.ForestConfig("depth_diff2", 9)
    ts = pg.training_set(9, px, lb, sm)
    tp = pg.TreeTrainerParameters(2000, 50, [-60000] * 4, [60000] * 4, -500, 500, 20)
    return cfg, ts, tp


def _compare_trees(tree, o, tr, n_samples):
    assert np.array_equal(tree.left_child, o["left_child"])
    assert np.array_equal(tree.features.astype(np.int32), o["features"])
    assert np.array_equal(tree.thresholds.astype(np.int32), o["thresholds"])
    assert np.array_equal(tree.posteriors.view(np.uint32), o["posteriors"].view(np.uint32))
    assert np.array_equal(tr.sample_nodes(n_samples), o["sample_leaf"])


def test_depth_config_full_candidates_tree_bit_exact_on_100_images():
    cfg, ts, tp = _depth_config(100)
    tr = pg.TreeTrainer(cfg)
    tree = pg.Tree(cfg, 0, 16)
    tr.train(tree, ts, tp)
    o = ob.train_tree(ob.params(cfg, tp), ob.OracleSet(ts, cfg), 0, 16, ts.priors, threads=THREADS)
    assert o["nodes_split"] > 500
    _compare_trees(tree, o, tr, ts.n_samples)


def test_depth_config_root_on_all_2000_images():
    cfg, ts, tp = _depth_config(2000)
    tr = pg.TreeTrainer(cfg)
    tr.upload(ts)
    node = np.zeros(ts.n_samples, np.int32)
    h = tr.hist(tp, 0, node, [0])
    p = ob.params(cfg, tp)
    ho = ob.hist(p, ob.OracleSet(ts, cfg), 0, node, [0], threads=THREADS)
    assert np.array_equal(h, ho)
    ctot = np.bincount(sample_labels(ts), minlength=9).astype(np.uint32)[None, :]
    t, f, g = tr.split(tp, h, ctot)
    to, fo, go, _, _ = ob.split(p, ho, ctot)
    assert (t[0], f[0]) == (to[0], fo[0]) and g[0] == go[0]


def test_rgb_config_full_candidates_tree_bit_exact_on_40_images():
    px, lb, sm = pg.synth_rgb(0, 40, 320, 240, n_classes=21, samples_per_image=2000)
    cfg = pg.ForestConfig("channel_diff", 21)
    ts = pg.training_set(21, px, lb, sm)
    tp = pg.TreeTrainerParameters(1000, 30, [0, 0, -30, -30, -30, -30], [3, 3, 30, 30, 30, 30], -255, 255, 20)
    tr = pg.TreeTrainer(cfg)
    tree = pg.Tree(cfg, 0, 18)
    tr.train(tree, ts, tp)
    o = ob.train_tree(ob.params(cfg, tp), ob.OracleSet(ts, cfg), 0, 18, ts.priors, threads=THREADS)
    assert o["nodes_split"] > 500
    _compare_trees(tree, o, tr, ts.n_samples)
