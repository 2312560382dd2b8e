"""Seeded workloads shared by the parity tests: small versions of the depth-map,
single-offset and RGB channel-difference configurations."""
from __future__ import annotations

import numpy as np

import padenti_gb300 as pg


def depth_case(n_images=16, width=160, height=120, n_features=64, n_thresholds=20, seed=0, parts=0,
               samples=500, min_leaf=20):
    """Depth maps made like the 64x160x120 configuration (3 classes, offsets +-60000 px*mm,
    thresholds +-500, out-of-image reads 10000)."""
    K = 9 if parts else 3
    px, lb, sm = pg.synth_depth(seed, n_images, width, height, parts=parts, samples_per_image=samples,
                                max_ellipses=5 if parts else 3, min_ellipses=2 if parts else 1)
    cfg = pg.ForestConfig("depth_diff2", K)
    ts = pg.training_set(K, px, lb, sm)
    tp = pg.TreeTrainerParameters(n_features, n_thresholds, [-60000] * 4, [60000] * 4, -500, 500, min_leaf)
    return cfg, ts, tp, (px, lb, sm)


def depth1_case(n_images=8, width=160, height=120, n_features=48, n_thresholds=10, seed=3):
    """The reference example plugin (test/feature.cl): short features, offsets +-60, thresholds +-200
    (test/test_tree_trainer.cpp:66-77)."""
    px, lb, sm = pg.synth_depth(seed, n_images, width, height, samples_per_image=400)
    cfg = pg.ForestConfig("depth_diff1", 3)
    ts = pg.training_set(3, px, lb, sm)
    tp = pg.TreeTrainerParameters(n_features, n_thresholds, [-60, -60], [60, 60], -200, 200, 400 // 3)
    return cfg, ts, tp, (px, lb, sm)


def rgb_case(n_images=8, width=80, height=60, n_features=40, n_thresholds=12, seed=5, samples=600):
    """RGB Voronoi images, 21 classes, channel-difference feature (c1,c2 in [0,3), u,v in +-30)."""
    px, lb, sm = pg.synth_rgb(seed, n_images, width, height, n_classes=21, samples_per_image=samples)
    cfg = pg.ForestConfig("channel_diff", 21)
    ts = pg.training_set(21, px, lb, sm)
    tp = pg.TreeTrainerParameters(n_features, n_thresholds, [0, 0, -30, -30, -30, -30], [3, 3, 30, 30, 30, 30],
                                  -255, 255, 10)
    return cfg, ts, tp, (px, lb, sm)


def tree_tuple(tree):
    return (tree.depth, tree.left_child, np.asarray(tree.features, np.int32), np.asarray(tree.thresholds, np.int32),
            tree.posteriors)


def sample_labels(ts) -> np.ndarray:
    """Class (0-based) of every sample of a TrainingSet, in upload order."""
    return np.concatenate([im.labels.reshape(-1)[im.samples] for im in ts.images]).astype(np.int64) - 1
