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


# A feature that reads the tree (auto-context): the oracle's OR_PLUGIN_AUTO_CONTEXT
# (and oracle/ref_shim/cl/actx/feature.cl) written as a user feature.
AUTO_CONTEXT_SOURCE = r"""
__device__ feat_t computeFeature(const pd::ImageView &img, int2 c, const pd::TreeView &tree, const feat_t *f,
                                 unsigned featDim) {
  const int n1 = img.nodeID(c.x + f[0], c.y + f[1]);
  const int K = (int)tree.nClasses;
  const int k = ((f[2] % K) + K) % K;
  const float pv = tree.posterior(n1, k);
  const int inner = tree.leftChild(n1) >= 0 ? 2000 : 0;
  const int a = img.read(c.x + f[3], c.y, 0), b = img.read(c.x, c.y, 0);
  return (int)__fmul_rn(pv, 1000.0f) + inner + (a - b) / 16 + n1 % 5;
}
"""


def actx_case(n_images=6, width=64, height=48, n_features=64, n_thresholds=8, seed=11, samples=300, min_leaf=10):
    """Depth maps (3 classes) with the auto-context feature: offsets +-12 px, class selector
    in [0, 3], thresholds over [-400, 3400] (the posterior term spans 0..1000, the
    children term 0 or 2000)."""
    px, lb, sm = pg.synth_depth(seed, n_images, width, height, samples_per_image=samples)
    cfg = pg.ForestConfig("user", 3, source=AUTO_CONTEXT_SOURCE, shape="u16x1_i32x4")
    ts = pg.training_set(3, px, lb, sm)
    tp = pg.TreeTrainerParameters(n_features, n_thresholds, [-12, -12, 0, -12], [12, 12, 3, 12], -400, 3400,
                                  min_leaf)
    return cfg, ts, tp, (px, lb, sm)


def tree_tuple(tree):
    return (tree.depth, tree.left_child, np.asarray(tree.features, np.int32), np.asarray(tree.thresholds, np.int32),
            tree.posteriors)


def sample_labels(ts) -> np.ndarray:
    """Class (0-based) of every sample of a TrainingSet, in upload order."""
    return np.concatenate([im.labels.reshape(-1)[im.samples] for im in ts.images]).astype(np.int64) - 1


def sampler_images():
    """Images for the pixel-sampler tests: (name, img_type, data, labels, n_classes).  Depth maps
    of several sizes (an odd one among them), RGB images, and label images with one, two or no
    labelled pixels."""
    out = []
    px, lb, _ = pg.synth_depth(5, 3, 80, 60, parts=1, min_ellipses=2, max_ellipses=4, samples_per_image=4)
    out += [(f"depth80x60_{i}", 2, px[i], lb[i], 9) for i in range(3)]
    px, lb, _ = pg.synth_depth(8, 2, 161, 121, parts=1, min_ellipses=2, max_ellipses=4, samples_per_image=4)
    out += [(f"depth161x121_{i}", 2, px[i], lb[i], 9) for i in range(2)]
    rgb, rlb, _ = pg.synth_rgb(5, 2, 47, 39, n_classes=6, samples_per_image=4)
    out += [(f"rgb47x39_{i}", 1, rgb[i], rlb[i], 6) for i in range(2)]
    sparse = np.zeros((60, 80), np.uint8)
    sparse[10, 7], sparse[30, 50] = 2, 5
    single = np.zeros((60, 80), np.uint8)
    single[20, 20] = 1
    out += [("sparse", 2, px[0][:60, :80].copy(), sparse, 9), ("single", 2, px[1][:60, :80].copy(), single, 9)]
    return out


# (name, kind, n_samples, seed, weights) of the sampler fixtures; weights name a rule
SAMPLER_CONFIGS = [
    ("uniform_500", 1, 500, 0, None),
    ("uniform_37", 1, 37, 123456, None),
    ("uniform_3000", 1, 3000, 7, None),
    ("cw_300", 2, 300, 0, None),
    ("cw_2000_skewed", 2, 2000, 99, "skewed"),
    ("cw_250_zero", 2, 250, 5, "zero"),
]


def sampler_weights(rule, k):
    if rule is None:
        return None
    if rule == "skewed":
        return np.linspace(0.02, 0.3, k).astype(np.float32)
    w = np.full(k, 1.0 / (k - 1), np.float32)
    w[1] = 0
    return w
