"""The CUDA path against outputs of the reference's own device code.

tests/golden/ref_kernels.npz (made by tests/golden/make_ref_kernel_golden.py)
holds what the reference's kernels/hist_update.cl, kernels/predict.cl and
kernels/learn_best_feature.cl, compiled as C from the Padenti sources, give on
three seeded workloads (the reference's own test/feature.cl, the
depth-difference feature and the RGB channel-difference feature): each
sample's node at every depth from the reference's traversal kernel, the
frontier histograms summed from its per-image indicators, its split choices,
and forest posteriors and leaf maps of two images with and without a mask.
The fixture's trees are oracle trees that tests/test_reference_kernels.py
checks against the same kernels.  Here the CUDA library must give the same
numbers bit for bit.
"""
import hashlib
import pathlib
import sys

import numpy as np
import pytest

import padenti_gb300 as pg
from cases import sample_labels

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))

import make_ref_kernel_golden as mk  # noqa: E402
import test_reference_kernels as rkt  # noqa: E402

pytestmark = pytest.mark.gpu
GOLD = dict(np.load(HERE / "golden" / "ref_kernels.npz"))


def _g(plugin, key):
    return GOLD[f"{plugin}/{key}"]


def _sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _tree(cfg, plugin, tid):
    t = pg.Tree(cfg, tid, mk.DEPTH)
    t.left_child[:] = _g(plugin, f"tree{tid}_left_child")
    t.features[:] = _g(plugin, f"tree{tid}_features").astype(t.features.dtype)
    t.thresholds[:] = _g(plugin, f"tree{tid}_thresholds").astype(t.thresholds.dtype)
    t.posteriors[:] = _g(plugin, f"tree{tid}_posteriors")
    return t


@pytest.mark.parametrize("plugin", sorted(rkt.CASES))
def test_cuda_path_matches_reference_kernel_outputs(plugin):
    cfg, ts, tp, (px, lb, sm) = rkt.CASES[plugin]()
    inputs = np.concatenate([px.reshape(-1).view(np.uint8), lb.reshape(-1), sm.reshape(-1).view(np.uint8)])
    assert _sha(inputs) == str(_g(plugin, "inputs_sha256")), "the seeded inputs changed"
    K = cfg.n_classes
    tr = pg.TreeTrainer(cfg)
    tr.upload(ts)
    labels = sample_labels(ts)
    # every depth: the frontier's histograms given each sample's node from the reference's traversal
    for d in range(1, mk.DEPTH):
        key = f"d{d}_hist_sha256"
        if f"{plugin}/{key}" not in GOLD:
            continue
        node = _g(plugin, f"d{d}_sample_node")
        frontier = _g(plugin, f"d{d}_frontier")
        h = tr.hist(tp, mk.TREE_ID, node, frontier)
        assert _sha(h.astype(np.uint32)) == str(_g(plugin, key)), (plugin, d)
        # the split of every frontier node: the reference's choice, or an FP32 near-tie of it
        ctot = np.stack([np.bincount(labels[node == n], minlength=K) for n in frontier]).astype(np.uint32)
        t, f, g = tr.split(tp, h, ctot)
        for i, (rt, rf) in enumerate(_g(plugin, f"d{d}_ref_split")):
            if (rt, rf) != (t[i], f[i]):
                gap = g[i] - rkt._exact_gain(h[i], ctot[i], int(rt), int(rf))
                assert -1e-12 <= gap <= 2 * (3 * K + 3) * 4.4e-7, (plugin, d, i, gap)
    # the whole tree, and every sample's final node as the reference's traversal puts it
    tree = pg.Tree(cfg, mk.TREE_ID, mk.DEPTH)
    tr.train(tree, ts, tp)
    assert np.array_equal(tree.left_child, _g(plugin, f"tree{mk.TREE_ID}_left_child"))
    assert np.array_equal(tree.features.astype(np.int32), _g(plugin, f"tree{mk.TREE_ID}_features"))
    assert np.array_equal(tree.thresholds.astype(np.int32), _g(plugin, f"tree{mk.TREE_ID}_thresholds"))
    assert np.array_equal(tree.posteriors.view(np.uint32),
                          _g(plugin, f"tree{mk.TREE_ID}_posteriors").view(np.uint32))
    assert np.array_equal(tr.sample_nodes(ts.n_samples), _g(plugin, f"d{mk.DEPTH}_sample_node"))
    # forest posterior and leaf maps of the reference's predict/computePosterior kernels
    clf = pg.Classifier(cfg)
    clf << _tree(cfg, plugin, mk.TREE_ID)
    clf << _tree(cfg, plugin, 0)
    for i, im in enumerate(ts.images[:2]):
        for mi, mask in enumerate(mk.masks_of(im)):
            post = clf.predict(im.data, mask)
            assert _sha(post.astype(np.float32)) == str(_g(plugin, f"img{i}_mask{mi}_posterior_sha256")), (i, mi)
            for k in range(2):
                leaf = clf.predict_leaf(k, im.data, mask)
                assert _sha(leaf.astype(np.int32)) == str(_g(plugin, f"img{i}_mask{mi}_tree{k}_leaf_sha256")), (i, k)
