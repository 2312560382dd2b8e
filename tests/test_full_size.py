"""The full training configuration (2000 × 640×480 depth maps, 2000 samples per image, F=2000,
T=50, depth 16, 9 classes) checked through properties that hold at any size, where the CPU
oracle would take too long: the tree's structure rules, every node's posterior equal to the
class frequencies of the samples that reach it (computed here from the samples' final nodes),
and the same tree under other launch shapes."""
import numpy as np
import pytest

import padenti_gb300 as pg


def _node_class_counts(final, labels, n_nodes, K):
    """Class counts of every heap node from the samples' final nodes (each sample counts in
    every node on its path from the root)."""
    counts = np.zeros(n_nodes * K, np.int64)
    node = final.astype(np.int64)
    live = np.ones(node.size, bool)
    while live.any():
        counts += np.bincount(node[live] * K + labels[live], minlength=n_nodes * K)
        live &= node > 0
        node = np.where(node > 0, (node - 1) // 2, 0)
    return counts.reshape(n_nodes, K)


def test_node_class_counts_on_an_oracle_tree():
    import oracle_bind as ob
    from cases import depth_case

    cfg, ts, tp, _ = depth_case(n_images=6, n_features=24, n_thresholds=10)
    o = ob.train_tree(ob.params(cfg, tp), ob.OracleSet(ts, cfg), 1, 7, ts.priors)
    labels = np.concatenate([im.labels.reshape(-1)[im.samples] for im in ts.images]).astype(np.int64) - 1
    counts = _node_class_counts(o["sample_leaf"], labels, o["left_child"].size, 3)
    assert np.array_equal(counts[0], np.bincount(labels, minlength=3))
    made = np.nonzero(o["left_child"] != -2)[0]
    made = made[made > 0]
    want = (counts[made].astype(np.float32) / counts[made].sum(1, keepdims=True).astype(np.float32))
    assert np.array_equal(o["posteriors"][made].view(np.uint32), want.astype(np.float32).view(np.uint32))


@pytest.mark.gpu
def test_full_size_tree_properties():
    px, lb, sm = pg.synth_depth(0, 2000, 640, 480, parts=1, min_ellipses=2, max_ellipses=5, samples_per_image=2000,
                                bg_permille=100)
    cfg = pg.ForestConfig("depth_diff2", 9)
    ts = pg.training_set(9, px, lb, sm)
    tp = pg.TreeTrainerParameters(2000, 50, [-60000] * 4, [60000] * 4, -500, 500, 20)
    tr = pg.TreeTrainer(cfg)
    tree = pg.Tree(cfg, 0, 16)
    tr.train(tree, ts, tp)
    final = tr.sample_nodes(ts.n_samples)
    labels = np.take_along_axis(lb.reshape(2000, -1), sm.astype(np.int64), axis=1).reshape(-1).astype(np.int64) - 1
    lc = tree.left_child
    n_nodes = lc.size
    # every sample ends on a leaf
    assert np.all(lc[final] == -1)
    # class counts of every node from the samples' paths
    counts = _node_class_counts(final, labels, n_nodes, 9)
    tot = counts.sum(axis=1)
    split = np.nonzero(lc >= 0)[0]
    assert split.size > 1000
    assert np.all(lc[split] == 2 * split + 1)
    assert np.all(tot[split] > tp.per_leaf_samples_thr)
    assert np.all(tot[2 * split + 1] > 0) and np.all(tot[2 * split + 2] > 0)
    assert np.all(counts[lc == -2] == 0) and np.all(tree.posteriors[lc == -2] == 0)
    created = np.nonzero(lc != -2)[0]
    created = created[created > 0]
    want = (counts[created].astype(np.float32) / tot[created, None].astype(np.float32)).astype(np.float32)
    assert np.array_equal(tree.posteriors[created].view(np.uint32), want.view(np.uint32))
    # launch shapes change no result
    tr.set_tuning("chunk", 4096)
    tr.set_tuning("hist_spi", 4)
    tr.set_tuning("cand_order", 0)
    tr.set_tuning("persist", 0)
    again = pg.Tree(cfg, 0, 16)
    tr.train(again, ts, tp)
    assert np.array_equal(again.left_child, lc)
    assert np.array_equal(again.features, tree.features) and np.array_equal(again.thresholds, tree.thresholds)
    assert np.array_equal(again.posteriors.view(np.uint32), tree.posteriors.view(np.uint32))
