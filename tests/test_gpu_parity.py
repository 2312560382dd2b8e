"""Parity of the sm_103a kernels (through the C ABI) with the CPU oracle.

Integer outputs (candidates, histograms, tree structure, leaf ids) must be
bit-identical; the split gain is the exact FP64 value (bit-identical); tree
posteriors and forest posteriors are IEEE float results of the same operation
sequence and must be bit-identical too (tolerance 0).
"""
import numpy as np
import pytest

import oracle_bind as ob
import padenti_gb300 as pg
from cases import depth1_case, depth_case, rgb_case, sample_labels, tree_tuple

pytestmark = pytest.mark.gpu


def _oracle_tree(cfg, ts, tp, tree_id, depth):
    p = ob.params(cfg, tp)
    ds = ob.OracleSet(ts, cfg)
    return ob.train_tree(p, ds, tree_id, depth, ts.priors)


def test_log2_table_bit_identical():
    cfg, ts, tp, _ = depth_case(n_images=2)
    tr = pg.TreeTrainer(cfg)
    n = 300_000
    g = tr.log2_table(n)
    o = ob.log2_table(n)
    assert np.array_equal(g.view(np.uint64), o.view(np.uint64))


@pytest.mark.parametrize("thr_bounds,T", [((-500, 500), 50), ((-(1 << 30), 1 << 30), 50), ((-500, 500), 3),
                                          ((-500, 500), 17), ((-500, 500), 64), ((-500, 500), 100),
                                          ((-20, 20), 64)])
def test_candidates_match_oracle(thr_bounds, T):
    """Narrow threshold bounds sort (value, index) packed in one word -- in registers by
    a bitonic network for T <= 64 (16, 32 or 64 keys with padding), by insertion in
    shared memory above; wide bounds (a range of 2^24 or more) sort them as two columns.
    Bounds of +-20 with 64 thresholds give equal values, ordered by index."""
    cfg, ts, tp, _ = depth_case(n_images=2, n_features=100, n_thresholds=50)
    tp = pg.TreeTrainerParameters(100, T, [-60000] * 4, [60000] * 4, thr_bounds[0], thr_bounds[1], 20)
    tr = pg.TreeTrainer(cfg)
    nodes = np.array([0, 1, 2, 77, 4095, 123456], np.int32)
    feat, thr = tr.candidates(tp, 7, nodes)
    p = ob.params(cfg, tp)
    for i, n in enumerate(nodes):
        for f in range(tp.n_features):
            of, ot = ob.candidate(p, 7, int(n), f)
            assert np.array_equal(feat[i, f], of), (n, f)
            assert np.array_equal(thr[i, f], ot), (n, f)


def test_hist_root_bit_exact():
    """8000 samples at the root: two sample chunks accumulate into the same rows."""
    cfg, ts, tp, _ = depth_case(n_images=16)
    tr = pg.TreeTrainer(cfg)
    tr.upload(ts)
    S = ts.n_samples
    sample_node = np.zeros(S, np.int32)
    g = tr.hist(tp, 0, sample_node, [0])
    o = ob.hist(ob.params(cfg, tp), ob.OracleSet(ts, cfg), 0, sample_node, [0])
    assert g.shape == o.shape
    assert np.array_equal(g, o)
    assert g.sum() > 0


def test_hist_many_nodes_with_empty_and_ragged():
    cfg, ts, tp, _ = depth_case(n_images=16, n_features=50, n_thresholds=17)
    tr = pg.TreeTrainer(cfg)
    tr.upload(ts)
    rng = np.random.default_rng(1)
    S = ts.n_samples
    # uneven node sizes, one node absent from the samples, some samples on other nodes
    sample_node = rng.choice([3, 4, 5, 6, 9, 10], size=S, p=[0.6, 0.25, 0.1, 0.03, 0.01, 0.01]).astype(np.int32)
    nodes = [6, 3, 4, 5, 11]
    g = tr.hist(tp, 2, sample_node, nodes)
    o = ob.hist(ob.params(cfg, tp), ob.OracleSet(ts, cfg), 2, sample_node, nodes)
    assert np.array_equal(g, o)
    assert g[4].sum() == 0


def test_split_matches_oracle_on_oracle_histograms():
    cfg, ts, tp, _ = depth_case(n_images=16)
    p = ob.params(cfg, tp)
    ds = ob.OracleSet(ts, cfg)
    rng = np.random.default_rng(2)
    S = ts.n_samples
    sample_node = rng.choice([3, 4, 5, 6], size=S, p=[0.7, 0.2, 0.09, 0.01]).astype(np.int32)
    nodes = [3, 4, 5, 6]
    h = ob.hist(p, ds, 0, sample_node, nodes)
    labels = sample_labels(ts)
    ctot = np.zeros((len(nodes), cfg.n_classes), np.uint32)
    for i, n in enumerate(nodes):
        ctot[i] = np.bincount(labels[sample_node == n], minlength=cfg.n_classes)
    ot, of, og, _, err = ob.split(p, h, ctot)
    tr = pg.TreeTrainer(cfg)
    gt, gf, gg = tr.split(tp, h, ctot)
    assert np.array_equal(gt, ot) and np.array_equal(gf, of)
    assert np.array_equal(gg.view(np.uint64), og.view(np.uint64))
    assert err < 5e-5


def test_split_ties_pick_lowest_index():
    cfg, ts, tp, _ = depth_case(n_images=1, n_features=8, n_thresholds=4)
    # every candidate identical -> winner (t=0, f=0); then make (t=2,f=5) and (t=1,f=7) equal best
    K, T, F = 3, 4, 8
    ctot = np.array([[10, 10, 10]], np.uint32)
    h = np.tile(np.array([5, 5, 5], np.uint32)[None, :, None, None], (1, 1, T, F))
    tr = pg.TreeTrainer(cfg)
    t, f, g = tr.split(tp, h, ctot)
    assert (t[0], f[0]) == (0, 0)
    h2 = h.copy()
    h2[0, :, 2, 5] = [10, 0, 0]
    h2[0, :, 1, 7] = [10, 0, 0]
    t, f, g = tr.split(tp, h2, ctot)
    assert (t[0], f[0]) == (1, 7)
    p = ob.params(cfg, tp)
    ot, of, og, _, _ = ob.split(p, h2, ctot)
    assert (ot[0], of[0]) == (1, 7) and og[0] == g[0]


def _assert_same_tree(g: pg.Tree, o: dict):
    assert np.array_equal(g.left_child, o["left_child"])
    assert np.array_equal(np.asarray(g.features, np.int32), o["features"])
    assert np.array_equal(np.asarray(g.thresholds, np.int32), o["thresholds"])
    assert np.array_equal(g.posteriors.view(np.uint32), o["posteriors"].view(np.uint32))


def test_pure_nodes_bit_exact():
    """Single-class and half-single-class training sets: every node (or every node of the
    right-half subtrees) is pure, every exact gain there is 0 and the split is the lowest
    index t*F + f -- the closed form of the fused split; also through the unfused split."""
    cfg, ts, tp, (px, lb, sm) = depth_case(n_images=12, n_features=96, n_thresholds=20, min_leaf=5)
    one = np.where(lb > 0, 1, 0).astype(lb.dtype)
    x = np.arange(lb.shape[-1])
    half = np.where((lb > 0) & (x >= lb.shape[-1] // 2), 1, lb).astype(lb.dtype)
    for labels in (one, half):
        ts1 = pg.training_set(3, px, labels, sm)
        o = _oracle_tree(cfg, ts1, tp, 2, 7)
        for fuse in (4096, 0):
            tr = pg.TreeTrainer(cfg)
            tr.set_tuning("fuse_max", fuse)
            t = pg.Tree(cfg, 2, 7)
            tr.train(t, ts1, tp)
            _assert_same_tree(t, o)


def test_upload_rejects_bad_samples_and_keeps_the_previous_set():
    """A sample outside its image or on an unlabelled pixel fails the upload with the first
    bad sample in sample order (the check runs on several host threads); the training set
    uploaded before stays in place."""
    import ctypes as C
    from padenti_gb300 import _native as N

    cfg, ts, tp, _ = depth_case(n_images=10, n_features=32, n_thresholds=10)
    tr = pg.TreeTrainer(cfg)
    tr.upload(ts)
    a = pg.Tree(cfg, 0, 5)
    tr.train(a, ts, tp)
    flat = ts.flat()
    w, h = int(flat["width"][0]), int(flat["height"][0])
    first7, first3 = int(flat["samp_off"][7]) + 5, int(flat["samp_off"][3]) + 2
    bad = {k: v.copy() for k, v in flat.items()}
    bad["samples"][first7] = w * h          # outside image 7
    bad["samples"][first3] = w * h + 10     # outside image 3: the first in sample order
    with pytest.raises(pg.PadentiError, match=f"sample {first3} of image 3 outside the image"):
        N.check(N.lib().pd_dataset_upload(tr.h, C.byref(pg.TrainingSet.desc(bad))))
    unl = {k: v.copy() for k, v in flat.items()}
    lab_off = int(flat["lab_off"][4])
    k4 = int(flat["samp_off"][4])
    unl["labels"][lab_off + int(unl["samples"][k4])] = 0
    with pytest.raises(pg.PadentiError, match=f"sample {k4} of image 4 has label 0"):
        N.check(N.lib().pd_dataset_upload(tr.h, C.byref(pg.TrainingSet.desc(unl))))
    b = pg.Tree(cfg, 0, 5)
    tr.train(b, ts, tp)  # the set uploaded first is still there
    assert np.array_equal(a.left_child, b.left_child)
    assert np.array_equal(a.features, b.features) and np.array_equal(a.thresholds, b.thresholds)


def _mixed_size_set(n_per_size=4, samples=600):
    """Depth maps of the three sizes of the mixed-size configuration (160x120, 320x240,
    640x480), 9 classes, in one training set."""
    imgs, raw = [], []
    for k, (w, h) in enumerate([(160, 120), (320, 240), (640, 480)]):
        px, lb, sm = pg.synth_depth(7, n_per_size, w, h, first_image=n_per_size * k, parts=1, min_ellipses=2,
                                    max_ellipses=5, samples_per_image=samples)
        imgs += [pg.TrainingSetImage(px[i], lb[i], 9, sm[i]) for i in range(n_per_size)]
        raw += [px[i] for i in range(n_per_size)]
    return pg.TrainingSet(9, imgs), raw


def test_mixed_image_sizes_bit_exact():
    """One training set of mixed image sizes: the tree is the oracle's."""
    ts, _ = _mixed_size_set()
    cfg = pg.ForestConfig("depth_diff2", 9)
    tp = pg.TreeTrainerParameters(96, 24, [-60000] * 4, [60000] * 4, -500, 500, 10)
    tree = pg.Tree(cfg, 4, 10)
    pg.TreeTrainer(cfg).train(tree, ts, tp)
    _assert_same_tree(tree, _oracle_tree(cfg, ts, tp, 4, 10))
    assert (tree.left_child >= 0).sum() > 20


def test_mixed_size_batch_prediction_matches_per_image():
    """A mixed-size batch (one launch replayed from a CUDA graph) gives the per-image
    posteriors bit for bit: twice with the same layout, with another layout, and after the
    forest grows (the cached graph must not be reused then)."""
    ts, raw = _mixed_size_set(n_per_size=2, samples=400)
    cfg = pg.ForestConfig("depth_diff2", 9)
    tp = pg.TreeTrainerParameters(64, 16, [-60000] * 4, [60000] * 4, -500, 500, 10)
    trees = []
    for tid in range(2):
        t = pg.Tree(cfg, tid, 8)
        pg.TreeTrainer(cfg).train(t, ts, tp)
        trees.append(t)
    clf = pg.Classifier(cfg)
    clf << trees[0]
    rng = np.random.default_rng(1)
    masks = [None, (rng.random(raw[1].shape) < 0.7).astype(np.uint8), None, None,
             (rng.random(raw[4].shape) < 0.5).astype(np.uint8), None]

    def check_batch(images, mks):
        got = clf.predict_batch(images, mks)
        for im, m, g in zip(images, mks, got):
            ref = clf.predict(im, m)
            assert np.array_equal(g.view(np.uint32), ref.view(np.uint32))

    check_batch(raw, masks)
    check_batch(raw, masks)                       # replayed graph
    check_batch(raw[::-1], masks[::-1])           # another layout
    clf << trees[1]                               # a grown forest
    check_batch(raw, masks)


def test_train_tree_config0_bit_exact():
    """The full 64-image 160x120 configuration: F=200, T=20, depth 8, min 20 pixels per leaf."""
    cfg, ts, tp, _ = depth_case(n_images=64, n_features=200, n_thresholds=20)
    tr = pg.TreeTrainer(cfg)
    tree = pg.Tree(cfg, 0, 8)
    tr.train(tree, ts, tp, 1, 8)
    o = _oracle_tree(cfg, ts, tp, 0, 8)
    _assert_same_tree(tree, o)
    assert np.array_equal(tr.sample_nodes(ts.n_samples), o["sample_leaf"])
    st = tr.stats()
    assert st["evals"] == o["evals"] and st["nodes_split"] == o["nodes_split"]
    assert (tree.left_child >= 0).sum() > 20


def test_train_tree_sliced_histograms_identical():
    """A 1 MiB histogram budget forces many slices per depth; the tree must not change."""
    cfg, ts, tp, _ = depth_case(n_images=16, n_features=96, n_thresholds=20)
    a = pg.Tree(cfg, 4, 7)
    b = pg.Tree(cfg, 4, 7)
    pg.TreeTrainer(cfg).train(a, ts, tp)
    pg.TreeTrainer(cfg, hist_budget=1 << 20).train(b, ts, tp)
    assert np.array_equal(a.left_child, b.left_child)
    assert np.array_equal(a.features, b.features) and np.array_equal(a.thresholds, b.thresholds)
    _assert_same_tree(a, _oracle_tree(cfg, ts, tp, 4, 7))


def test_launch_shape_knobs_do_not_change_the_tree():
    cfg, ts, tp, _ = depth_case(n_images=16, n_features=96, n_thresholds=20)
    a = pg.Tree(cfg, 5, 7)
    pg.TreeTrainer(cfg).train(a, ts, tp)
    for chunk, spi, fuse, order, persist in [(256, 4, 0, 1, 1), (1000, 2, 300, 0, 0), (65535, 8, 65535, 1, 1),
                                             (4096, 8, 0, 0, 0), (16384, 8, 4096, 1, 0)]:
        tr = pg.TreeTrainer(cfg)
        tr.set_tuning("chunk", chunk)
        tr.set_tuning("hist_spi", spi)
        tr.set_tuning("fuse_max", fuse)
        tr.set_tuning("cand_order", order)
        tr.set_tuning("persist", persist)
        b = pg.Tree(cfg, 5, 7)
        tr.train(b, ts, tp)
        assert np.array_equal(a.left_child, b.left_child)
        assert np.array_equal(a.features, b.features) and np.array_equal(a.thresholds, b.thresholds)
        assert np.array_equal(a.posteriors, b.posteriors)
    with pytest.raises(pg.PadentiError):
        pg.TreeTrainer(cfg).set_tuning("hist_spi", 3)
    with pytest.raises(pg.PadentiError):
        pg.TreeTrainer(cfg).set_tuning("cand_order", 2)


def test_train_tree_nine_classes_bit_exact():
    cfg, ts, tp, _ = depth_case(n_images=12, width=320, height=240, n_features=64, n_thresholds=50, parts=1,
                                samples=1000)
    tree = pg.Tree(cfg, 1, 9)
    pg.TreeTrainer(cfg).train(tree, ts, tp)
    _assert_same_tree(tree, _oracle_tree(cfg, ts, tp, 1, 9))


def test_train_tree_reference_plugin_int16():
    cfg, ts, tp, _ = depth1_case()
    tree = pg.Tree(cfg, 2, 7)
    pg.TreeTrainer(cfg).train(tree, ts, tp)
    _assert_same_tree(tree, _oracle_tree(cfg, ts, tp, 2, 7))


def test_train_tree_rgb_channel_diff():
    cfg, ts, tp, _ = rgb_case()
    tree = pg.Tree(cfg, 0, 8)
    pg.TreeTrainer(cfg).train(tree, ts, tp)
    _assert_same_tree(tree, _oracle_tree(cfg, ts, tp, 0, 8))


def test_predict_posterior_and_leaf_bit_exact():
    cfg, ts, tp, (px, lb, sm) = depth_case(n_images=16, n_features=64)
    tr = pg.TreeTrainer(cfg)
    trees = []
    for t in range(3):
        tree = pg.Tree(cfg, t, 7)
        tr.train(tree, ts, tp)
        trees.append(tree)
    clf = pg.Classifier(cfg)
    for tree in trees:
        clf << tree
    tpx, tlb, _ = pg.synth_depth(0, 3, 160, 120, first_image=1000)
    p = ob.params(cfg, tp)
    for i in range(3):
        mask = (tpx[i] < 3000).astype(np.uint8) if i == 1 else None
        g = clf.predict(tpx[i], mask)
        o = ob.predict_posterior(p, tpx[i], mask, [tree_tuple(t) for t in trees])
        assert np.array_equal(g.view(np.uint32), o.view(np.uint32))
        if mask is not None:
            assert np.all(g[:, mask == 0] == 0)
        for t, tree in enumerate(trees):
            gl = clf.predict_leaf(t, tpx[i], mask)
            ol = ob.predict_leaf(p, tpx[i], mask, tree.depth, tree.left_child, tree.features, tree.thresholds)
            assert np.array_equal(gl, ol)


def test_predict_rgb_bit_exact():
    cfg, ts, tp, (px, lb, sm) = rgb_case()
    tree = pg.Tree(cfg, 0, 8)
    pg.TreeTrainer(cfg).train(tree, ts, tp)
    clf = pg.Classifier(cfg)
    clf << tree
    g = clf.predict(px[0])
    o = ob.predict_posterior(ob.params(cfg, tp), px[0], None, [tree_tuple(tree)], n_channels=3)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))


def test_upload_from_pinned_memory_by_sm_copy():
    """A training set in pinned host memory goes up through the SM copy kernel (the
    default, upload_copy = 1) or the copy engine (0); both train the oracle's tree."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    from padenti_gb300 import _native as N

    cfg, ts, tp, _ = depth_case(n_images=10, n_features=32, n_thresholds=10)
    flat = ts.flat()
    pinned = {k: torch.empty(max(1, v.nbytes), dtype=torch.uint8, pin_memory=True) for k, v in flat.items()}
    for k, v in flat.items():
        pinned[k].numpy()[: v.nbytes] = v.view(np.uint8).reshape(-1)
    pf = {k: pinned[k].numpy()[: v.nbytes].view(v.dtype) for k, v in flat.items()}
    o = ob.train_tree(ob.params(cfg, tp), ob.OracleSet(ts, cfg), 4, 6, ts.priors)
    prior = np.ascontiguousarray(ts.priors, np.float32)
    for mode in (1, 0):
        tr = pg.TreeTrainer(cfg)
        N.check(N.lib().pd_ctx_set_tuning(tr.h, b"upload_copy", mode))
        N.check(N.lib().pd_dataset_upload(tr.h, C.byref(pg.TrainingSet.desc(pf))))
        t = pg.Tree(cfg, 4, 6)
        N.check(N.lib().pd_train_tree(tr.h, C.byref(tp.c()), 4, 1, 6, prior.ctypes.data, t.left_child.ctypes.data,
                                      t.features.ctypes.data, t.thresholds.ctypes.data, t.posteriors.ctypes.data))
        assert np.array_equal(t.left_child, o["left_child"]), mode
        assert np.array_equal(np.asarray(t.features, np.int32), o["features"]), mode
        assert np.array_equal(t.posteriors.view(np.uint32), o["posteriors"].view(np.uint32)), mode


def test_offsets_beyond_the_exact_division_range():
    """Offsets above 2^21 px*mm take the plugin's float path (roundf of the float quotient)
    in training and in prediction (the forest is then not all-fast: the prediction kernels
    with the per-visit test run); trees and posteriors equal the oracle's."""
    cfg, ts, tp, (px, lb, sm) = depth_case(n_images=8, n_features=64, n_thresholds=12)
    # the first probe's offsets reach 2^22 (it reads the background), the second's stay small
    big, small = 1 << 22, 60000
    tp = pg.TreeTrainerParameters(64, 12, [-big, -big, -small, -small], [big, big, small, small], -500, 9500, 20)
    p = ob.params(cfg, tp)
    o = ob.train_tree(p, ob.OracleSet(ts, cfg), 2, 6, ts.priors)
    t = pg.Tree(cfg, 2, 6)
    pg.TreeTrainer(cfg).train(t, ts, tp)
    assert (t.left_child >= 0).sum() >= 4
    assert np.array_equal(t.left_child, o["left_child"])
    assert np.array_equal(np.asarray(t.features, np.int32), o["features"])
    assert np.array_equal(t.posteriors.view(np.uint32), o["posteriors"].view(np.uint32))
    assert np.abs(np.asarray(t.features)[t.left_child >= 0]).max() > (1 << 21), "splits on float-path offsets"
    clf = pg.Classifier(cfg)
    clf << t
    want = ob.predict_posterior(p, px[0], None, [tree_tuple(t)])
    assert np.array_equal(clf.predict(px[0]).view(np.uint32), want.view(np.uint32))
    assert np.array_equal(clf.predict_leaf(0, px[0]), ob.predict_leaf(p, px[0], None, 6, t.left_child, t.features,
                                                                      t.thresholds))


def test_device_batch_prediction_matches_per_image():
    """pd_predict_posterior_device on three same-size images in device memory, with masks,
    gives each image's host-buffer posterior (which the other tests pin to the oracle)."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    from padenti_gb300 import _native as N

    cfg, ts, tp, (px, lb, sm) = depth_case(n_images=6, n_features=48, n_thresholds=12)
    t = pg.Tree(cfg, 1, 7)
    pg.TreeTrainer(cfg).train(t, ts, tp)
    clf = pg.Classifier(cfg)
    clf << t
    imgs = np.ascontiguousarray(px[:3])
    rng = np.random.default_rng(9)
    masks = (rng.random(imgs.shape) < 0.8).astype(np.uint8)
    H, W = imgs.shape[1:3]
    dimg = torch.from_numpy(imgs.view(np.int16)).cuda()
    dmask = torch.from_numpy(masks).cuda()
    dout = torch.zeros((3, cfg.n_classes, H, W), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()  # the buffers are ready before the context's stream uses them
    N.check(N.lib().pd_predict_posterior_device(clf.h, 3, dimg.data_ptr(), W, H, dmask.data_ptr(), dout.data_ptr()))
    N.check(N.lib().pd_ctx_sync(clf.h))
    got = dout.cpu().numpy()
    for i in range(3):
        assert np.array_equal(got[i].view(np.uint32), clf.predict(imgs[i], masks[i]).view(np.uint32)), i
