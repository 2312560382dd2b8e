"""Pins of the oracle against the reference's own device code (no GPU).

The reference's per-image histogram kernel (kernels/hist_update.cl:36-187), its
traversal kernel (kernels/predict.cl:36-85) and its posterior kernel
(kernels/predict.cl:88-117) are compiled as C from the Padenti sources
(oracle/ref_shim/ref_hist.c, ref_predict.c, over oracle/ref_shim/cl/cl_shim.h)
and executed over their NDRanges.  The host steps around them are restated here
from the reference's host code, line for line:

- node maps: every depth starts from a zero node image and runs depth-1
  `predict` launches over the labels image as mask, each followed by a copy of
  the prediction image into the node image
  (cl_tree_trainer_impl_traverse_ts.hpp:140-244);
- global histograms: per-image uint8 indicators summed into
  hist[frontier index][label-1][t][f] for the samples whose node lies in
  [startNode, endNode] and holds more than perLeafSamplesThr samples
  (cl_tree_trainer_impl_traverse_ts.hpp:518-617);
- forest posteriors: per tree, depth-1 `predict` launches and one
  `computePosterior`, summed over the masked pixels in tree order and divided
  by the number of trees (cl_classifier_impl.hpp:478-552);
- the split of each frontier node: the reference's learnBestFeature kernel
  (kernels/learn_best_feature.cl, compiled as C) and std::max_element
  (cl_tree_trainer_impl_learn_best_featthr.hpp:86-112).

On an oracle-trained tree every depth is checked: each sample's node, each
frontier node's K x T x F histogram, its winning split (identical, or an FP32
near-tie of the reference's float gains), the stored feature and threshold of
the winner, and every child posterior.  These tests skip where the Padenti
sources are absent (oracle/_ref is built from them).
"""
import ctypes as C

import numpy as np
import pytest

import oracle_bind as ob
from cases import actx_case, depth1_case, depth_case, rgb_case

_U = C.c_uint
_I = C.c_int


def _kernels(plugin):
    rk = ob.ref_kernels(plugin)
    if rk is None:
        pytest.skip("reference kernels not compiled here (oracle/_ref absent)")
    return rk


def _img_type(cfg):
    return 1 if np.dtype(cfg.img_dtype) == np.uint8 else 2


def _ref_node_map(rk, cfg, im, tree, steps, mask):
    """The node image of one image after `steps` predict launches (traverse_ts.hpp:140-244;
    cl_classifier_impl.hpp:480-516): starts from zeros; each launch writes the prediction
    image for masked pixels, which is then copied into the node image."""
    H, W = im.labels.shape[:2]
    lc, feats, thrs, posts = tree
    nodes = np.zeros((H, W), np.int32)
    img = np.ascontiguousarray(im.data)
    m = np.ascontiguousarray(mask, np.uint8)
    f = np.ascontiguousarray(np.asarray(feats, np.int32).reshape(-1))
    t = np.ascontiguousarray(np.asarray(thrs, np.int32))
    p = np.ascontiguousarray(posts, np.float32)
    for _ in range(steps):
        out = nodes.copy()
        rc = rk.ref_predict_step(_I(_img_type(cfg)), _U(cfg.n_channels), ob.P(img), _U(W), _U(H), ob.P(m),
                                 ob.P(lc), ob.P(f), _U(cfg.feat_dim), ob.P(t), _U(len(lc)), ob.P(p), ob.P(nodes),
                                 ob.P(out))
        assert rc == 0
        nodes = out
    return nodes


def _ref_indicators(rk, cfg, tp, im, nodes_img, tree_id, start, end, tree=None):
    """computePerImageHistogram over (nSamples, nFeatures), local (1, 256): uint8 [s][t][f];
    tree = (left children, posteriors) passed to the feature (null when None)."""
    keep = None
    if tree is not None:
        keep = (np.ascontiguousarray(tree[0], np.int32), np.ascontiguousarray(tree[1], np.float32))
        rk.ref_hist_tree(ob.P(keep[0]), ob.P(keep[1]))
    H, W = im.labels.shape[:2]
    S = len(im.samples)
    out = np.zeros((S, tp.n_thresholds, tp.n_features), np.uint8)
    lo = np.array(list(tp.feat_low_bounds) + [0] * 8, np.int32)[:8]
    up = np.array(list(tp.feat_up_bounds) + [0] * 8, np.int32)[:8]
    smp = np.ascontiguousarray(im.samples, np.uint32)
    img = np.ascontiguousarray(im.data)
    rc = rk.ref_per_image_hist(_I(_img_type(cfg)), _U(cfg.n_channels), ob.P(img), _U(W), _U(H), ob.P(nodes_img),
                               ob.P(smp), _U(S), _U(tp.n_features), _U(cfg.feat_dim), ob.P(lo), ob.P(up),
                               _U(tp.n_thresholds), _I(int(tp.thr_low_bound)), _I(int(tp.thr_up_bound)),
                               _U(tree_id), _I(int(start)), _I(int(end)), ob.P(out))
    if keep is not None:
        rk.ref_hist_tree(None, None)
    assert rc == 0
    return out


def _ancestor_at(leaf, depth):
    """The node a sample occupies at `depth` (root level 1): the ancestor of its final
    node at that level, or the final node itself when it ends higher up."""
    n = leaf.astype(np.int64).copy()
    lvl = np.floor(np.log2(n + 1)).astype(np.int64) + 1
    while np.any(lvl > depth):
        m = lvl > depth
        n[m] = (n[m] - 1) // 2
        lvl[m] -= 1
    return n.astype(np.int32)


def _exact_gain(h, tot, t, f):
    """The canonical gain of candidate (t, f) in float64 (entropy with the p <= 1e-6 cutoff)."""
    def ent(c, n):
        c = c[(c > 0) & (c * 1e6 > n)].astype(np.float64)
        return float(-(c / n * np.log2(c / n)).sum()) if n else 0.0

    cl = h[:, t, f].astype(np.float64)
    cr = tot.astype(np.float64) - cl
    N, nl, nr = float(tot.sum()), float(cl.sum()), float(cr.sum())
    return ent(tot.astype(np.float64), N) - (nl / N * ent(cl, nl) + nr / N * ent(cr, nr))


def _ref_learn(hist, tot, F, T, K):
    ref = ob.ref("learn")
    if ref is None:
        pytest.skip("reference learn_best_feature.cl not compiled here (oracle/_ref absent)")
    n = hist.shape[0]
    per_thread = 64
    n_threads = n * F * T // per_thread
    bf = np.zeros(n_threads, np.uint32)
    bt = np.zeros(n_threads, np.uint32)
    be = np.zeros(n_threads, np.float32)
    h = np.ascontiguousarray(hist, np.uint32)
    tt = np.ascontiguousarray(tot, np.uint32)
    ref.ref_learn_best_feature(ob.P(h), ob.P(tt), _U(F), _U(T), _U(K), _U(per_thread), ob.P(bf), ob.P(bt),
                               ob.P(be), C.c_size_t(n_threads))
    per_node = n_threads // n
    out = []
    for i in range(n):
        e = be[i * per_node:(i + 1) * per_node]
        b = int(np.argmax(e))  # std::max_element: the first maximum
        out.append((int(bt[i * per_node + b]), int(bf[i * per_node + b])))
    return out


CASES = {
    # the reference's own feature (test/feature.cl, short features): offsets +-60, thresholds +-200
    "depth_diff1": lambda: depth1_case(n_images=5, width=64, height=48, n_features=256, n_thresholds=8),
    # the depth-difference feature of the benchmark configurations (int features, +-60000 px*mm)
    "depth_diff2": lambda: depth_case(n_images=6, width=64, height=48, n_features=256, n_thresholds=8,
                                      samples=140, min_leaf=10),
    # the RGB channel-difference feature, 21 classes
    "channel_diff": lambda: rgb_case(n_images=4, width=48, height=40, n_features=256, n_thresholds=8,
                                     samples=200),
}


@pytest.mark.parametrize("plugin", sorted(CASES))
def test_tree_depths_match_reference_kernels(plugin):
    rk = _kernels(plugin)
    cfg, ts, tp, _ = CASES[plugin]()
    depth, tree_id = 5, 3
    p = ob.params(cfg, tp)
    ds = ob.OracleSet(ts, cfg)
    o = ob.train_tree(p, ds, tree_id, depth, ts.priors)
    lc = o["left_child"]
    tree = (lc, o["features"], o["thresholds"], o["posteriors"])
    K, T, F = cfg.n_classes, tp.n_thresholds, tp.n_features
    thr = tp.per_leaf_samples_thr
    labels = np.concatenate([im.labels.reshape(-1)[im.samples] for im in ts.images]).astype(np.int64)
    img_of = np.concatenate([np.full(len(im.samples), i) for i, im in enumerate(ts.images)])
    assert o["nodes_split"] >= 3, "the case should split more than the root"
    checked_nodes = 0
    eps = (3 * K + 3) * 4.4e-7
    for d in range(1, depth):
        node_d = _ancestor_at(o["sample_leaf"], d)
        maps = [_ref_node_map(rk, cfg, im, tree, d - 1, im.labels != 0) for im in ts.images]
        ref_node = np.concatenate([m.reshape(-1)[im.samples] for m, im in zip(maps, ts.images)])
        # a10: the reference's traversal puts every sample on the oracle's node
        assert np.array_equal(ref_node, node_d), d
        tot = np.bincount(node_d, minlength=len(lc))
        level = np.arange((1 << (d - 1)) - 1, (1 << d) - 1)
        frontier = [int(n) for n in level if lc[n] != -2 and tot[n] > thr]
        if not frontier:
            break
        start, end = frontier[0], frontier[-1]
        idx = {n: i for i, n in enumerate(frontier)}
        href = np.zeros((len(frontier), K, T, F), np.uint32)
        for i, (im, m) in enumerate(zip(ts.images, maps)):
            ind = _ref_indicators(rk, cfg, tp, im, m, tree_id, start, end)
            sel = img_of == i
            for s, (n, lab) in enumerate(zip(ref_node[sel], labels[sel])):
                if start <= n <= end and tot[n] > thr:  # traverse_ts.hpp:533-535
                    href[idx[int(n)], lab - 1] += ind[s]
        # a5 + a6: the reference's indicators, summed as its host does, equal the oracle's histograms
        horc = ob.hist(p, ds, tree_id, node_d, frontier)
        assert np.array_equal(href, horc), d
        # a7: the reference's split (learnBestFeature + max_element) picks the oracle's winner,
        # or an FP32 near-tie of it
        ctot = np.stack([np.bincount(labels[node_d == n] - 1, minlength=K) for n in frontier]).astype(np.uint32)
        t, f, g, _, _ = ob.split(p, href, ctot)
        for i, n in enumerate(frontier):
            rt, rf = _ref_learn(href[i:i + 1], ctot[i:i + 1], F, T, K)[0]
            if (rt, rf) != (int(t[i]), int(f[i])) and t[i] >= 0:
                gap = g[i] - _exact_gain(href[i], ctot[i], rt, rf)
                assert -1e-12 <= gap <= 2 * eps, (d, n, gap)
            if lc[n] < 0:
                continue
            # a8: the stored split is candidate (t, f) regenerated from its seeds, and each
            # child's posterior is its class counts over its total, in float
            feat, thr_t = ob.candidate(p, tree_id, n, int(f[i]))
            assert np.array_equal(np.asarray(o["features"][n], np.int32), feat), (d, n)
            assert int(o["thresholds"][n]) == int(thr_t[t[i]]), (d, n)
            node_next = _ancestor_at(o["sample_leaf"], d + 1)
            for c in (2 * n + 1, 2 * n + 2):
                cnt = np.bincount(labels[node_next == c] - 1, minlength=K).astype(np.float32)
                post = (cnt / np.float32(cnt.sum())).astype(np.float32)
                assert np.array_equal(o["posteriors"][c].view(np.uint32), post.view(np.uint32)), (d, c)
            checked_nodes += 1
    assert checked_nodes >= 3


@pytest.mark.parametrize("plugin", sorted(CASES))
def test_forest_posterior_and_leaves_match_reference_kernels(plugin):
    rk = _kernels(plugin)
    cfg, ts, tp, _ = CASES[plugin]()
    p = ob.params(cfg, tp)
    ds = ob.OracleSet(ts, cfg)
    depth = 5
    trees = []
    for tid in (0, 1):
        o = ob.train_tree(p, ds, tid, depth, ts.priors)
        trees.append((depth, o["left_child"], o["features"], o["thresholds"], o["posteriors"]))
    K = cfg.n_classes
    rng = np.random.default_rng(2)
    for im in ts.images[:2]:
        H, W = im.labels.shape[:2]
        for mask in (np.ones((H, W), np.uint8), (rng.random((H, W)) < 0.6).astype(np.uint8)):
            # cl_classifier_impl.hpp:478-552
            post = np.zeros((K, H, W), np.float32)
            buf = np.zeros((K, H, W), np.float32)
            for (dep, lc, ft, th, po) in trees:
                nodes = _ref_node_map(rk, cfg, im, (lc, ft, th, po), dep - 1, mask)
                pp = np.ascontiguousarray(po, np.float32)
                rk.ref_compute_posterior(ob.P(nodes), _U(W), _U(H), _U(K), ob.P(pp), ob.P(mask), ob.P(buf))
                m = mask != 0
                for c in range(K):
                    post[c][m] = post[c][m] + buf[c][m]
                # leaf ids of this tree (predict(treeID, ...), cl_classifier_impl.hpp:200-341), masked pixels
                leaf = ob.predict_leaf(p, im.data, mask, dep, lc, ft, th, n_channels=cfg.n_channels)
                assert np.array_equal(leaf[m], nodes[m])
            post = (post / np.float32(len(trees))).astype(np.float32)
            o = ob.predict_posterior(p, im.data, mask, trees, n_channels=cfg.n_channels)
            assert np.array_equal(o.view(np.uint32), post.view(np.uint32))


@pytest.mark.parametrize("plugin", sorted(CASES))
def test_oracle_reproduces_reference_kernel_fixture(plugin):
    """The oracle gives the fixture's numbers (made from the reference's kernels by
    tests/golden/make_ref_kernel_golden.py): trees, and the frontier histograms of every depth
    given the reference's sample nodes.  Runs without the Padenti sources."""
    import hashlib
    import pathlib

    gold = dict(np.load(pathlib.Path(__file__).resolve().parent / "golden" / "ref_kernels.npz"))
    cfg, ts, tp, _ = CASES[plugin]()
    p = ob.params(cfg, tp)
    ds = ob.OracleSet(ts, cfg)
    for tid in (3, 0):
        o = ob.train_tree(p, ds, tid, 5, ts.priors)
        for k in ("left_child", "features", "thresholds", "posteriors"):
            assert np.array_equal(o[k], gold[f"{plugin}/tree{tid}_{k}"]), (tid, k)
    for d in range(1, 5):
        key = f"{plugin}/d{d}_hist_sha256"
        if key not in gold:
            continue
        h = ob.hist(p, ds, 3, gold[f"{plugin}/d{d}_sample_node"], gold[f"{plugin}/d{d}_frontier"])
        assert hashlib.sha256(np.ascontiguousarray(h).tobytes()).hexdigest() == str(gold[key]), d


# A feature that reads the tree (auto-context): oracle/ref_shim/cl/actx/feature.cl is
# the oracle's OR_PLUGIN_AUTO_CONTEXT as a Padenti feature.cl; the reference's kernels
# pass it their treeLeftChildren, treePosteriors and imageNodesID.
def _actx():
    return actx_case(n_images=4, width=64, height=48, n_features=256, n_thresholds=8, samples=200, min_leaf=10)


def test_auto_context_tree_depths_match_reference_kernels():
    """Every depth of an oracle-trained auto-context tree: the reference's traversal
    (with the tree passed to the feature) puts each sample on the oracle's node, and its
    per-image indicators over the node maps, summed as its host does, equal the oracle's
    histograms; the split and the stored candidate follow as for the other features."""
    rk = _kernels("auto_context")
    cfg, ts, tp, _ = _actx()
    depth, tree_id = 5, 3
    p = ob.params(cfg, tp, "auto_context")
    ds = ob.OracleSet(ts, cfg)
    o = ob.train_tree(p, ds, tree_id, depth, ts.priors)
    lc, posts = o["left_child"], o["posteriors"]
    tree = (lc, o["features"], o["thresholds"], posts)
    K, T, F = cfg.n_classes, tp.n_thresholds, tp.n_features
    thr = tp.per_leaf_samples_thr
    labels = np.concatenate([im.labels.reshape(-1)[im.samples] for im in ts.images]).astype(np.int64)
    img_of = np.concatenate([np.full(len(im.samples), i) for i, im in enumerate(ts.images)])
    assert o["nodes_split"] >= 3
    checked = 0
    for d in range(1, depth):
        node_d = _ancestor_at(o["sample_leaf"], d)
        maps = [_ref_node_map(rk, cfg, im, tree, d - 1, im.labels != 0) for im in ts.images]
        ref_node = np.concatenate([m.reshape(-1)[im.samples] for m, im in zip(maps, ts.images)])
        assert np.array_equal(ref_node, node_d), d
        tot = np.bincount(node_d, minlength=len(lc))
        level = np.arange((1 << (d - 1)) - 1, (1 << d) - 1)
        frontier = [int(n) for n in level if lc[n] != -2 and tot[n] > thr]
        if not frontier:
            break
        start, end = frontier[0], frontier[-1]
        idx = {n: i for i, n in enumerate(frontier)}
        href = np.zeros((len(frontier), K, T, F), np.uint32)
        for i, (im, m) in enumerate(zip(ts.images, maps)):
            ind = _ref_indicators(rk, cfg, tp, im, m, tree_id, start, end, tree=(lc, posts))
            sel = img_of == i
            for s, (n, lab) in enumerate(zip(ref_node[sel], labels[sel])):
                if start <= n <= end and tot[n] > thr:
                    href[idx[int(n)], lab - 1] += ind[s]
        horc = ob.hist_tree(p, ds, tree_id, node_d, frontier, maps, lc, posts, d - 1)
        assert np.array_equal(href, horc), d
        ctot = np.stack([np.bincount(labels[node_d == n] - 1, minlength=K) for n in frontier]).astype(np.uint32)
        t, f, g, _, _ = ob.split(p, href, ctot)
        for i, n in enumerate(frontier):
            if lc[n] < 0:
                continue
            feat, thr_t = ob.candidate(p, tree_id, n, int(f[i]))
            assert np.array_equal(np.asarray(o["features"][n], np.int32), feat), (d, n)
            assert int(o["thresholds"][n]) == int(thr_t[t[i]]), (d, n)
            checked += 1
    assert checked >= 3


def test_auto_context_forest_matches_reference_kernels():
    """Forest posterior and leaf maps of two auto-context trees: the reference's predict
    launches (the tree and the node image passed to the feature) and computePosterior,
    summed in tree order, equal the oracle's level-synchronous prediction."""
    rk = _kernels("auto_context")
    cfg, ts, tp, _ = _actx()
    p = ob.params(cfg, tp, "auto_context")
    ds = ob.OracleSet(ts, cfg)
    depth = 5
    trees = []
    for tid in (0, 1):
        o = ob.train_tree(p, ds, tid, depth, ts.priors)
        trees.append((depth, o["left_child"], o["features"], o["thresholds"], o["posteriors"]))
    K = cfg.n_classes
    rng = np.random.default_rng(2)
    for im in ts.images[:2]:
        H, W = im.labels.shape[:2]
        for mask in (np.ones((H, W), np.uint8), (rng.random((H, W)) < 0.6).astype(np.uint8)):
            post = np.zeros((K, H, W), np.float32)
            buf = np.zeros((K, H, W), np.float32)
            for (dep, lc, ft, th, po) in trees:
                nodes = _ref_node_map(rk, cfg, im, (lc, ft, th, po), dep - 1, mask)
                pp = np.ascontiguousarray(po, np.float32)
                rk.ref_compute_posterior(ob.P(nodes), _U(W), _U(H), _U(K), ob.P(pp), ob.P(mask), ob.P(buf))
                m = mask != 0
                for c in range(K):
                    post[c][m] = post[c][m] + buf[c][m]
                leaf = ob.predict_leaf(p, im.data, mask, dep, lc, ft, th, posts=po)
                assert np.array_equal(leaf[m], nodes[m])
            post = (post / np.float32(len(trees))).astype(np.float32)
            o = ob.predict_posterior(p, im.data, mask, trees)
            assert np.array_equal(o.view(np.uint32), post.view(np.uint32))


def test_auto_context_feature_reads_the_tree():
    """The auto-context oracle's training is self-consistent (every sample's node is the
    leaf its pixel reaches in level-synchronous prediction over the labels as mask), and
    the tree term matters: the same splits read without the tree route pixels differently."""
    cfg, ts, tp, _ = actx_case()
    p = ob.params(cfg, tp, "auto_context")
    ds = ob.OracleSet(ts, cfg)
    o = ob.train_tree(p, ds, 3, 6, ts.priors)
    lc = o["left_child"]
    assert (lc >= 0).sum() >= 8
    leaf, off, moved = o["sample_leaf"], 0, 0
    for im in ts.images:
        m = (im.labels != 0).astype(np.uint8)
        pl = ob.predict_leaf(p, im.data, m, 6, lc, o["features"], o["thresholds"], posts=o["posteriors"])
        s = im.samples
        assert np.array_equal(pl.reshape(-1)[s], leaf[off:off + len(s)])
        off += len(s)
        # the same tree with the posteriors zeroed: the context term changes, and so do leaves
        pz = ob.predict_leaf(p, im.data, m, 6, lc, o["features"], o["thresholds"],
                             posts=np.zeros_like(o["posteriors"]))
        moved += int((pz != pl).sum())
    assert moved > 0


def test_oracle_reproduces_auto_context_fixture():
    """The auto-context oracle gives the fixture's numbers from the reference's kernels
    (tests/golden/make_ref_kernel_golden.py): both trees, every depth's histograms given
    the reference's sample nodes and node maps (the oracle's own maps, labels as mask),
    the leaf maps and the two-tree forest posterior.  Runs without the Padenti sources."""
    import hashlib
    import pathlib

    def sha(a):
        return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()

    gold = dict(np.load(pathlib.Path(__file__).resolve().parent / "golden" / "ref_kernels.npz"))
    g = {k.split("/", 1)[1]: v for k, v in gold.items() if k.startswith("auto_context/")}
    cfg, ts, tp, _ = _actx()
    p = ob.params(cfg, tp, "auto_context")
    ds = ob.OracleSet(ts, cfg)
    trees = {}
    for tid in (3, 0):
        o = ob.train_tree(p, ds, tid, 5, ts.priors)
        trees[tid] = o
        for k in ("left_child", "features", "thresholds", "posteriors"):
            assert np.array_equal(o[k], g[f"tree{tid}_{k}"]), (tid, k)
    o = trees[3]
    for d in range(1, 5):
        if f"d{d}_hist_sha256" not in g:
            continue
        maps = [ob.predict_leaf(p, im.data, (im.labels != 0).astype(np.uint8), d, o["left_child"], o["features"],
                                o["thresholds"], posts=o["posteriors"]) for im in ts.images]
        node = np.concatenate([m.reshape(-1)[im.samples] for m, im in zip(maps, ts.images)])
        assert np.array_equal(node, g[f"d{d}_sample_node"]), d
        h = ob.hist_tree(p, ds, 3, node, g[f"d{d}_frontier"], maps, o["left_child"], o["posteriors"], d - 1)
        assert sha(h) == str(g[f"d{d}_hist_sha256"]), d
    forest = [(5, trees[t]["left_child"], trees[t]["features"], trees[t]["thresholds"], trees[t]["posteriors"])
              for t in (3, 0)]
    for i, im in enumerate(ts.images[:2]):
        H, W = im.labels.shape[:2]
        rng = np.random.default_rng(2)  # the generator's masks: the same draw for every image
        for mi, mask in enumerate([np.ones((H, W), np.uint8), (rng.random((H, W)) < 0.6).astype(np.uint8)]):
            for k, (dep, lc, ft, th, po) in enumerate(forest):
                leaf = ob.predict_leaf(p, im.data, mask, dep, lc, ft, th, posts=po)
                assert sha(leaf) == str(g[f"img{i}_mask{mi}_tree{k}_leaf_sha256"]), (i, mi, k)
            post = ob.predict_posterior(p, im.data, mask, forest)
            assert sha(post) == str(g[f"img{i}_mask{mi}_posterior_sha256"]), (i, mi)
