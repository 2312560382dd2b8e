"""Regenerates tests/golden/ref_kernels.npz: outputs of the reference's own
device code -- kernels/hist_update.cl (computePerImageHistogram),
kernels/predict.cl (predict, computePosterior) and
kernels/learn_best_feature.cl, compiled as C from the Padenti sources
(oracle/ref_shim) -- on the seeded workloads of tests/test_reference_kernels.py,
so the GPU machine, which has no Padenti sources, can check the CUDA path against
them.

    make -C oracle ref REF=<Padenti source tree> && python tests/golden/make_ref_kernel_golden.py

Per workload (the reference's test/feature.cl, the depth-difference feature,
the RGB channel-difference feature, and a feature that reads the tree and the
node map, oracle/ref_shim/cl/actx/feature.cl): an oracle-trained tree (tree 3, depth 5)
that tests/test_reference_kernels.py checks depth by depth against the
reference kernels; for every depth, the frontier, each sample's node given by
the reference's traversal kernel and the sha256 of the frontier's histograms
summed from the reference's per-image indicators; a second tree (tree 0); and
the sha256 of the two-tree forest posterior and of both trees' leaf maps of the
first two images, from the reference's kernels, with and without a mask.
"""
from __future__ import annotations

import hashlib
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
sys.path.insert(0, str(HERE.parent))

import oracle_bind as ob  # noqa: E402
import test_reference_kernels as rkt  # noqa: E402

DEPTH = 5
TREE_ID = 3


def sha(a) -> np.ndarray:
    return np.array(hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest())


def masks_of(im):
    H, W = im.labels.shape[:2]
    rng = np.random.default_rng(2)
    return [np.ones((H, W), np.uint8), (rng.random((H, W)) < 0.6).astype(np.uint8)]


def compute(plugin: str) -> dict:
    rk = ob.ref_kernels(plugin)
    assert rk is not None, "build the reference kernels first (make -C oracle ref REF=...)"
    actx = plugin == "auto_context"
    cfg, ts, tp, (px, lb, sm) = rkt._actx() if actx else rkt.CASES[plugin]()
    p = ob.params(cfg, tp, plugin)
    ds = ob.OracleSet(ts, cfg)
    K, T, F = cfg.n_classes, tp.n_thresholds, tp.n_features
    out = {"inputs_sha256": sha(np.concatenate([px.reshape(-1).view(np.uint8), lb.reshape(-1),
                                                sm.reshape(-1).view(np.uint8)]))}
    trees = {}
    for tid in (TREE_ID, 0):
        o = ob.train_tree(p, ds, tid, DEPTH, ts.priors)
        trees[tid] = o
        out[f"tree{tid}_left_child"] = o["left_child"]
        out[f"tree{tid}_features"] = o["features"]
        out[f"tree{tid}_thresholds"] = o["thresholds"]
        out[f"tree{tid}_posteriors"] = o["posteriors"]
    o = trees[TREE_ID]
    lc = o["left_child"]
    tree = (lc, o["features"], o["thresholds"], o["posteriors"])
    labels = np.concatenate([im.labels.reshape(-1)[im.samples] for im in ts.images]).astype(np.int64)
    img_of = np.concatenate([np.full(len(im.samples), i) for i, im in enumerate(ts.images)])
    thr = tp.per_leaf_samples_thr
    for d in range(1, DEPTH + 1):
        maps = [rkt._ref_node_map(rk, cfg, im, tree, d - 1, im.labels != 0) for im in ts.images]
        node = np.concatenate([m.reshape(-1)[im.samples] for m, im in zip(maps, ts.images)]).astype(np.int32)
        out[f"d{d}_sample_node"] = node
        if d == DEPTH:
            break
        tot = np.bincount(node, minlength=len(lc))
        level = np.arange((1 << (d - 1)) - 1, (1 << d) - 1)
        frontier = np.array([int(n) for n in level if lc[n] != -2 and tot[n] > thr], np.int32)
        out[f"d{d}_frontier"] = frontier
        if not len(frontier):
            continue
        start, end = int(frontier[0]), int(frontier[-1])
        idx = {int(n): i for i, n in enumerate(frontier)}
        href = np.zeros((len(frontier), K, T, F), np.uint32)
        for i, (im, m) in enumerate(zip(ts.images, maps)):
            ind = rkt._ref_indicators(rk, cfg, tp, im, m, TREE_ID, start, end,
                                      tree=(lc, o["posteriors"]) if actx else None)
            sel = img_of == i
            for s, (n, lab) in enumerate(zip(node[sel], labels[sel])):
                if start <= n <= end and tot[n] > thr:
                    href[idx[int(n)], lab - 1] += ind[s]
        out[f"d{d}_hist_sha256"] = sha(href)
        out[f"d{d}_ref_split"] = np.array(rkt._ref_learn(
            href, np.stack([np.bincount(labels[node == n] - 1, minlength=K) for n in frontier]).astype(np.uint32),
            F, T, K), np.int32)
    forest = [(DEPTH, trees[t]["left_child"], trees[t]["features"], trees[t]["thresholds"], trees[t]["posteriors"])
              for t in (TREE_ID, 0)]
    for i, im in enumerate(ts.images[:2]):
        H, W = im.labels.shape[:2]
        for mi, mask in enumerate(masks_of(im)):
            post = np.zeros((K, H, W), np.float32)
            buf = np.zeros((K, H, W), np.float32)
            m = mask != 0
            for k, (dep, tlc, ft, th, po) in enumerate(forest):
                nodes = rkt._ref_node_map(rk, cfg, im, (tlc, ft, th, po), dep - 1, mask)
                pp = np.ascontiguousarray(po, np.float32)
                rk.ref_compute_posterior(ob.P(nodes), rkt._U(W), rkt._U(H), rkt._U(K), ob.P(pp), ob.P(mask), ob.P(buf))
                for c in range(K):
                    post[c][m] = post[c][m] + buf[c][m]
                out[f"img{i}_mask{mi}_tree{k}_leaf_sha256"] = sha(np.where(m, nodes, 0).astype(np.int32))
            post = (post / np.float32(len(forest))).astype(np.float32)
            out[f"img{i}_mask{mi}_posterior_sha256"] = sha(post)
    return out


def main() -> None:
    data = {}
    for plugin in sorted(rkt.CASES) + ["auto_context"]:
        for k, v in compute(plugin).items():
            data[f"{plugin}/{k}"] = v
    np.savez_compressed(HERE / "ref_kernels.npz", **data)
    print("wrote", HERE / "ref_kernels.npz")


if __name__ == "__main__":
    main()
