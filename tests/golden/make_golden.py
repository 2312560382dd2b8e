"""Regenerates the golden fixtures of tests/golden/ from the CPU oracle.

    python tests/golden/make_golden.py

Each fixture holds a seeded small workload (identified by the sha256 of its
synthetic inputs) and the oracle's outputs on it: candidate vectors, a root
histogram, the best split, one trained tree with every sample's final node, and
the forest prediction of a held-out image.  The reference's own tests hold no
golden vectors for this path, so these fixtures pin the oracle (and, through
the GPU tests, the CUDA path) against later changes.
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
import padenti_gb300 as pg  # noqa: E402
from cases import depth1_case, depth_case, rgb_case, sample_labels, tree_tuple  # noqa: E402

CASES = {
    "depth_small": lambda: depth_case(n_images=8, n_features=32, n_thresholds=20),
    "depth1_small": lambda: depth1_case(n_images=6, n_features=24, n_thresholds=10),
    "rgb_small": lambda: rgb_case(n_images=6, n_features=24, n_thresholds=12),
}
DEPTH = 6
TREE_ID = 3


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def compute(name: str) -> dict:
    cfg, ts, tp, (px, lb, sm) = CASES[name]()
    p = ob.params(cfg, tp)
    ds = ob.OracleSet(ts, cfg)
    out = {"inputs_sha256": np.array(digest(px, lb, sm))}
    nodes = np.array([0, 5, 777], np.int32)
    feats, thrs = [], []
    for n in nodes:
        for f in range(tp.n_features):
            a, b = ob.candidate(p, TREE_ID, int(n), f)
            feats.append(a)
            thrs.append(b)
    out["cand_nodes"] = nodes
    out["cand_features"] = np.array(feats, np.int32)
    out["cand_thresholds"] = np.array(thrs, np.int32)
    root = ob.hist(p, ds, TREE_ID, np.zeros(ds.n_samples, np.int32), [0])
    out["root_hist"] = root
    ctot = np.bincount(sample_labels(ts), minlength=cfg.n_classes).astype(np.uint32)[None, :]
    t, f, g, _, _ = ob.split(p, root, ctot)
    out["root_split"] = np.array([t[0], f[0]], np.int32)
    out["root_gain"] = g
    tr = ob.train_tree(p, ds, TREE_ID, DEPTH, ts.priors)
    for k in ("left_child", "features", "thresholds", "posteriors", "sample_leaf"):
        out["tree_" + k] = tr[k]
    tree = (DEPTH, tr["left_child"], tr["features"], tr["thresholds"], tr["posteriors"])
    img = px[0]
    post = ob.predict_posterior(p, img, None, [tree], n_channels=cfg.n_channels)
    out["predict_argmax"] = np.argmax(post, axis=0).astype(np.uint8)
    out["predict_sha256"] = np.array(digest(post))
    return out


def main():
    for name in CASES:
        np.savez_compressed(HERE / f"{name}.npz", **compute(name))
        print("wrote", HERE / f"{name}.npz")


if __name__ == "__main__":
    main()
