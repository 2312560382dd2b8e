"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py):
the oracle must reproduce them on CPU, and the CUDA path on the GPU."""
import hashlib
import pathlib
import sys

import numpy as np
import pytest

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))

import make_golden as mg  # noqa: E402
import padenti_gb300 as pg  # noqa: E402
from cases import sample_labels  # noqa: E402

NAMES = sorted(mg.CASES)


def _load(name):
    return dict(np.load(HERE / "golden" / f"{name}.npz"))


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(name):
    gold = _load(name)
    got = mg.compute(name)
    assert set(got) == set(gold)
    for k in gold:
        assert np.array_equal(np.asarray(got[k]), gold[k]), k


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_reproduces_golden(name):
    gold = _load(name)
    cfg, ts, tp, (px, lb, sm) = mg.CASES[name]()
    assert mg.digest(px, lb, sm) == str(gold["inputs_sha256"])
    tr = pg.TreeTrainer(cfg)
    tr.upload(ts)
    feat, thr = tr.candidates(tp, mg.TREE_ID, gold["cand_nodes"])
    assert np.array_equal(feat.reshape(-1, cfg.feat_dim).astype(np.int32), gold["cand_features"])
    assert np.array_equal(thr.reshape(-1, tp.n_thresholds).astype(np.int32), gold["cand_thresholds"])
    root = tr.hist(tp, mg.TREE_ID, np.zeros(ts.n_samples, np.int32), [0])
    assert np.array_equal(root, gold["root_hist"])
    ctot = np.bincount(sample_labels(ts), minlength=cfg.n_classes).astype(np.uint32)[None, :]
    t, f, g = tr.split(tp, root, ctot)
    assert [t[0], f[0]] == list(gold["root_split"]) and g[0] == gold["root_gain"][0]
    tree = pg.Tree(cfg, mg.TREE_ID, mg.DEPTH)
    tr.train(tree, ts, tp)
    assert np.array_equal(tree.left_child, gold["tree_left_child"])
    assert np.array_equal(tree.features.astype(np.int32), gold["tree_features"])
    assert np.array_equal(tree.thresholds.astype(np.int32), gold["tree_thresholds"])
    assert np.array_equal(tree.posteriors.view(np.uint32), gold["tree_posteriors"].view(np.uint32))
    assert np.array_equal(tr.sample_nodes(ts.n_samples), gold["tree_sample_leaf"])
    clf = pg.Classifier(cfg)
    clf << tree
    post = clf.predict(px[0])
    assert np.array_equal(np.argmax(post, axis=0).astype(np.uint8), gold["predict_argmax"])
    assert hashlib.sha256(np.ascontiguousarray(post).tobytes()).hexdigest() == str(gold["predict_sha256"])
