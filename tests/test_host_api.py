"""Host-side mirror of the reference API (no GPU): tree XML layout, priors,
parameters."""
import numpy as np
import pytest

import oracle_bind as ob
import padenti_gb300 as pg
from cases import depth_case


def _tree():
    cfg = pg.ForestConfig("depth_diff2", 3)
    t = pg.Tree(cfg, 4, 3)
    t.left_child[:] = [1, -1, 5, -2, -2, -1, -1]
    t.features[0] = [1, -2, 3, -4]
    t.thresholds[0] = -17
    t.features[2] = [5, 6, 7, 8]
    t.thresholds[2] = 9
    t.posteriors[:] = np.array([[0.1, 0.2, 0.7]] * 7, np.float32)
    t.posteriors[5] = [1 / 3, 1 / 3, 1 / 3]
    return cfg, t


def test_tree_xml_layout():
    cfg, t = _tree()
    x = t.to_xml()
    assert x.startswith('<?xml version="1.0" encoding="utf-8"?>\n<Trees><TreeNumber>1</TreeNumber><MaxDepth>3</MaxDepth><Tree4>')
    assert "<Node3>" not in x and "<Node4>" not in x  # absent nodes omitted (tree_impl.hpp:201)
    assert "<Node0><LeftChild>1</LeftChild><SplitParameters>1 -2 3 -4 -17</SplitParameters><Histogram>0.1 0.2 0.7</Histogram></Node0>" in x
    assert "<Histogram>0.333333 0.333333 0.333333</Histogram>" in x  # 6 significant digits
    assert "<Node1><LeftChild>-1</LeftChild><Histogram>" in x
    assert x.endswith("</Tree4></Trees>")
    assert "<Tree9>" in t.to_xml(idx=9)


def test_tree_xml_round_trip(tmp_path):
    cfg, t = _tree()
    p = tmp_path / "tree.xml"
    t.save(str(p))
    u = pg.Tree(cfg)
    u.load(str(p), 4)
    assert u.depth == 3 and u.id == 4
    assert np.array_equal(u.left_child, t.left_child)
    assert np.array_equal(u.features[[0, 2]], t.features[[0, 2]])
    assert np.array_equal(u.thresholds, t.thresholds)
    assert np.allclose(u.posteriors[t.left_child != -2], t.posteriors[t.left_child != -2], atol=5e-7)
    assert np.all(u.posteriors[t.left_child == -2] == 0)


def test_priors_mean_of_image_priors_matches_oracle():
    cfg, ts, tp, _ = depth_case(n_images=6)
    o = ob.priors(ob.OracleSet(ts, cfg), 3)
    assert np.array_equal(o.view(np.uint32), ts.priors.view(np.uint32))


def test_priors_incremental_operator():
    cfg, ts, tp, (px, lb, sm) = depth_case(n_images=4)
    inc = pg.TrainingSet(3)
    for i in range(4):
        inc << pg.TrainingSetImage(px[i], lb[i], 3, sm[i])
    exp = np.zeros(3, np.float32)
    for i, im in enumerate(inc.images):
        exp = (exp.astype(np.float64) * i / (i + 1) + im.priors.astype(np.float64) / (i + 1)).astype(np.float32)
    assert np.array_equal(inc.priors, exp)
    assert np.allclose(inc.priors, ts.priors, atol=1e-6)


def test_config_and_params():
    with pytest.raises(ValueError):
        pg.ForestConfig("nope", 3)
    cfg = pg.ForestConfig("channel_diff", 21)
    assert cfg.feat_dim == 6 and cfg.n_channels == 3 and cfg.img_dtype == np.uint8
    tp = pg.TreeTrainerParameters(10, 5, [0, 0, -30, -30, -30, -30], [3, 3, 30, 30, 30, 30], -255, 255, 7)
    c = tp.c()
    assert c.n_features == 10 and list(c.feat_up)[:6] == [3, 3, 30, 30, 30, 30] and c.per_leaf_samples_thr == 7


def test_bench_reads_the_committed_profile_figures():
    """bench.py's roofline objects take traffic and instruction figures from profiles/."""
    import importlib.util
    import pathlib

    root = pathlib.Path(__file__).resolve().parent.parent
    spec = importlib.util.spec_from_file_location("bench_mod", root / "bench.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    assert b.profile_traffic()["dram_bytes_per_launch"] > 1e9
    for k in ("k_sample_scan", "k_rgb_to_labels"):
        assert 0.5e6 < b.profile_dram_per_image(k) < 2e6
    assert b.profile_dram_per_image("no_such_kernel") is None


def test_oracle_synth_equals_library_synth():
    """The oracle's restatement of the synthetic depth maps (used where the CUDA library must not
    be loaded) gives the library's bytes."""
    import oracle_bind as ob

    for kw in (dict(parts=1, min_ellipses=2, max_ellipses=5, samples_per_image=2000, bg_permille=100),
               dict(parts=0, samples_per_image=500, first_image=7), dict(parts=1, samples_per_image=37,
                                                                          bg_permille=0)):
        a = pg.synth_depth(3, 4, 97, 61, **kw)
        b = ob.synth_depth(3, 4, 97, 61, **kw)
        for x, y in zip(a, b):
            assert np.array_equal(x, y), kw
