"""The header-only C++ facade (include/padenti/*.hpp) over the C ABI: the tree
XML interoperates byte for byte with the Python implementation, the prior rules
match, and (GPU) training + prediction through CUDATreeTrainer / CUDAClassifier
give exactly what the Python API gives."""
import pathlib
import shutil
import subprocess

import numpy as np
import pytest

import padenti_gb300 as pg
from cases import depth_case

ROOT = pathlib.Path(__file__).resolve().parent.parent
CPP = ROOT / "tests" / "cpp"


def _compile(src, out, link=False):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", f"-I{ROOT / 'include'}", str(src), "-o", str(out)]
    if link:
        from padenti_gb300.build import LIB
        cmd += [f"-L{LIB.parent}", "-lpadenti_gb300", f"-Wl,-rpath,{LIB.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_tree_xml_round_trip_between_python_and_cpp(tmp_path):
    exe = tmp_path / "facade_xml"
    _compile(CPP / "facade_xml.cpp", exe)
    cfg = pg.ForestConfig("depth_diff2", 3)
    t = pg.Tree(cfg, 5, 4)
    t.left_child[:] = [1, 3, -1, -1, -1, -2, -2, -2, -2, -2, -2, -2, -2, -2, -2]
    t.features[0] = [-1234, 56789, 0, -60000]
    t.thresholds[0] = -499
    t.features[1] = [1, 2, 3, 4]
    t.thresholds[1] = 17
    rng = np.random.default_rng(0)
    t.posteriors[:] = rng.random(t.posteriors.shape).astype(np.float32)
    t.posteriors[t.left_child == -2] = 0
    src, dst = tmp_path / "py.xml", tmp_path / "cpp.xml"
    t.save(str(src))
    r = subprocess.run([str(exe), str(src), "5", str(dst)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert dst.read_text() == src.read_text()
    mean, inc = r.stdout.split("|")
    # same prior rules as the Python mirror
    px = np.array([[1, 2], [3, 4]], np.uint16)
    lab = np.array([[1, 2], [2, 0]], np.uint8)
    a = pg.TrainingSetImage(px, lab, 3, np.array([0, 1, 2], np.uint32))
    b = pg.TrainingSetImage(px, lab, 3, np.array([1, 1], np.uint32))
    pm = pg.TrainingSet(3, [a, b]).priors
    pi = pg.TrainingSet(3)
    pi << a
    pi << b
    assert np.array_equal(np.array([float(x) for x in mean.split()], np.float32), pm)
    assert np.array_equal(np.array([float(x) for x in inc.split()], np.float32), pi.priors)


@pytest.mark.gpu
def test_cpp_facade_trains_and_predicts_like_the_python_api(tmp_path):
    exe = tmp_path / "facade_train"
    _compile(CPP / "facade_train.cpp", exe, link=True)
    xml, post = tmp_path / "tree.xml", tmp_path / "post.bin"
    r = subprocess.run([str(exe), str(xml), str(post)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    cfg, ts, tp, (px, lb, sm) = depth_case(n_images=8, n_features=64, n_thresholds=20)
    tree = pg.Tree(cfg, 3, 7)
    pg.TreeTrainer(cfg).train(tree, ts, tp)
    assert xml.read_text() == tree.to_xml()
    clf = pg.Classifier(cfg)
    clf << tree
    ref = clf.predict(px[0])
    got = np.fromfile(post, np.float32).reshape(ref.shape)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


@pytest.mark.gpu
def test_cpp_facade_with_a_user_feature_matches_the_builtin(tmp_path):
    """CUDATreeTrainer / CUDAClassifier built from a feature.cu directory (the reference's
    CLTreeTrainer(featureKernelPath)) train and predict exactly as with the built-in plugin."""
    from test_user_plugin import SOURCES

    exe = tmp_path / "facade_train"
    _compile(CPP / "facade_train.cpp", exe, link=True)
    fdir = tmp_path / "feature"
    fdir.mkdir()
    (fdir / "feature.cu").write_text(SOURCES["depth_diff2"][1])
    out = {}
    for tag, extra in (("builtin", []), ("user", [str(fdir)])):
        xml, post = tmp_path / f"{tag}.xml", tmp_path / f"{tag}.bin"
        r = subprocess.run([str(exe), str(xml), str(post), *extra], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr + r.stdout
        out[tag] = (xml.read_text(), post.read_bytes())
    assert out["user"] == out["builtin"]


def test_cpp_sampler_facade_compiles(tmp_path):
    _compile(CPP / "facade_sample.cpp", tmp_path / "facade_sample", link=True)


@pytest.mark.gpu
def test_cpp_sampler_facade_matches_the_oracle(tmp_path):
    """CUDAUniformImageSampler / CUDAClassWeightedImageSampler (sample(), sampleBatch() and
    sampledTrainingSet) return the oracle's samples."""
    import oracle_bind as ob

    exe = tmp_path / "facade_sample"
    _compile(CPP / "facade_sample.cpp", exe, link=True)
    r = subprocess.run([str(exe), str(tmp_path / "s.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    got = np.fromfile(tmp_path / "s.bin", np.uint32)
    px, lb, _ = pg.synth_depth(4, 4, 160, 120, min_ellipses=1, max_ellipses=3, parts=0, samples_per_image=1)
    w = np.array([0.5, 0.25, 0.3], np.float32)
    want = [ob.sample_uniform(px[i], lb[i], 500, 3) for i in range(4)]
    want += [ob.sample_class_weighted(px[i], lb[i], 400, 3, w, 7) for i in range(4)] * 2
    pos = 0
    for wv in want:
        n = int(got[pos])
        assert np.array_equal(got[pos + 1:pos + 1 + n], wv)
        pos += 1 + n
    assert pos == got.size
