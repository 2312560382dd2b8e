"""Pixel samplers (UniformImageSampler, ClassWeightedImageSampler) on the GPU.

tests/golden/samplers.npz holds the samples the reference's own sampler sources return
(compiled here over libstdc++'s mt19937 and zlib's CRC-32; tests/golden/make_sampler_golden.py);
the CPU oracle must reproduce them, and the CUDA samplers must reproduce both, bit for bit.
"""
import ctypes as C
import pathlib

import numpy as np
import pytest

import oracle_bind as ob
import padenti_gb300 as pg
from cases import SAMPLER_CONFIGS, sampler_images, sampler_weights
from padenti_gb300 import _native as N

GOLDEN = np.load(pathlib.Path(__file__).parent / "golden" / "samplers.npz")


def _sampler(kind, ns, seed, k, rule):
    if kind == 1:
        return pg.UniformImageSampler(ns, seed)
    return pg.ClassWeightedImageSampler(ns, k, sampler_weights(rule, k), seed)


def _oracle(kind, data, labels, ns, seed, k, rule):
    if kind == 1:
        return ob.sample_uniform(data, labels, ns, seed)
    return ob.sample_class_weighted(data, labels, ns, k, sampler_weights(rule, k), seed)


# ------------------------------------------------------------------ CPU ------
def test_oracle_reproduces_reference_fixture():
    n = 0
    for name, _, data, labels, k in sampler_images():
        for cname, kind, ns, seed, rule in SAMPLER_CONFIGS:
            key = f"{cname}/{name}"
            if key not in GOLDEN:
                continue
            assert np.array_equal(_oracle(kind, data, labels, ns, seed, k, rule), GOLDEN[key]), key
            n += 1
    assert n == len(GOLDEN.files) - 1


def test_reference_sources_reproduce_the_fixture():
    """The fixture is what the reference's sampler sources return (where they were built)."""
    if ob.ref("sampler") is None:
        pytest.skip("reference sampler not built (Padenti sources absent at build time)")
    for name, img_type, data, labels, k in sampler_images():
        for cname, kind, ns, seed, rule in SAMPLER_CONFIGS:
            key = f"{cname}/{name}"
            if key not in GOLDEN:
                continue
            got = (ob.ref_sample_uniform(img_type, data, labels, ns, seed) if kind == 1 else
                   ob.ref_sample_class_weighted(img_type, data, labels, ns, k, sampler_weights(rule, k), seed))
            assert np.array_equal(got, GOLDEN[key]), key


def test_sampler_stride_and_argument_errors():
    assert pg.UniformImageSampler(500).stride == 500
    # ceil(float(1/9) * 2000) = 223 per class
    assert pg.ClassWeightedImageSampler(2000, 9).stride == 2007
    w = np.array([0.5, 0.25, 0.0], np.float32)
    assert pg.ClassWeightedImageSampler(1001, 3, w).stride == 501 + 251
    with pytest.raises(pg.PadentiError, match="outside"):
        _ = pg.ClassWeightedImageSampler(10, 0).stride
    with pytest.raises(pg.PadentiError, match="finite"):
        _ = pg.ClassWeightedImageSampler(10, 2, np.array([np.nan, 1], np.float32)).stride
    with pytest.raises(pg.PadentiError, match="max 16384"):
        _ = pg.UniformImageSampler(20000).stride
    with pytest.raises(pg.PadentiError, match="at least 1"):
        _ = pg.UniformImageSampler(0).stride


# ------------------------------------------------------------------ GPU ------
@pytest.mark.gpu
@pytest.mark.parametrize("cfg", SAMPLER_CONFIGS, ids=[c[0] for c in SAMPLER_CONFIGS])
def test_gpu_sampler_matches_reference_fixture_and_oracle(cfg):
    cname, kind, ns, seed, rule = cfg
    cases = sampler_images()
    for img_type in (2, 1):  # one batch per pixel type, images of mixed sizes
        sel = [c for c in cases if c[1] == img_type]
        k = sel[0][4]
        got = _sampler(kind, ns, seed, k, rule).sample_batch([c[2] for c in sel], [c[3] for c in sel])
        for (name, _, data, labels, _), g in zip(sel, got):
            want = _oracle(kind, data, labels, ns, seed, k, rule)
            assert np.array_equal(g, want), f"{cname}/{name}"
            key = f"{cname}/{name}"
            if key in GOLDEN:
                assert np.array_equal(g, GOLDEN[key]), key
            else:
                assert g.size == 0  # uniform sampler, no labelled pixel


@pytest.mark.gpu
def test_gpu_samplers_full_size_images():
    """640x480 and 1280x1024 depth maps (several checksum slices and many reservoir steps),
    2000 samples (the training configuration) and the largest stride."""
    px, lb, _ = pg.synth_depth(11, 4, 640, 480, parts=1, min_ellipses=2, max_ellipses=5, samples_per_image=4)
    big, blb, _ = pg.synth_depth(12, 1, 1280, 1024, parts=1, min_ellipses=3, max_ellipses=5, samples_per_image=4)
    images, labels = list(px) + [big[0]], list(lb) + [blb[0]]
    for s in [pg.UniformImageSampler(2000, 3), pg.UniformImageSampler(16384, 4),
              pg.ClassWeightedImageSampler(2000, 9, seed=5), pg.ClassWeightedImageSampler(16000, 9, seed=6)]:
        got = s.sample_batch(images, labels)
        for data, lab, g in zip(images, labels, got):
            if s.kind == 1:
                want = ob.sample_uniform(data, lab, s.n_samples, s.seed)
            else:
                want = ob.sample_class_weighted(data, lab, s.n_samples, 9, None, s.seed)
            assert np.array_equal(g, want)


@pytest.mark.gpu
def test_gpu_sampler_groups_and_device_entry():
    """Batches split into several staging groups give the same samples; pd_sample_device on
    images already in device memory gives the same samples as the host entry."""
    import torch

    px, lb, _ = pg.synth_depth(21, 6, 320, 240, parts=1, min_ellipses=2, max_ellipses=4, samples_per_image=4)
    s = pg.ClassWeightedImageSampler(1500, 9, seed=17)
    ref = s.sample_batch(list(px), list(lb))
    h = pg._sampler_ctx(0)
    N.check(N.lib().pd_ctx_set_tuning(h, b"sample_group", 200000))  # two images per group
    try:
        assert all(np.array_equal(a, b) for a, b in zip(ref, s.sample_batch(list(px), list(lb))))
        # the stacked-array form, through the two pipeline slots
        assert all(np.array_equal(a, b) for a, b in zip(ref, s.sample_batch(px, lb)))
    finally:
        N.check(N.lib().pd_ctx_set_tuning(h, b"sample_group", 512 << 20))
    dpx = torch.from_numpy(px.view(np.int16)).cuda()
    dlb = torch.from_numpy(lb).cuda()
    for sm in [s, pg.UniformImageSampler(777, 9)]:
        stride = sm.stride
        out = torch.zeros((6, stride), dtype=torch.int32, device="cuda")
        cnt = torch.zeros(6, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        N.check(N.lib().pd_sample_device(h, C.byref(sm._c(2)), 6, dpx.data_ptr(), dlb.data_ptr(), 320, 240, stride,
                                         out.data_ptr(), cnt.data_ptr()))
        o, c = out.cpu().numpy().view(np.uint32), cnt.cpu().numpy()
        want = sm.sample_batch(list(px), list(lb))
        for i in range(6):
            assert np.array_equal(o[i, :c[i]], want[i])
        st = sm.stats()
        assert st["images"] == 6 and st["kernel_launches"] == 2


@pytest.mark.gpu
def test_gpu_sampler_label_errors_and_empty_images():
    px, lb, _ = pg.synth_depth(3, 2, 64, 48, parts=1, samples_per_image=4)
    bad = lb[1].copy()
    bad[5, 5] = 10  # class 9 of a 9-class sampler
    with pytest.raises(pg.PadentiError, match="image 1 has a label above nClasses 9"):
        pg.ClassWeightedImageSampler(100, 9).sample_batch([px[0], px[1]], [lb[0], bad])
    # the uniform sampler takes any nonzero label; an image without labels gets no samples
    got = pg.UniformImageSampler(50, 1).sample_batch([px[0], px[1], px[1]], [lb[0], bad, np.zeros_like(bad)])
    assert np.array_equal(got[1], ob.sample_uniform(px[1], bad, 50, 1))
    assert got[2].size == 0


@pytest.mark.gpu
def test_sampled_training_set_trains_like_the_oracle():
    """TrainingSet(dir, …, sampler) without the loaders: GPU-sampled images, then a GPU tree
    equal to the oracle's on the same samples."""
    px, lb, _ = pg.synth_depth(31, 6, 160, 120, parts=0, samples_per_image=4)
    ts = pg.sampled_training_set(3, list(px), list(lb), pg.UniformImageSampler(400, 2))
    for im, d, lab in zip(ts.images, px, lb):
        assert np.array_equal(im.samples, ob.sample_uniform(d, lab, 400, 2))
    cfg = pg.ForestConfig("depth_diff2", 3)
    tp = pg.TreeTrainerParameters(48, 16, [-60000] * 4, [60000] * 4, -500, 500, 10)
    tree = pg.Tree(cfg, 2, 6)
    pg.TreeTrainer(cfg).train(tree, ts, tp)
    o = ob.train_tree(ob.params(cfg, tp), ob.OracleSet(ts, cfg), 2, 6, ts.priors)
    assert np.array_equal(tree.left_child, o["left_child"])
    assert np.array_equal(tree.thresholds, o["thresholds"])


@pytest.mark.gpu
def test_gpu_samplers_tiny_and_ragged_images():
    """Images of 1, 6, 17 and 255 pixels (shorter than one checksum block or label vector)
    beside a normal one, in one batch."""
    rng = np.random.default_rng(5)
    shapes = [(1, 1), (2, 3), (1, 17), (15, 17), (48, 64)]
    images = [rng.integers(0, 65536, s, dtype=np.uint16) for s in shapes]
    labels = [rng.integers(0, 4, s, dtype=np.uint8) for s in shapes]
    labels[0][:] = 2
    labels[1][:] = 0  # nothing labelled
    for s in [pg.UniformImageSampler(40, 9), pg.ClassWeightedImageSampler(60, 3, seed=4)]:
        got = s.sample_batch(images, labels)
        for d, lab, g in zip(images, labels, got):
            want = (ob.sample_uniform(d, lab, 40, 9) if s.kind == 1
                    else ob.sample_class_weighted(d, lab, 60, 3, None, 4))
            assert np.array_equal(g, want)
