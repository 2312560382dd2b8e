"""User feature plugins compiled at run time (the reference's feature.cl, here CUDA
source with computeFeature compiled by NVRTC).

Each built-in feature is written again as user source; a tree trained with it and its
forest prediction must be bit-identical to the built-in plugin's (which the parity tests
pin to the oracle).  Compilation itself needs no GPU.
"""
import numpy as np
import pytest

import oracle_bind as ob
import padenti_gb300 as pg
from cases import AUTO_CONTEXT_SOURCE, actx_case, depth1_case, depth_case, rgb_case

# kernels/feature.cl-style features written against pd::ImageView (read() is 0 outside)
SOURCES = {
    # the depth-difference feature of the benchmark configurations
    "depth_diff2": ("u16x1_i32x4", r"""
__device__ feat_t computeFeature(const pd::ImageView &img, int2 c, const feat_t *f, unsigned featDim) {
  int d = img.read(c.x, c.y, 0);
  if (d == 0) d = 10000;
  const float fd = (float)d;
  const int x1 = c.x + (int)roundf(__fdiv_rn((float)f[0], fd)), y1 = c.y + (int)roundf(__fdiv_rn((float)f[1], fd));
  const int x2 = c.x + (int)roundf(__fdiv_rn((float)f[2], fd)), y2 = c.y + (int)roundf(__fdiv_rn((float)f[3], fd));
  int a = img.read(x1, y1, 0), b = img.read(x2, y2, 0);
  if (a == 0) a = 10000;
  if (b == 0) b = 10000;
  return a - b;
}
"""),
    # the reference's own test/feature.cl: D(x) - D(x + round(u*500/D(x)))
    "depth_diff1": ("u16x1_i16x2", r"""
__device__ feat_t computeFeature(const pd::ImageView &img, int2 c, const feat_t *f, unsigned featDim) {
  const short depth = (short)img.read(c.x, c.y, 0);
  int probe = 10000;
  if (depth != 0) {
    const int ox = c.x + (int)roundf(__fdiv_rn(__fmul_rn((float)f[0], 500.0f), (float)depth));
    const int oy = c.y + (int)roundf(__fdiv_rn(__fmul_rn((float)f[1], 500.0f), (float)depth));
    const short v = (short)img.read(ox, oy, 0);
    probe = v ? v : 10000;
  }
  return (feat_t)(depth - probe);
}
"""),
    # RGB channel difference; channel indices clamped to [0, 2]
    "channel_diff": ("u8x3_i32x6", r"""
__device__ feat_t computeFeature(const pd::ImageView &img, int2 c, const feat_t *f, unsigned featDim) {
  const int c1 = min(max((int)f[0], 0), 2), c2 = min(max((int)f[1], 0), 2);
  return (int)img.read(c.x + f[2], c.y + f[3], c1) - (int)img.read(c.x + f[4], c.y + f[5], c2);
}
"""),
}
CASES = {"depth_diff2": lambda: depth_case(n_images=12, n_features=64, n_thresholds=20),
         "depth_diff1": lambda: depth1_case(),
         "channel_diff": lambda: rgb_case()}


def _user_config(name, n_classes):
    shape, src = SOURCES[name]
    return pg.ForestConfig("user", n_classes, source=src, shape=shape)


@pytest.mark.parametrize("name", sorted(SOURCES))
def test_user_plugin_compiles_without_a_gpu(name):
    cfg, *_ = CASES[name]()
    assert isinstance(pg.check_plugin(_user_config(name, cfg.n_classes)), str)


def test_user_plugin_compile_errors_carry_the_log():
    shape, src = SOURCES["depth_diff1"]
    bad = pg.ForestConfig("user", 3, source=src.replace("roundf", "no_such_function"), shape=shape)
    with pytest.raises(pg.PadentiError, match=r"feature\.cu\(\d+\): error: identifier \"no_such_function\""):
        pg.check_plugin(bad)


def test_user_plugin_config_needs_a_supported_shape():
    with pytest.raises(ValueError):
        pg.ForestConfig("user", 3, source="", shape="u16x1_i32x4")
    for bad in ("u16x5_i32x4", "u16x1_i32x9", "u16x1_i32x0", "f64x1_i32x4", "u16x1_f32x4"):
        with pytest.raises(ValueError):
            pg.ForestConfig("user", 3, source="x", shape=bad)
    assert pg.user_shape("f32x2_i16x7")["feat_dim"] == 7


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(SOURCES))
def test_user_plugin_trains_and_predicts_like_the_builtin(name):
    cfg, ts, tp, data = CASES[name]()
    ucfg = _user_config(name, cfg.n_classes)
    a = pg.Tree(cfg, 3, 7)
    pg.TreeTrainer(cfg).train(a, ts, tp)
    b = pg.Tree(ucfg, 3, 7)
    pg.TreeTrainer(ucfg).train(b, ts, tp)
    assert np.array_equal(a.left_child, b.left_child)
    assert np.array_equal(a.features, b.features) and np.array_equal(a.thresholds, b.thresholds)
    assert np.array_equal(a.posteriors.view(np.uint32), b.posteriors.view(np.uint32))
    assert (a.left_child >= 0).sum() > 3
    image = data[0][0]
    ca, cb = pg.Classifier(cfg), pg.Classifier(ucfg)
    ca << a
    cb << b
    assert np.array_equal(ca.predict(image).view(np.uint32), cb.predict(image).view(np.uint32))
    assert np.array_equal(ca.predict_leaf(0, image), cb.predict_leaf(0, image))
    (batch,) = cb.predict_batch([image])
    assert np.array_equal(batch.view(np.uint32), cb.predict(image).view(np.uint32))


@pytest.mark.gpu
def test_user_plugin_must_compile_before_use():
    from padenti_gb300 import _native as N
    import ctypes as C

    cfg, ts, tp, _ = depth1_case()
    ucfg = _user_config("depth_diff1", cfg.n_classes)
    h = C.c_void_p()
    N.check(N.lib().pd_ctx_create(C.byref(ucfg.c()), 0, C.byref(h)))
    try:
        rc = N.lib().pd_dataset_upload(h, C.byref(pg.TrainingSet.desc(ts.flat())))
        assert rc != 0 and b"pd_plugin_compile" in N.lib().pd_last_error()
    finally:
        N.lib().pd_ctx_destroy(h)


# Features of other types and dimensions than the built-in ones, each written so that it
# computes a built-in feature exactly: its trees and predictions must equal the built-in
# plugin's on the same data (which the parity tests pin to the oracle).
GENERIC = {
    # float images: the depth difference read from float32 depths
    "f32x1_i32x4": ("depth_diff2", lambda px: px.astype(np.float32), r"""
__device__ feat_t computeFeature(const pd::ImageView &img, int2 c, const feat_t *f, unsigned featDim) {
  int d = (int)img.read(c.x, c.y, 0);
  if (d == 0) d = 10000;
  const float fd = (float)d;
  const int x1 = c.x + (int)roundf(__fdiv_rn((float)f[0], fd)), y1 = c.y + (int)roundf(__fdiv_rn((float)f[1], fd));
  const int x2 = c.x + (int)roundf(__fdiv_rn((float)f[2], fd)), y2 = c.y + (int)roundf(__fdiv_rn((float)f[3], fd));
  int a = (int)img.read(x1, y1, 0), b = (int)img.read(x2, y2, 0);
  if (a == 0) a = 10000;
  if (b == 0) b = 10000;
  return a - b;
}
"""),
    # int16 images and FeatDim 3 (the third value unused): test/feature.cl
    "i16x1_i16x3": ("depth_diff1", lambda px: px.astype(np.int16), r"""
__device__ feat_t computeFeature(const pd::ImageView &img, int2 c, const feat_t *f, unsigned featDim) {
  const short depth = img.read(c.x, c.y, 0);
  int probe = 10000;
  if (depth != 0) {
    const int ox = c.x + (int)roundf(__fdiv_rn(__fmul_rn((float)f[0], 500.0f), (float)depth));
    const int oy = c.y + (int)roundf(__fdiv_rn(__fmul_rn((float)f[1], 500.0f), (float)depth));
    const short v = img.read(ox, oy, 0);
    probe = v ? v : 10000;
  }
  return (feat_t)(depth - probe);
}
"""),
    # four-channel images (RGBA, alpha unused): the RGB channel difference
    "u8x4_i32x6": ("channel_diff",
                   lambda px: np.concatenate([px, np.full(px.shape[:-1] + (1,), 255, np.uint8)], axis=-1), r"""
__device__ feat_t computeFeature(const pd::ImageView &img, int2 c, const feat_t *f, unsigned featDim) {
  const int c1 = min(max((int)f[0], 0), 2), c2 = min(max((int)f[1], 0), 2);
  return (int)img.read(c.x + f[2], c.y + f[3], c1) - (int)img.read(c.x + f[4], c.y + f[5], c2);
}
"""),
}


@pytest.mark.parametrize("shape", sorted(GENERIC))
def test_generic_user_plugin_compiles_without_a_gpu(shape):
    base, _, src = GENERIC[shape]
    assert isinstance(pg.check_plugin(pg.ForestConfig("user", 3, source=src, shape=shape)), str)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", sorted(GENERIC))
def test_generic_user_plugin_equals_the_builtin(shape):
    base, convert, src = GENERIC[shape]
    cfg, ts, tp, (px, lb, sm) = CASES[base]()
    ucfg = pg.ForestConfig("user", cfg.n_classes, source=src, shape=shape)
    upx = convert(px)
    uts = pg.training_set(cfg.n_classes, upx, lb, sm)
    D = cfg.feat_dim
    lo = list(tp.feat_low_bounds) + [0] * (ucfg.feat_dim - D)
    up = list(tp.feat_up_bounds) + [1] * (ucfg.feat_dim - D)
    utp = pg.TreeTrainerParameters(tp.n_features, tp.n_thresholds, lo, up, tp.thr_low_bound, tp.thr_up_bound,
                                   tp.per_leaf_samples_thr)
    a = pg.Tree(cfg, 3, 7)
    pg.TreeTrainer(cfg).train(a, ts, tp)
    b = pg.Tree(ucfg, 3, 7)
    pg.TreeTrainer(ucfg).train(b, uts, utp)
    assert (a.left_child >= 0).sum() > 3
    assert np.array_equal(a.left_child, b.left_child)
    assert np.array_equal(a.features, np.asarray(b.features)[:, :D]) and np.array_equal(a.thresholds, b.thresholds)
    assert np.array_equal(a.posteriors.view(np.uint32), b.posteriors.view(np.uint32))
    ca, cb = pg.Classifier(cfg), pg.Classifier(ucfg)
    ca << a
    cb << b
    assert np.array_equal(ca.predict(px[0]).view(np.uint32), cb.predict(upx[0]).view(np.uint32))
    assert np.array_equal(ca.predict_leaf(0, px[0]), cb.predict_leaf(0, upx[0]))
    # and directly against the oracle (the built-in feature on the original pixels)
    p = ob.params(cfg, tp)
    o = ob.train_tree(p, ob.OracleSet(ts, cfg), 3, 7, ts.priors)
    assert np.array_equal(b.left_child, o["left_child"])
    assert np.array_equal(np.asarray(b.features, np.int32)[:, :D], o["features"])
    assert np.array_equal(np.asarray(b.thresholds, np.int32), o["thresholds"])
    assert np.array_equal(b.posteriors.view(np.uint32), o["posteriors"].view(np.uint32))
    want = ob.predict_posterior(p, px[0], None, [(7, o["left_child"], o["features"], o["thresholds"],
                                                  o["posteriors"])], n_channels=cfg.n_channels)
    assert np.array_equal(cb.predict(upx[0]).view(np.uint32), want.view(np.uint32))


# A feature that reads the tree (auto-context): computeFeature takes a pd::TreeView and
# reads the node map through ImageView::nodeID; the library keeps a per-pixel node map.
def test_auto_context_plugin_compiles_without_a_gpu():
    assert isinstance(pg.check_plugin(pg.ForestConfig("user", 3, source=AUTO_CONTEXT_SOURCE, shape="u16x1_i32x4")),
                      str)


@pytest.mark.gpu
def test_auto_context_feature_matches_the_oracle():
    """Trees, forest posteriors (with and without a mask), leaf maps and the mixed batch of
    the auto-context feature, bit-identical to the oracle's OR_PLUGIN_AUTO_CONTEXT (which
    tests/test_reference_kernels.py pins to the reference's kernels)."""
    cfg, ts, tp, (px, lb, sm) = actx_case()
    p = ob.params(cfg, tp, "auto_context")
    ds = ob.OracleSet(ts, cfg)
    trainer = pg.TreeTrainer(cfg)
    clf = pg.Classifier(cfg)
    forest = []
    for tid in (3, 0):
        o = ob.train_tree(p, ds, tid, 6, ts.priors)
        t = pg.Tree(cfg, tid, 6)
        trainer.train(t, ts, tp)
        assert (o["left_child"] >= 0).sum() >= 8
        assert np.array_equal(t.left_child, o["left_child"]), tid
        assert np.array_equal(np.asarray(t.features, np.int32), o["features"]), tid
        assert np.array_equal(np.asarray(t.thresholds, np.int32), o["thresholds"]), tid
        assert np.array_equal(t.posteriors.view(np.uint32), o["posteriors"].view(np.uint32)), tid
        clf << t
        forest.append((6, o["left_child"], o["features"], o["thresholds"], o["posteriors"]))
    rng = np.random.default_rng(4)
    for image in px[:2]:
        mask = (rng.random(image.shape[:2]) < 0.7).astype(np.uint8)
        for m in (None, mask):
            want = ob.predict_posterior(p, image, m, forest)
            assert np.array_equal(clf.predict(image, m).view(np.uint32), want.view(np.uint32))
            for k, (dep, lc, ft, th, po) in enumerate(forest):
                assert np.array_equal(clf.predict_leaf(k, image, m), ob.predict_leaf(p, image, m, dep, lc, ft, th,
                                                                                     posts=po))
    # three same-size images in device memory: the node maps of all three in one set of steps
    import ctypes as C
    torch = pytest.importorskip("torch")
    from padenti_gb300 import _native as N
    imgs = np.ascontiguousarray(px[:3])
    H, W = imgs.shape[1:3]
    dimg = torch.from_numpy(imgs.view(np.int16)).cuda()
    dout = torch.zeros((3, cfg.n_classes, H, W), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()  # the buffers are ready before the context's stream uses them
    N.check(N.lib().pd_predict_posterior_device(clf.h, 3, dimg.data_ptr(), W, H, None, dout.data_ptr()))
    N.check(N.lib().pd_ctx_sync(clf.h))
    got = dout.cpu().numpy()
    for i in range(3):
        assert np.array_equal(got[i].view(np.uint32), ob.predict_posterior(p, imgs[i], None, forest).view(np.uint32)), i
    batch = clf.predict_batch([px[0], px[1][:40, :50]])
    assert np.array_equal(batch[0].view(np.uint32), ob.predict_posterior(p, px[0], None, forest).view(np.uint32))
    assert np.array_equal(batch[1].view(np.uint32),
                          ob.predict_posterior(p, np.ascontiguousarray(px[1][:40, :50]), None, forest).view(np.uint32))


@pytest.mark.gpu
def test_auto_context_refuses_the_histogram_stage_call():
    from padenti_gb300 import _native as N
    import ctypes as C

    cfg, ts, tp, _ = actx_case(n_images=2)
    trainer = pg.TreeTrainer(cfg)
    t = pg.Tree(cfg, 0, 3)
    trainer.train(t, ts, tp)  # uploads the set and compiles the plugin
    with pytest.raises(pg.PadentiError, match="node map"):
        trainer.hist(tp, 0, np.zeros(len(ts.flat()["samples"]), np.int32), np.array([0], np.int32))
