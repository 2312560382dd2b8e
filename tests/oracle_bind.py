"""ctypes binding of the CPU oracle (oracle/padenti_oracle.c) for the tests.

Test infrastructure: loads oracle/_build/libpadenti_oracle.so, building it with
``make -C oracle`` if it is missing.  The reference pieces compiled from the
Padenti sources (oracle/_ref) are optional: ``ref()`` returns None when absent.
"""
from __future__ import annotations

import ctypes as C
import pathlib
import subprocess

import numpy as np

REPO = pathlib.Path(__file__).resolve().parent.parent
ORACLE_SO = REPO / "oracle" / "_build" / "libpadenti_oracle.so"
REF_DIR = REPO / "oracle" / "_ref"

PLUGIN_IDS = {"depth_diff2": 1, "depth_diff1": 2, "channel_diff": 3, "auto_context": 16}
FEAT_IDS = {np.dtype(np.int16): 1, np.dtype(np.int32): 2}


class Params(C.Structure):
    _fields_ = [
        ("plugin", C.c_int32), ("feat_type", C.c_int32), ("feat_dim", C.c_int32), ("n_classes", C.c_int32),
        ("n_features", C.c_uint32), ("n_thresholds", C.c_uint32),
        ("feat_low", C.c_int32 * 8), ("feat_up", C.c_int32 * 8),
        ("thr_low", C.c_int32), ("thr_up", C.c_int32), ("per_leaf_samples_thr", C.c_uint32),
    ]


class Dataset(C.Structure):
    _fields_ = [
        ("n_images", C.c_uint32), ("n_channels", C.c_uint32), ("img_type", C.c_uint32),
        ("pixels", C.c_void_p), ("pix_off", C.c_void_p), ("width", C.c_void_p), ("height", C.c_void_p),
        ("labels", C.c_void_p), ("lab_off", C.c_void_p), ("samples", C.c_void_p), ("samp_off", C.c_void_p),
    ]


class Stats(C.Structure):
    _fields_ = [("evals", C.c_uint64), ("nodes_trained", C.c_uint64), ("nodes_split", C.c_uint64),
                ("seconds_hist", C.c_double), ("seconds_split", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not ORACLE_SO.exists():
            subprocess.run(["make", "-C", str(REPO / "oracle"), "all"], check=True, capture_output=True)
        _lib = C.CDLL(str(ORACLE_SO))
        _lib.or_feature.restype = C.c_int32
    return _lib


def ref(name: str):
    p = REF_DIR / f"libref_{name}.so"
    return C.CDLL(str(p)) if p.exists() else None


def P(a):
    """Pointer argument (ctypes would pass a bare int as a 32-bit C int)."""
    return None if a is None else C.c_void_p(a.ctypes.data)


def params(config, tp, plugin=None) -> Params:
    """Oracle parameters from a ForestConfig and TreeTrainerParameters (plugin: the
    oracle's feature when the config's is a user feature)."""
    p = Params()
    p.plugin = PLUGIN_IDS[plugin or config.plugin]
    p.feat_type = FEAT_IDS[np.dtype(config.feat_dtype)]
    p.feat_dim = config.feat_dim
    p.n_classes = config.n_classes
    p.n_features = tp.n_features
    p.n_thresholds = tp.n_thresholds
    for i, v in enumerate(tp.feat_low_bounds):
        p.feat_low[i] = int(v)
    for i, v in enumerate(tp.feat_up_bounds):
        p.feat_up[i] = int(v)
    p.thr_low = int(tp.thr_low_bound)
    p.thr_up = int(tp.thr_up_bound)
    p.per_leaf_samples_thr = int(tp.per_leaf_samples_thr)
    return p


class OracleSet:
    """Keeps the flattened arrays of a TrainingSet alive for the oracle."""

    def __init__(self, ts, config):
        self.flat = ts.flat()
        d = Dataset()
        d.n_images = len(self.flat["width"])
        d.n_channels = config.n_channels
        d.img_type = 1 if np.dtype(config.img_dtype) == np.uint8 else 2
        for k in ("pixels", "pix_off", "width", "height", "labels", "lab_off", "samples", "samp_off"):
            setattr(d, k, self.flat[k].ctypes.data)
        self.c = d
        self.n_samples = int(self.flat["samp_off"][-1])


def md5(words) -> tuple:
    a = (C.c_uint32 * 4)(*words)
    b = (C.c_uint32 * 4)()
    lib().or_md5(a, b)
    return tuple(b)


def candidate(p: Params, tree: int, node: int, f: int):
    feat = np.zeros(p.feat_dim, np.int32)
    thr = np.zeros(p.n_thresholds, np.int32)
    lib().or_candidate(C.byref(p), tree, node, f, P(feat), P(thr))
    return feat, thr


def log2_table(n: int) -> np.ndarray:
    out = np.zeros(n, np.float64)
    lib().or_log2_table(n, P(out))
    return out


def hist(p: Params, ds: OracleSet, tree: int, sample_node, nodes, reference_cost=False, threads=0):
    nodes = np.ascontiguousarray(nodes, np.int32)
    sample_node = np.ascontiguousarray(sample_node, np.int32)
    out = np.zeros((len(nodes), p.n_classes, p.n_thresholds, p.n_features), np.uint32)
    rc = lib().or_hist(C.byref(p), C.byref(ds.c), tree, P(sample_node), P(nodes), len(nodes), P(out),
                       int(reference_cost), threads)
    assert rc == 0
    return out


def hist_tree(p: Params, ds: OracleSet, tree: int, sample_node, nodes, maps, lc, post, level, threads=0):
    """hist for a feature that reads the tree: maps = every image's node map at `level`, lc / post the tree."""
    nodes = np.ascontiguousarray(nodes, np.int32)
    sample_node = np.ascontiguousarray(sample_node, np.int32)
    m = np.ascontiguousarray(np.concatenate([np.asarray(x, np.int32).reshape(-1) for x in maps]))
    out = np.zeros((len(nodes), p.n_classes, p.n_thresholds, p.n_features), np.uint32)
    rc = lib().or_hist_tree(C.byref(p), C.byref(ds.c), tree, P(sample_node), P(nodes), len(nodes), P(out), P(m),
                            P(np.ascontiguousarray(lc, np.int32)), P(np.ascontiguousarray(post, np.float32)),
                            C.c_int32(level), C.c_int32(len(lc)), threads)
    assert rc == 0
    return out


def split(p: Params, hist_, class_tot, table=None):
    hist_ = np.ascontiguousarray(hist_, np.uint32)
    class_tot = np.ascontiguousarray(class_tot, np.uint32)
    n = hist_.shape[0]
    if table is None:
        table = log2_table(int(class_tot.sum(axis=1).max()) + 2)
    t = np.zeros(n, np.int32)
    f = np.zeros(n, np.int32)
    g = np.zeros(n, np.float64)
    g32 = np.zeros(n, np.float32)
    err = C.c_double(0.0)
    rc = lib().or_split(C.byref(p), P(hist_), P(class_tot), n, P(table), C.c_uint64(len(table)), P(t), P(f), P(g),
                        P(g32), C.byref(err))
    assert rc == 0
    return t, f, g, g32, err.value


def priors(ds: OracleSet, n_classes: int) -> np.ndarray:
    out = np.zeros(n_classes, np.float32)
    lib().or_priors(C.byref(ds.c), n_classes, P(out))
    return out


def train_tree(p: Params, ds: OracleSet, tree_id: int, depth: int, root_prior, reference_cost=False, threads=0):
    n = (1 << depth) - 1
    lc = np.full(n, -2, np.int32)
    feats = np.zeros((n, p.feat_dim), np.int32)
    thrs = np.zeros(n, np.int32)
    posts = np.zeros((n, p.n_classes), np.float32)
    leaf = np.zeros(ds.n_samples, np.int32)
    st = Stats()
    prior = np.ascontiguousarray(root_prior, np.float32)
    rc = lib().or_train_tree(C.byref(p), C.byref(ds.c), tree_id, depth, P(prior), P(lc), P(feats), P(thrs),
                             P(posts), P(leaf), int(reference_cost), threads, C.byref(st))
    assert rc == 0
    return dict(left_child=lc, features=feats, thresholds=thrs, posteriors=posts, sample_leaf=leaf,
                evals=st.evals, nodes_split=st.nodes_split, seconds_hist=st.seconds_hist)


def predict_posterior(p: Params, image, mask, trees, n_channels=1, threads=0):
    """trees: list of (depth, left_child, features, thresholds, posteriors) with int32 features."""
    H, W = image.shape[:2]
    img = np.ascontiguousarray(image)
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    depth = np.array([t[0] for t in trees], np.uint32)
    off = np.zeros(len(trees), np.uint64)
    acc = 0
    for i, t in enumerate(trees):
        off[i] = acc
        acc += (1 << t[0]) - 1
    lc = np.ascontiguousarray(np.concatenate([t[1] for t in trees]), np.int32)
    ft = np.ascontiguousarray(np.concatenate([np.asarray(t[2], np.int32).reshape(-1) for t in trees]), np.int32)
    th = np.ascontiguousarray(np.concatenate([np.asarray(t[3], np.int32) for t in trees]), np.int32)
    po = np.ascontiguousarray(np.concatenate([np.asarray(t[4], np.float32).reshape(-1) for t in trees]), np.float32)
    out = np.zeros((p.n_classes, H, W), np.float32)
    rc = lib().or_predict_posterior(C.byref(p), P(img), W, H, n_channels, P(m), len(trees), P(depth), P(off), P(lc),
                                    P(ft), P(th), P(po), P(out), threads)
    assert rc == 0
    return out


def predict_leaf(p: Params, image, mask, depth, lc, feats, thrs, n_channels=1, threads=0, posts=None):
    """Leaf ids of one tree; posts (the tree's posteriors) for a feature that reads the tree."""
    H, W = image.shape[:2]
    img = np.ascontiguousarray(image)
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    out = np.zeros((H, W), np.int32)
    po = np.zeros((len(lc), p.n_classes), np.float32) if posts is None else np.ascontiguousarray(posts, np.float32)
    rc = lib().or_predict_leaf_tree(C.byref(p), P(img), W, H, n_channels, P(m), depth,
                                    P(np.ascontiguousarray(lc, np.int32)),
                                    P(np.ascontiguousarray(np.asarray(feats, np.int32).reshape(-1))),
                                    P(np.ascontiguousarray(np.asarray(thrs, np.int32))), P(po), P(out), threads)
    assert rc == 0
    return out


# ---------------------------------------------------------------- samplers ----
class MT(C.Structure):
    _fields_ = [("x", C.c_uint32 * 624), ("i", C.c_int)]


def crc32(data) -> int:
    b = np.ascontiguousarray(data).view(np.uint8).reshape(-1)
    lib().or_crc32.restype = C.c_uint32
    return int(lib().or_crc32(P(b), C.c_uint64(b.size)))


def mt_outputs(seed: int, n: int) -> np.ndarray:
    m = MT()
    lib().or_mt_seed(C.byref(m), C.c_uint32(seed))
    lib().or_mt_next.restype = C.c_uint32
    return np.array([lib().or_mt_next(C.byref(m)) for _ in range(n)], np.uint64).astype(np.uint32)


def uniform_ints(seed: int, range_: int, n: int) -> np.ndarray:
    m = MT()
    lib().or_mt_seed(C.byref(m), C.c_uint32(seed))
    lib().or_uniform_int.restype = C.c_uint32
    return np.array([lib().or_uniform_int(C.byref(m), C.c_uint32(range_)) for _ in range(n)], np.uint32)


def bucket_sizes(n_samples: int, n_classes: int, weights=None) -> np.ndarray:
    out = np.zeros(n_classes, np.uint32)
    w = None if weights is None else np.ascontiguousarray(weights, np.float32)
    lib().or_bucket_sizes(C.c_uint32(n_samples), C.c_uint32(n_classes), P(w), P(out))
    return out


def sample_uniform(data, labels, n_samples: int, seed: int) -> np.ndarray:
    d = np.ascontiguousarray(data)
    lb = np.ascontiguousarray(labels, np.uint8).reshape(-1)
    out = np.zeros(max(n_samples, 1), np.uint32)
    lib().or_sample_uniform.restype = C.c_uint32
    n = lib().or_sample_uniform(P(d), C.c_uint64(d.nbytes), P(lb), C.c_uint32(lb.size), C.c_uint32(n_samples),
                                C.c_uint32(seed), P(out))
    return out[:n]


def sample_class_weighted(data, labels, n_samples: int, n_classes: int, weights, seed: int) -> np.ndarray:
    d = np.ascontiguousarray(data)
    lb = np.ascontiguousarray(labels, np.uint8).reshape(-1)
    sizes = bucket_sizes(n_samples, n_classes, weights)
    out = np.zeros(max(int(sizes.sum()), 1), np.uint32)
    lib().or_sample_class_weighted.restype = C.c_int64
    n = lib().or_sample_class_weighted(P(d), C.c_uint64(d.nbytes), P(lb), C.c_uint32(lb.size),
                                       C.c_uint32(n_classes), P(sizes), C.c_uint32(seed), P(out))
    assert n >= 0, "label above n_classes"
    return out[:n]


def sample_batch(kind: int, images, labels, n_samples: int, seed: int, n_classes=0, weights=None):
    """Samples of a batch of same-size images on all host threads: (samples [n][stride], counts)."""
    imgs = np.ascontiguousarray(images)
    lbs = np.ascontiguousarray(labels, np.uint8)
    n = imgs.shape[0]
    sizes = bucket_sizes(n_samples, n_classes, weights) if kind == 2 else np.zeros(1, np.uint32)
    stride = n_samples if kind == 1 else int(sizes.sum())
    out = np.zeros((n, max(stride, 1)), np.uint32)
    counts = np.zeros(n, np.int64)
    lib().or_sample_batch(kind, P(imgs), C.c_uint64(imgs[0].nbytes), P(lbs), C.c_uint32(lbs[0].size),
                          C.c_uint32(n), C.c_uint32(n_samples), C.c_uint32(n_classes), P(sizes), C.c_uint32(seed),
                          C.c_uint32(max(stride, 1)), P(out), P(counts))
    return out, counts


def ref_sample_uniform(img_type: int, data, labels, n_samples: int, seed: int):
    """The reference's UniformImageSampler compiled from its sources (None when absent)."""
    r = ref("sampler")
    if r is None:
        return None
    d = np.ascontiguousarray(data)
    lb = np.ascontiguousarray(labels, np.uint8)
    h, w = lb.shape
    out = np.zeros(max(n_samples, 1), np.uint32)
    r.ref_sample_uniform.restype = C.c_uint
    n = r.ref_sample_uniform(img_type, P(d), P(lb), w, h, n_samples, C.c_uint(seed), P(out))
    return out[:n]


def ref_sample_class_weighted(img_type: int, data, labels, n_samples: int, n_classes: int, weights, seed: int):
    r = ref("sampler")
    if r is None:
        return None
    d = np.ascontiguousarray(data)
    lb = np.ascontiguousarray(labels, np.uint8)
    h, w = lb.shape
    sizes = bucket_sizes(n_samples, n_classes, weights)
    out = np.zeros(max(int(sizes.sum()), 1), np.uint32)
    wt = None if weights is None else np.ascontiguousarray(weights, np.float32)
    r.ref_sample_class_weighted.restype = C.c_uint
    n = r.ref_sample_class_weighted(img_type, P(d), P(lb), w, h, n_samples, n_classes, P(wt), C.c_uint(seed), P(out))
    return out[:n]


def rgb_to_labels(image, colours) -> np.ndarray:
    """_rgb2label on an [H][W][3|4] uint8 image; colours [K][3]."""
    img = np.ascontiguousarray(image, np.uint8)
    cmap = np.ascontiguousarray(colours, np.uint8).reshape(-1)
    out = np.zeros(img.shape[:2], np.uint8)
    lib().or_rgb_to_labels(P(img), C.c_uint64(out.size), C.c_uint32(img.shape[2]), P(cmap),
                           C.c_uint32(cmap.size // 3), P(out))
    return out


# ------------------------------------------------- reference kernels as C ----
REF_KERNEL_LIBS = {"depth_diff1": "kernels_dd1", "depth_diff2": "kernels_dd2", "channel_diff": "kernels_chd",
                   "auto_context": "kernels_actx"}


def ref_kernels(plugin: str):
    """The reference's hist_update.cl and predict.cl compiled as C with the plugin's
    feature.cl (oracle/ref_shim/ref_hist.c, ref_predict.c); None when absent."""
    r = ref(REF_KERNEL_LIBS[plugin])
    if r is not None:
        r.ref_per_image_hist.restype = C.c_int
        r.ref_predict_step.restype = C.c_int
        r.ref_hist_tree.restype = None
    return r


def synth_depth(seed: int, n_images: int, width: int, height: int, *, first_image: int = 0, min_ellipses: int = 1,
                max_ellipses: int = 3, parts: int = 0, samples_per_image: int = 500, bg_permille: int = 100):
    """The benchmark's seeded depth maps from the oracle's restatement (synth.c), without the
    CUDA library: the same bytes as padenti_gb300.synth_depth."""
    px = np.zeros((n_images, height, width), np.uint16)
    lb = np.zeros((n_images, height, width), np.uint8)
    sm = np.zeros((n_images, samples_per_image), np.uint32)
    rc = lib().or_synth_depth(C.c_uint64(seed), C.c_uint32(first_image), C.c_uint32(n_images), C.c_uint32(width),
                              C.c_uint32(height), C.c_uint32(min_ellipses), C.c_uint32(max_ellipses),
                              C.c_uint32(parts), C.c_uint32(samples_per_image), C.c_uint32(bg_permille), P(px),
                              P(lb), P(sm))
    assert rc == 0
    return px, lb, sm


def prop_forward(params, IN, H, OUT, x, bf16=True):
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros((x.shape[0], OUT), np.float32)
    rc = lib().or_prop_forward(P(np.ascontiguousarray(params, np.float32)), C.c_uint32(IN), C.c_uint32(H),
                               C.c_uint32(OUT), P(x), C.c_uint32(x.shape[0]), C.c_int(int(bf16)), P(out))
    assert rc == 0
    return out


def prop_loss_grad(params, IN, H, OUT, DY, x, y, w=None, bf16=True):
    params = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    w = None if w is None else np.ascontiguousarray(w, np.float32)
    grad = np.zeros(params.size, np.float64)
    loss = C.c_double()
    rc = lib().or_prop_loss_grad(P(params), C.c_uint32(IN), C.c_uint32(H), C.c_uint32(OUT), C.c_uint32(DY), P(x),
                                 P(y), P(w), C.c_uint32(x.shape[0]), C.c_int(int(bf16)), C.byref(loss), P(grad))
    assert rc == 0
    return loss.value, grad



def train_tree_sharded(p: Params, ds: OracleSet, tree_id: int, depth: int, root_prior, f0: int, f1: int, exchange,
                       threads=0):
    """or_train_tree_sharded with a Python exchange(key, idx, counts) -> (idx, counts)."""
    from padenti_gb300 import dist as pdist

    n = (1 << depth) - 1
    lc = np.full(n, -2, np.int32)
    feats = np.zeros((n, p.feat_dim), np.int32)
    thrs = np.zeros(n, np.int32)
    posts = np.zeros((n, p.n_classes), np.float32)
    leaf = np.zeros(ds.n_samples, np.int32)
    prior = np.ascontiguousarray(root_prior, np.float32)
    cb = pdist.c_exchange(exchange)  # kept alive for the call
    rc = lib().or_train_tree_sharded(C.byref(p), C.byref(ds.c), tree_id, depth, P(prior), C.c_uint32(f0),
                                     C.c_uint32(f1), cb, None, P(lc), P(feats), P(thrs), P(posts), P(leaf), threads)
    assert rc == 0, rc
    return dict(left_child=lc, features=feats, thresholds=thrs, posteriors=posts, sample_leaf=leaf)
