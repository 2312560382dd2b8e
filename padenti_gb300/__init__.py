"""padenti_gb300 -- GB300-native training and prediction hot path of Padenti.

Python mirror of the reference's C++ API (src/padenti/): ``TrainingSetImage`` /
``TrainingSet`` (training_set*.hpp), ``Tree`` with its XML file layout
(tree.hpp, tree_impl.hpp), ``TreeTrainerParameters`` and ``TreeTrainer``
(tree_trainer.hpp, cl_tree_trainer.hpp) and ``Classifier``
(classifier.hpp, cl_classifier.hpp).  The reference's class template
parameters <ImgType, nChannels, FeatType, FeatDim, nClasses> are a
``ForestConfig``.  All compute runs in libpadenti_gb300.so (sm_103a CUDA
kernels behind the C ABI of include/padenti_gb300.h).
"""
from __future__ import annotations

import ctypes as C
import threading
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from ._native import PadentiError, check, lib

__all__ = [
    "ForestConfig", "TreeTrainerParameters", "TrainingSetImage", "TrainingSet", "Tree", "TreeTrainer",
    "Classifier", "PadentiError", "synth_depth", "synth_rgb", "PLUGINS", "USER_SHAPES", "user_shape", "check_plugin",
    "ImageSampler", "UniformImageSampler", "ClassWeightedImageSampler", "sampled_training_set",
    "ProposalNetwork", "RECORD_DTYPE", "read_pnm", "write_pnm", "PNMImageLoader", "RGBLabelsLoader", "load_training_set", "image_roi",
    "PNMImageROILoader", "RGBLabelsROILoader",
]

FEAT_DTYPE = {N.PD_FEAT_I16: np.int16, N.PD_FEAT_I32: np.int32}
IMG_DTYPE = {N.PD_IMG_U8: np.uint8, N.PD_IMG_U16: np.uint16, N.PD_IMG_I16: np.int16, N.PD_IMG_I32: np.int32,
             N.PD_IMG_F32: np.float32}

# Built-in feature plugins and the template parameters they are compiled for.
PLUGINS = {
    "depth_diff2": dict(plugin=N.PD_PLUGIN_DEPTH_DIFF2, img_type=N.PD_IMG_U16, n_channels=1,
                        feat_type=N.PD_FEAT_I32, feat_dim=4),
    "depth_diff1": dict(plugin=N.PD_PLUGIN_DEPTH_DIFF1, img_type=N.PD_IMG_U16, n_channels=1,
                        feat_type=N.PD_FEAT_I16, feat_dim=2),
    "channel_diff": dict(plugin=N.PD_PLUGIN_CHANNEL_DIFF, img_type=N.PD_IMG_U8, n_channels=3,
                         feat_type=N.PD_FEAT_I32, feat_dim=6),
}

# Types and dimensions a user feature (plugin "user", compiled at run time from
# CUDA source defining computeFeature) may have: those of the built-in plugins.
_IMG_CODES = {"u8": N.PD_IMG_U8, "u16": N.PD_IMG_U16, "i16": N.PD_IMG_I16, "i32": N.PD_IMG_I32, "f32": N.PD_IMG_F32}
_FEAT_CODES = {"i16": N.PD_FEAT_I16, "i32": N.PD_FEAT_I32}


def user_shape(shape: str) -> dict:
    """The template parameters of a user plugin from "<img><C>_<feat>x<D>": img in u8, u16, i16,
    i32, f32; C channels in 1..4; feat in i16, i32; FeatDim D in 1..8 (e.g. "u16x1_i32x4",
    "f32x1_i32x4", "u8x4_i32x6")."""
    import re

    m = re.fullmatch(r"(u8|u16|i16|i32|f32)x([1-4])_(i16|i32)x([1-8])", shape or "")
    if not m:
        raise ValueError(f"user plugin shape {shape!r}: expected <u8|u16|i16|i32|f32>x<1-4>_<i16|i32>x<1-8>")
    return dict(img_type=_IMG_CODES[m[1]], n_channels=int(m[2]), feat_type=_FEAT_CODES[m[3]], feat_dim=int(m[4]))


# the shapes of the built-in plugins, kept as names
USER_SHAPES = {s: user_shape(s) for s in ("u16x1_i32x4", "u16x1_i16x2", "u8x3_i32x6")}


def _ptr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


@dataclass(frozen=True)
class ForestConfig:
    """<ImgType, nChannels, FeatType, FeatDim, nClasses> for one plugin: a built-in one, or
    plugin="user" with the CUDA `source` of computeFeature (the reference's feature.cl) and a
    shape "<img><C>_<feat>x<D>" (user_shape)."""

    plugin: str
    n_classes: int
    source: str | None = None
    shape: str | None = None

    def __post_init__(self):
        if self.plugin == "user":
            if not self.source:
                raise ValueError("a user plugin needs its computeFeature source")
            user_shape(self.shape)
        elif self.plugin not in PLUGINS:
            raise ValueError(f"unknown plugin {self.plugin!r}; built-in: {sorted(PLUGINS)} or 'user'")

    @property
    def spec(self) -> dict:
        if self.plugin == "user":
            return dict(plugin=N.PD_PLUGIN_USER, **user_shape(self.shape))
        return PLUGINS[self.plugin]

    @property
    def img_dtype(self):
        return IMG_DTYPE[self.spec["img_type"]]

    @property
    def feat_dtype(self):
        return FEAT_DTYPE[self.spec["feat_type"]]

    @property
    def n_channels(self) -> int:
        return self.spec["n_channels"]

    @property
    def feat_dim(self) -> int:
        return self.spec["feat_dim"]

    def c(self) -> N.Config:
        s = self.spec
        return N.Config(s["plugin"], s["img_type"], s["n_channels"], s["feat_type"], s["feat_dim"], self.n_classes)


@dataclass
class TreeTrainerParameters:
    """tree_trainer.hpp:35-51 (computeFRange and randomThrSampling are unused there too)."""

    n_features: int
    n_thresholds: int
    feat_low_bounds: list
    feat_up_bounds: list
    thr_low_bound: int
    thr_up_bound: int
    per_leaf_samples_thr: int = 0

    def c(self) -> N.TrainParams:
        p = N.TrainParams()
        p.n_features = self.n_features
        p.n_thresholds = self.n_thresholds
        for i, v in enumerate(self.feat_low_bounds):
            p.feat_low[i] = int(v)
        for i, v in enumerate(self.feat_up_bounds):
            p.feat_up[i] = int(v)
        p.thr_low = int(self.thr_low_bound)
        p.thr_up = int(self.thr_up_bound)
        p.per_leaf_samples_thr = int(self.per_leaf_samples_thr)
        return p


class TrainingSetImage:
    """training_set_image.hpp: pixels, labels (0 = unlabelled, class k stored as k+1) and
    sampled pixel indices.  Priors over labelled samples (training_set_image_impl.hpp:38-52)."""

    def __init__(self, data: np.ndarray, labels: np.ndarray, n_classes: int, samples: np.ndarray):
        self.data = np.ascontiguousarray(data)
        self.labels = np.ascontiguousarray(labels, dtype=np.uint8)
        self.samples = np.ascontiguousarray(samples, dtype=np.uint32)
        self.height, self.width = self.labels.shape
        self.n_classes = n_classes
        lab = self.labels.reshape(-1)[self.samples]
        lab = lab[lab != 0]
        cnt = np.bincount(lab.astype(np.int64) - 1, minlength=n_classes)[:n_classes].astype(np.uint32)
        tot = np.float32(len(lab))
        self.priors = (cnt.astype(np.float32) / tot).astype(np.float32)


class TrainingSet:
    """training_set.hpp.  ``TrainingSet(n_classes, images)`` sets the priors to the mean of the
    per-image priors (training_set_impl.hpp:116-133); ``ts << image`` updates them incrementally
    as the reference's operator<< does (training_set_impl.hpp:157-170)."""

    def __init__(self, n_classes: int, images: list | None = None):
        self.n_classes = n_classes
        self.images: list[TrainingSetImage] = []
        self.priors = np.zeros(n_classes, np.float32)
        self._version = 0
        if images:
            self.images = list(images)
            acc = np.zeros(n_classes, np.float64)
            for im in self.images:
                acc += im.priors.astype(np.float64)
            self.priors = (acc / len(self.images)).astype(np.float32)

    def __lshift__(self, image: TrainingSetImage) -> "TrainingSet":
        n = len(self.images)
        pc = self.priors.astype(np.float64)
        self.priors = (pc * n / (n + 1) + image.priors.astype(np.float64) / (n + 1)).astype(np.float32)
        self.images.append(image)
        self._version += 1
        return self

    @property
    def n_samples(self) -> int:
        return int(sum(len(im.samples) for im in self.images))

    def flat(self) -> dict:
        """Concatenated host arrays in the layout of pd_dataset_desc."""
        n = len(self.images)
        pix = [np.ascontiguousarray(im.data).reshape(-1).view(np.uint8) for im in self.images]
        pix_off = np.zeros(n, np.uint64)
        lab_off = np.zeros(n, np.uint64)
        samp_off = np.zeros(n + 1, np.uint64)
        o = lo = 0
        for i, im in enumerate(self.images):
            pix_off[i], lab_off[i] = o, lo
            o += pix[i].nbytes
            lo += im.labels.size
            samp_off[i + 1] = samp_off[i] + len(im.samples)
        return dict(
            pixels=np.concatenate(pix) if n else np.zeros(1, np.uint8),
            pix_off=pix_off,
            width=np.array([im.width for im in self.images], np.uint32),
            height=np.array([im.height for im in self.images], np.uint32),
            labels=np.concatenate([im.labels.reshape(-1) for im in self.images]),
            lab_off=lab_off,
            samples=np.concatenate([im.samples for im in self.images]).astype(np.uint32),
            samp_off=samp_off,
        )

    @staticmethod
    def desc(flat: dict) -> N.DatasetDesc:
        d = N.DatasetDesc()
        d.n_images = len(flat["width"])
        for k in ("pixels", "pix_off", "width", "height", "labels", "lab_off", "samples", "samp_off"):
            setattr(d, k, flat[k].ctypes.data)
        return d


class Tree:
    """tree.hpp: complete binary heap of 2^depth-1 nodes as SoA arrays.  left_child is -2 for an
    absent node, -1 for a leaf, 2i+1 for a split node."""

    def __init__(self, config: ForestConfig, tree_id: int = 0, depth: int = 0):
        self.config = config
        self.id = tree_id
        self.depth = depth
        self._init()

    def _init(self):
        n = (1 << self.depth) - 1 if self.depth else 0
        self.left_child = np.full(n, -2, np.int32)
        self.features = np.zeros((n, self.config.feat_dim), self.config.feat_dtype)
        self.thresholds = np.zeros(n, self.config.feat_dtype)
        self.posteriors = np.zeros((n, self.config.n_classes), np.float32)

    @property
    def n_nodes(self) -> int:
        return len(self.left_child)

    # -- XML layout of tree_impl.hpp:103-234 (Boost.PropertyTree, no indentation) --
    def to_xml(self, idx: int = -1) -> str:
        tid = self.id if idx == -1 else idx
        out = [f"<Trees><TreeNumber>1</TreeNumber><MaxDepth>{self.depth}</MaxDepth><Tree{tid}>"]
        K = self.config.n_classes
        for i in range(self.n_nodes):
            c = int(self.left_child[i])
            if c == -2:
                continue
            out.append(f"<Node{i}><LeftChild>{c}</LeftChild>")
            if c != -1:
                vals = " ".join(str(int(v)) for v in self.features[i])
                out.append(f"<SplitParameters>{vals} {int(self.thresholds[i])}</SplitParameters>")
            hist = " ".join("%g" % float(self.posteriors[i, l]) for l in range(K))
            out.append(f"<Histogram>{hist}</Histogram></Node{i}>")
        out.append(f"</Tree{tid}></Trees>")
        return '<?xml version="1.0" encoding="utf-8"?>\n' + "".join(out)

    def save(self, path: str, idx: int = -1) -> None:
        with open(path, "w") as fh:
            fh.write(self.to_xml(idx))

    def load(self, path: str, idx: int = -1) -> None:
        root = ET.parse(path).getroot()
        if idx != -1:
            self.id = idx
        depth = int(root.findtext("MaxDepth"))
        if not self.depth or self.depth != depth:
            self.depth = depth
        self._init()
        t = root.find(f"Tree{self.id}")
        if t is None:
            return
        K, D = self.config.n_classes, self.config.feat_dim
        for node in t:
            i = int(node.tag[4:])
            c = int(node.findtext("LeftChild"))
            self.left_child[i] = c
            h = node.findtext("Histogram")
            if h is not None:
                self.posteriors[i] = np.array(h.split()[:K], np.float32)
            if c >= 0:
                v = node.findtext("SplitParameters").split()
                self.features[i] = np.array([int(x) for x in v[:D]], self.config.feat_dtype)
                self.thresholds[i] = int(v[D])


def check_plugin(config: ForestConfig) -> str:
    """Compiles a user plugin's source without a GPU; returns the compiler log, raises
    PadentiError (with the log) when it does not compile."""
    buf = C.create_string_buffer(1 << 16)
    rc = lib().pd_plugin_check(C.byref(config.c()), config.source.encode(), buf, len(buf))
    check(rc)
    return buf.value.decode()


class _Ctx:
    def __init__(self, config: ForestConfig, device: int = 0):
        self.config = config
        h = C.c_void_p()
        check(lib().pd_ctx_create(C.byref(config.c()), device, C.byref(h)))
        self.h = h
        if config.plugin == "user":
            check(lib().pd_plugin_compile(h, config.source.encode()))

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            lib().pd_ctx_destroy(h)
            self.h = None


class TreeTrainer(_Ctx):
    """CLTreeTrainer (cl_tree_trainer.hpp:115-120) on one GB300."""

    def __init__(self, config: ForestConfig, device: int = 0, hist_budget: int | None = None):
        super().__init__(config, device)
        self._uploaded = None
        if hist_budget:
            check(lib().pd_ctx_set_hist_budget(self.h, hist_budget))

    def set_tuning(self, name: str, value: int) -> None:
        """A knob of pd_ctx_set_tuning: launch shapes ("chunk", "hist_spi", "fuse_max", "cand_order", "persist",
        "cand_regs", "upload_copy"; results do not change) or "records" (keep split records)."""
        check(lib().pd_ctx_set_tuning(self.h, name.encode(), int(value)))

    def autotune(self, ts: TrainingSet, params: TreeTrainerParameters, end_depth: int, cache: str | None = None,
                 max_trials: int = 0) -> dict:
        """pd_autotune: searches the launch-shape knobs by timing trees of end_depth levels on `ts`
        (results never change), applies the best and caches it in the text file `cache`."""
        self.upload(ts)
        out = N.Tuning()
        check(lib().pd_autotune(self.h, C.byref(params.c()), end_depth, max_trials,
                                None if cache is None else str(cache).encode(), C.byref(out)))
        return {k: getattr(out, k) for k, _ in out._fields_}

    def upload(self, ts: TrainingSet) -> None:
        key = (id(ts), ts._version, len(ts.images))
        if self._uploaded == key:
            return
        flat = ts.flat()
        check(lib().pd_dataset_upload(self.h, C.byref(TrainingSet.desc(flat))))
        self._uploaded = key

    def train(self, tree: Tree, ts: TrainingSet, params: TreeTrainerParameters, start_depth: int = 1,
              end_depth: int | None = None) -> None:
        end_depth = tree.depth if end_depth is None else end_depth
        if end_depth > tree.depth:
            raise ValueError("end_depth exceeds the tree depth")
        self.upload(ts)
        n = (1 << end_depth) - 1
        lc = np.ascontiguousarray(tree.left_child[:n])
        ft = np.ascontiguousarray(tree.features[:n])
        th = np.ascontiguousarray(tree.thresholds[:n])
        po = np.ascontiguousarray(tree.posteriors[:n])
        prior = np.ascontiguousarray(ts.priors, np.float32)
        check(lib().pd_train_tree(self.h, C.byref(params.c()), tree.id, start_depth, end_depth, _ptr(prior),
                                  _ptr(lc), _ptr(ft), _ptr(th), _ptr(po)))
        tree.left_child[:n], tree.features[:n], tree.thresholds[:n], tree.posteriors[:n] = lc, ft, th, po

    def train_proposed(self, tree: Tree, ts: TrainingSet, params: TreeTrainerParameters, proposer: "ProposalNetwork",
                       n_proposed: int, end_depth: int | None = None) -> None:
        """train() with learned proposals: candidates f < n_proposed of every node are drawn from
        the proposal network's mixture, the others are the reference's uniform candidates."""
        end_depth = tree.depth if end_depth is None else end_depth
        self.upload(ts)
        n = (1 << end_depth) - 1
        lc = np.ascontiguousarray(tree.left_child[:n])
        ft = np.ascontiguousarray(tree.features[:n])
        th = np.ascontiguousarray(tree.thresholds[:n])
        po = np.ascontiguousarray(tree.posteriors[:n])
        prior = np.ascontiguousarray(ts.priors, np.float32)
        check(lib().pd_train_tree_proposed(self.h, proposer.h, C.byref(params.c()), n_proposed, tree.id, 1, end_depth,
                                           _ptr(prior), _ptr(lc), _ptr(ft), _ptr(th), _ptr(po)))
        tree.left_child[:n], tree.features[:n], tree.thresholds[:n], tree.posteriors[:n] = lc, ft, th, po

    def train_sharded(self, tree: Tree, ts: TrainingSet, params: TreeTrainerParameters, f_begin: int, f_end: int,
                      exchange, end_depth: int | None = None) -> None:
        """This rank's part of candidate-sharded training (pd_train_tree_sharded): it evaluates
        candidates [f_begin, f_end) of params.n_features, and exchange(key, idx, counts) ->
        (idx, counts) gives the global best split of every node of a slice (see
        padenti_gb300.dist: torch_exchange, LocalExchange).  Every rank ends with the same,
        unsharded tree."""
        from padenti_gb300 import dist as pdist

        end_depth = tree.depth if end_depth is None else end_depth
        self.upload(ts)
        n = (1 << end_depth) - 1
        lc = np.ascontiguousarray(tree.left_child[:n])
        ft = np.ascontiguousarray(tree.features[:n])
        th = np.ascontiguousarray(tree.thresholds[:n])
        po = np.ascontiguousarray(tree.posteriors[:n])
        prior = np.ascontiguousarray(ts.priors, np.float32)
        cb = pdist.c_exchange(exchange)
        check(lib().pd_train_tree_sharded(self.h, C.byref(params.c()), f_begin, f_end, C.cast(cb, C.c_void_p), None,
                                          tree.id, 1, end_depth, _ptr(prior), _ptr(lc), _ptr(ft), _ptr(th),
                                          _ptr(po)))
        tree.left_child[:n], tree.features[:n], tree.thresholds[:n], tree.posteriors[:n] = lc, ft, th, po

    def records(self) -> np.ndarray:
        """The records (one per split node) of the last training call; set_tuning("records", 1)
        before training to keep them."""
        n = C.c_uint64()
        check(lib().pd_train_records(self.h, None, 0, C.byref(n)))
        out = (N.Record * max(1, n.value))()
        check(lib().pd_train_records(self.h, C.cast(out, C.c_void_p), n.value, C.byref(n)))
        return np.ctypeslib.as_array(out)[: n.value].copy() if n.value else np.zeros(0, RECORD_DTYPE)

    def stats(self) -> dict:
        s = N.TrainStats()
        check(lib().pd_train_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    def sample_nodes(self, n_samples: int) -> np.ndarray:
        out = np.zeros(n_samples, np.int32)
        check(lib().pd_train_sample_nodes(self.h, _ptr(out)))
        return out

    # -- stage entry points of one depth --
    def candidates(self, params: TreeTrainerParameters, tree_id: int, nodes) -> tuple[np.ndarray, np.ndarray]:
        nodes = np.ascontiguousarray(nodes, np.int32)
        F, T, D = params.n_features, params.n_thresholds, self.config.feat_dim
        feat = np.zeros((len(nodes), F, D), self.config.feat_dtype)
        thr = np.zeros((len(nodes), F, T), self.config.feat_dtype)
        check(lib().pd_candidates(self.h, C.byref(params.c()), tree_id, _ptr(nodes), len(nodes), _ptr(feat),
                                  _ptr(thr)))
        return feat, thr

    def hist(self, params: TreeTrainerParameters, tree_id: int, sample_node, nodes) -> np.ndarray:
        nodes = np.ascontiguousarray(nodes, np.int32)
        sample_node = np.ascontiguousarray(sample_node, np.int32)
        K, T, F = self.config.n_classes, params.n_thresholds, params.n_features
        out = np.zeros((len(nodes), K, T, F), np.uint32)
        check(lib().pd_hist(self.h, C.byref(params.c()), tree_id, _ptr(sample_node), _ptr(nodes), len(nodes),
                            _ptr(out)))
        return out

    def split(self, params: TreeTrainerParameters, hist: np.ndarray, class_tot: np.ndarray):
        hist = np.ascontiguousarray(hist, np.uint32)
        class_tot = np.ascontiguousarray(class_tot, np.uint32)
        n = hist.shape[0]
        t = np.zeros(n, np.int32)
        f = np.zeros(n, np.int32)
        g = np.zeros(n, np.float64)
        check(lib().pd_split(self.h, C.byref(params.c()), _ptr(hist), _ptr(class_tot), n, _ptr(t), _ptr(f), _ptr(g)))
        return t, f, g

    def log2_table(self, n: int) -> np.ndarray:
        out = np.zeros(n, np.float64)
        check(lib().pd_log2_table(self.h, n, _ptr(out)))
        return out


RECORD_DTYPE = np.dtype([("depth", np.uint32), ("count", np.uint32), ("node", np.uint32), ("tree", np.uint32),
                         ("gain", np.float64), ("feat", np.int32, (8,)), ("thr", np.int32),
                         ("class_count", np.uint32, (64,))], align=True)


class ProposalNetwork:
    """The proposal network of learned candidate proposals (pd_proposer; no reference
    counterpart): a BF16 MLP on the trainer's GPU mapping a node's depth, log-count and class
    frequencies to a 16-component Gaussian mixture over the normalised feature values and
    threshold, fitted to the records of the plain trainer."""

    def __init__(self, trainer: TreeTrainer, bounds: TreeTrainerParameters, seed: int = 0):
        self.trainer = trainer  # keeps the context alive
        h = C.c_void_p()
        check(lib().pd_proposer_create(trainer.h, C.byref(bounds.c()), seed, C.byref(h)))
        self.h = h
        d = (C.c_uint32 * 6)()
        n = C.c_uint64()
        check(lib().pd_proposer_dims(h, d, C.byref(n)))
        self.in_dim, self.hidden, self.layers, self.out_dim, self.components, self.drawn = list(d)
        self.n_params = n.value

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            lib().pd_proposer_destroy(h)
            self.h = None

    @property
    def params(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        check(lib().pd_proposer_get_params(self.h, _ptr(out)))
        return out

    @params.setter
    def params(self, v: np.ndarray) -> None:
        v = np.ascontiguousarray(v, np.float32)
        if v.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters")
        check(lib().pd_proposer_set_params(self.h, _ptr(v)))

    def forward(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        out = np.zeros((x.shape[0], self.out_dim), np.float32)
        check(lib().pd_proposer_forward(self.h, _ptr(x), x.shape[0], _ptr(out)))
        return out

    def loss_grad(self, x: np.ndarray, y: np.ndarray, w: np.ndarray | None = None) -> tuple[float, np.ndarray]:
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        w = None if w is None else np.ascontiguousarray(w, np.float32)
        grad = np.zeros(self.n_params, np.float32)
        loss = C.c_float()
        check(lib().pd_proposer_loss_grad(self.h, _ptr(x), _ptr(y), _ptr(w), x.shape[0], C.byref(loss), _ptr(grad)))
        return loss.value, grad

    def fit(self, records: np.ndarray, steps: int = 400, batch: int = 4096, lr: float = 1e-3) -> dict:
        rec = np.ascontiguousarray(records, RECORD_DTYPE)
        loss = np.zeros(steps, np.float32)
        ms = C.c_float()
        check(lib().pd_proposer_fit(self.h, _ptr(rec), rec.size, steps, batch, C.c_float(lr), _ptr(loss),
                                    C.byref(ms)))
        return dict(loss=loss, ms=ms.value)


class Classifier(_Ctx):
    """CLClassifier (cl_classifier.hpp:81-94): a forest and per-pixel prediction."""

    def __init__(self, config: ForestConfig, device: int = 0):
        super().__init__(config, device)
        self.trees: list[Tree] = []

    def __lshift__(self, tree: Tree) -> "Classifier":
        check(lib().pd_forest_add_tree(self.h, tree.depth, _ptr(np.ascontiguousarray(tree.left_child)),
                                       _ptr(np.ascontiguousarray(tree.features)),
                                       _ptr(np.ascontiguousarray(tree.thresholds)),
                                       _ptr(np.ascontiguousarray(tree.posteriors))))
        self.trees.append(tree)
        return self

    def clear(self) -> None:
        check(lib().pd_forest_clear(self.h))
        self.trees = []

    def predict(self, image: np.ndarray, mask: np.ndarray | None = None) -> np.ndarray:
        """Posterior [nClasses][H][W] (cl_classifier_impl.hpp:356-557); masked-out pixels are 0."""
        image = np.ascontiguousarray(image, self.config.img_dtype)
        H, W = image.shape[:2]
        out = np.zeros((self.config.n_classes, H, W), np.float32)
        m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
        check(lib().pd_predict_posterior(self.h, _ptr(image), W, H, _ptr(m), _ptr(out)))
        return out

    def predict_batch(self, images: list, masks: list | None = None) -> list:
        """Posteriors of images of mixed sizes in one launch (pd_predict_posterior_batch)."""
        n = len(images)
        ims = [np.ascontiguousarray(im, self.config.img_dtype) for im in images]
        mks = [None if masks is None or masks[i] is None else np.ascontiguousarray(masks[i], np.uint8)
               for i in range(n)]
        outs = [np.empty((self.config.n_classes, im.shape[0], im.shape[1]), np.float32) for im in ims]
        P = C.c_void_p * n
        w = (C.c_uint32 * n)(*[im.shape[1] for im in ims])
        h = (C.c_uint32 * n)(*[im.shape[0] for im in ims])
        mp = P(*[None if m is None else m.ctypes.data for m in mks]) if masks is not None else None
        check(lib().pd_predict_posterior_batch(self.h, n, P(*[im.ctypes.data for im in ims]), w, h, mp,
                                               P(*[o.ctypes.data for o in outs])))
        return outs

    def predict_leaf(self, tree: int, image: np.ndarray, mask: np.ndarray | None = None) -> np.ndarray:
        """Leaf node id per pixel (cl_classifier_impl.hpp:200-341); masked-out pixels are 0."""
        image = np.ascontiguousarray(image, self.config.img_dtype)
        H, W = image.shape[:2]
        out = np.zeros((H, W), np.int32)
        m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
        check(lib().pd_predict_leaf(self.h, tree, _ptr(image), W, H, _ptr(m), _ptr(out)))
        return out


_SAMPLER_CTX: dict = {}
_SAMPLER_LOCK = threading.RLock()  # calls on one context are serialised (one stream, shared staging)


def _sampler_ctx(device: int):
    """A context per device for the samplers and the label loader (their own arguments fix
    the image type).  Callers hold _SAMPLER_LOCK while they use it."""
    with _SAMPLER_LOCK:
        h = _SAMPLER_CTX.get(device)
        if h is None:
            h = C.c_void_p()
            check(lib().pd_ctx_create(C.byref(ForestConfig("depth_diff2", 2).c()), device, C.byref(h)))
            _SAMPLER_CTX[device] = h
        return h


class ImageSampler:
    """ImageSampler (image_sampler.hpp:31-73) on the GPU: ``sample(data, labels)`` returns the
    sorted sampled pixel indices of one image, ``sample_batch`` those of many images (of any
    sizes) in one call.  The image's bytes (any dtype and channel count) seed the draws, as in
    the reference."""

    kind = 0

    def __init__(self, n_samples: int, seed: int = 0, device: int = 0):
        self.n_samples = int(n_samples)
        self.seed = int(seed) & 0xFFFFFFFF
        self.device = device
        self.n_classes = 0
        self._weights = None

    def _c(self, pixel_bytes: int = 1) -> N.Sampler:
        s = N.Sampler()
        s.kind, s.n_samples, s.seed, s.n_classes = self.kind, self.n_samples, self.seed, self.n_classes
        s.weights = None if self._weights is None else self._weights.ctypes.data
        s.pixel_bytes = pixel_bytes
        return s

    @property
    def stride(self) -> int:
        """Most samples one image can get (nSamples, or the sum of the class buckets)."""
        out = C.c_uint32()
        check(lib().pd_sampler_stride(C.byref(self._c()), C.byref(out)))
        return out.value

    def sample(self, data: np.ndarray, labels: np.ndarray) -> np.ndarray:
        return self.sample_batch([data], [labels])[0]

    def sample_batch(self, images, labels) -> list:
        """Samples of many images: lists of images and label images of any sizes, or one
        array of N same-size images ([N][H][W] or [N][H][W][C]) and one [N][H][W] label
        array.  Returns one index array per image (views into one result buffer)."""
        n = len(images)
        if n != len(labels):
            raise ValueError("one label image per image")
        if n == 0:
            return []
        stride = self.stride
        if isinstance(images, np.ndarray) and isinstance(labels, np.ndarray) and images.ndim >= 3:
            # stacked same-size images: pointers by arithmetic, no per-image Python work
            imgs = np.ascontiguousarray(images)
            lbs = np.ascontiguousarray(labels, np.uint8)
            if lbs.ndim != 3 or imgs.shape[:3] != lbs.shape:
                raise ValueError(f"images {imgs.shape} and labels {lbs.shape} differ in size")
            H, W = lbs.shape[1], lbs.shape[2]
            pixel_bytes = imgs[0].nbytes // max(H * W, 1)
            iptr = imgs.ctypes.data + np.arange(n, dtype=np.uint64) * np.uint64(imgs[0].nbytes)
            lptr = lbs.ctypes.data + np.arange(n, dtype=np.uint64) * np.uint64(H * W)
            w = np.full(n, W, np.uint32)
            h = np.full(n, H, np.uint32)
            keep = (imgs, lbs)
        else:
            imgs = [np.ascontiguousarray(a) for a in images]
            lbs = [np.ascontiguousarray(a, np.uint8) for a in labels]
            pb = {a.nbytes // max(a.shape[0] * a.shape[1], 1) for a in imgs}
            if len(pb) != 1:
                raise ValueError("all images of a batch need the same pixel type and channel count")
            pixel_bytes = pb.pop()
            for a, lb in zip(imgs, lbs):
                if a.shape[:2] != lb.shape:
                    raise ValueError(f"image {a.shape[:2]} and labels {lb.shape} differ in size")
            iptr = np.array([a.ctypes.data for a in imgs], np.uint64)
            lptr = np.array([a.ctypes.data for a in lbs], np.uint64)
            w = np.array([a.shape[1] for a in lbs], np.uint32)
            h = np.array([a.shape[0] for a in lbs], np.uint32)
            keep = (imgs, lbs)
        out = np.zeros((n, max(stride, 1)), np.uint32)
        counts = np.zeros(n, np.uint32)
        with _SAMPLER_LOCK:
            check(lib().pd_sample(_sampler_ctx(self.device), C.byref(self._c(pixel_bytes)), n, _ptr(iptr), _ptr(lptr),
                                  _ptr(w), _ptr(h), max(stride, 1), _ptr(out), _ptr(counts)))
        del keep
        return [row[:c] for row, c in zip(out, counts.tolist())]

    def _read_stats(self) -> dict:
        st = N.SampleStats()
        check(lib().pd_sample_get_stats(_sampler_ctx(self.device), C.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def stats(self) -> dict:
        """Counters and kernel times of the last call through this device's sampler context."""
        with _SAMPLER_LOCK:
            return self._read_stats()


class UniformImageSampler(ImageSampler):
    """UniformImageSampler (uniform_image_sampler_impl.hpp:34-63): n_samples labelled pixels,
    uniformly with replacement."""

    kind = N.PD_SAMPLER_UNIFORM


class ClassWeightedImageSampler(ImageSampler):
    """ClassWeightedImageSampler (classweighted_image_sampler_impl.hpp:25-120): a reservoir of
    ceil(weight_k * n_samples) pixels per class (weights None: 1/n_classes each)."""

    kind = N.PD_SAMPLER_CLASS_WEIGHTED

    def __init__(self, n_samples: int, n_classes: int, weights=None, seed: int = 0, device: int = 0):
        super().__init__(n_samples, seed, device)
        self.n_classes = int(n_classes)
        if weights is not None:
            self._weights = np.ascontiguousarray(weights, np.float32)
            if self._weights.shape != (self.n_classes,):
                raise ValueError("one weight per class")


def sampled_training_set(n_classes: int, images: list, labels: list, sampler: ImageSampler) -> TrainingSet:
    """TrainingSet(tsPath, …, sampler) (training_set_impl.hpp:40-112) without the image loaders:
    every image sampled by `sampler` (in one batch on the GPU), images and labels of different
    sizes skipped as the reference skips them."""
    keep = [i for i in range(len(images)) if np.shape(images[i])[:2] == np.shape(labels[i])]
    samples = sampler.sample_batch([images[i] for i in keep], [labels[i] for i in keep])
    return TrainingSet(n_classes, [TrainingSetImage(images[i], labels[i], n_classes, sm)
                                   for i, sm in zip(keep, samples)])


def read_pnm(path) -> np.ndarray:
    """A binary netpbm image: P5 (grey) as [H][W], P6 (RGB) as [H][W][3]; maxval < 256 gives
    uint8, else uint16 (stored big-endian, as the format says).  Stands in for the reference's
    OpenCV loaders (cv::imread), which are absent here."""
    with open(path, "rb") as f:
        raw = f.read()
    fields, pos = [], 0
    while len(fields) < 4:
        while raw[pos:pos + 1].isspace():
            pos += 1
        if raw[pos:pos + 1] == b"#":
            pos = raw.index(b"\n", pos) + 1
            continue
        end = pos
        while not raw[end:end + 1].isspace():
            end += 1
        fields.append(raw[pos:end])
        pos = end
    pos += 1  # the single whitespace byte before the pixels
    magic, w, h, maxval = fields[0], int(fields[1]), int(fields[2]), int(fields[3])
    if magic not in (b"P5", b"P6"):
        raise ValueError(f"{path}: not a binary PGM/PPM file")
    ch = 1 if magic == b"P5" else 3
    dt = np.dtype(np.uint8) if maxval < 256 else np.dtype(">u2")
    a = np.frombuffer(raw, dt, count=w * h * ch, offset=pos).astype(dt.newbyteorder("="))
    return a.reshape((h, w) if ch == 1 else (h, w, 3))


def write_pnm(path, image: np.ndarray) -> None:
    """Writes [H][W] (P5) or [H][W][3] (P6) uint8/uint16 as binary netpbm."""
    a = np.asarray(image)
    magic = b"P5" if a.ndim == 2 else b"P6"
    maxval = 255 if a.dtype == np.uint8 else 65535
    with open(path, "wb") as f:
        f.write(magic + b"\n%d %d\n%d\n" % (a.shape[1], a.shape[0], maxval))
        f.write(np.ascontiguousarray(a.astype(">u2") if maxval > 255 else a).tobytes())


class PNMImageLoader:
    """CVImageLoader (cv_image_loader_impl.hpp:37-73) for binary PGM/PPM files: ``load(path)``
    returns the image; its dtype and channel count must be the expected ones."""

    def __init__(self, dtype=np.uint16, n_channels: int = 1):
        self.dtype, self.n_channels = np.dtype(dtype), n_channels

    def load(self, path) -> np.ndarray:
        a = read_pnm(path)
        if a.dtype != self.dtype or (a.shape[2] if a.ndim == 3 else 1) != self.n_channels:
            raise ValueError(f"{path}: image type different from the expected one")
        return a


class RGBLabelsLoader:
    """CVRGBLabelsLoader (cv_image_loader.hpp:37-52): label images whose colours name the
    classes (``rgb2label[k]`` is the colour of class k).  ``convert`` maps an [H][W][3|4] RGB(A)
    image to labels (class k -> k+1, unknown colours -> 0) on the GPU; ``load`` reads a PPM file
    first."""

    def __init__(self, rgb2label, device: int = 0):
        self.map = np.ascontiguousarray(rgb2label, np.uint8).reshape(-1, 3)
        if not 1 <= len(self.map) <= 255:
            raise ValueError(f"{len(self.map)} colours (1 to 255 classes)")
        self.device = device

    def convert_batch(self, images: list) -> list:
        imgs = [np.ascontiguousarray(a, np.uint8) for a in images]
        if not imgs:
            return []
        ch = {a.shape[2] for a in imgs}
        if len(ch) != 1 or not ch <= {3, 4}:
            raise ValueError("label images of one batch need 3 or 4 channels, all the same")
        outs = [np.zeros(a.shape[:2], np.uint8) for a in imgs]
        n = len(imgs)
        ip = (C.c_void_p * n)(*[a.ctypes.data for a in imgs])
        op = (C.c_void_p * n)(*[o.ctypes.data for o in outs])
        w = np.array([a.shape[1] for a in imgs], np.uint32)
        h = np.array([a.shape[0] for a in imgs], np.uint32)
        with _SAMPLER_LOCK:
            check(lib().pd_rgb_to_labels(_sampler_ctx(self.device), n, ip, _ptr(w), _ptr(h), ch.pop(),
                                         _ptr(self.map), len(self.map), op))
        return outs

    def convert(self, image: np.ndarray) -> np.ndarray:
        return self.convert_batch([image])[0]

    def load(self, path) -> np.ndarray:
        return self.convert(read_pnm(path))


_ROI_TYPES = {np.dtype(np.uint8): N.PD_IMG_U8, np.dtype(np.uint16): N.PD_IMG_U16, np.dtype(np.int16): N.PD_IMG_I16,
              np.dtype(np.int32): N.PD_IMG_I32, np.dtype(np.float32): N.PD_IMG_F32}


def image_roi(image: np.ndarray) -> tuple:
    """_extractROI (cv_image_loader_impl.hpp:268-289): (x, y, width, height) of the largest
    bounding rectangle among the 8-connected components of the pixels whose value is > 0 (the
    reference's mask img > 0, compared in the image's own type), the one-pixel border counting
    as zero (pd_image_roi)."""
    a = np.ascontiguousarray(image)
    if a.dtype not in _ROI_TYPES:
        raise ValueError(f"image_roi: element type {a.dtype} (supported: {sorted(map(str, _ROI_TYPES))})")
    h, w = a.shape[:2]
    ch = a.size // max(w * h, 1)
    roi = np.zeros(4, np.uint32)
    check(lib().pd_image_roi(_ptr(a), w, h, _ROI_TYPES[a.dtype], ch, _ptr(roi)))
    return tuple(int(v) for v in roi)


class PNMImageROILoader(PNMImageLoader):
    """CVImageROILoader (cv_image_loader_impl.hpp:139-186): the image cropped to the ROI of its
    pixels > 0; ``roi_x``, ``roi_y`` (getRoiX, getRoiY) give the crop's corner."""

    roi_x = roi_y = 0

    def load(self, path) -> np.ndarray:
        a = super().load(path)
        x, y, w, h = image_roi(a)
        self.roi_x, self.roi_y = x, y
        return np.ascontiguousarray(a[y:y + h, x:x + w])


class RGBLabelsROILoader(RGBLabelsLoader):
    """CVRGBLabelsROILoader (cv_image_loader_impl.hpp:190-230): the labels (colours mapped on the
    GPU) cropped to the ROI of the labelled pixels; ``roi_x``, ``roi_y`` give the corner."""

    roi_x = roi_y = 0

    def convert(self, image: np.ndarray) -> np.ndarray:
        lab = RGBLabelsLoader.convert_batch(self, [image])[0]
        x, y, w, h = image_roi(lab)
        self.roi_x, self.roi_y = x, y
        return np.ascontiguousarray(lab[y:y + h, x:x + w])

    def convert_batch(self, images: list) -> list:
        return [self.convert(im) for im in images]


def load_training_set(path, data_suffix: str, labels_suffix: str, n_classes: int, data_loader: PNMImageLoader,
                      labels_loader: RGBLabelsLoader, sampler: ImageSampler) -> TrainingSet:
    """TrainingSet(tsPath, dataSuffix, labelsSuffix, nClasses, dataLoader, labelsLoader, sampler)
    (training_set_impl.hpp:40-112): every file ending in data_suffix with a labels file of the
    same stem; pairs of different sizes are skipped.  Files are taken in name order (the
    reference takes the directory's order).  Labels are converted and pixels sampled on the GPU,
    one batch each."""
    import os

    names = sorted(n for n in os.listdir(path) if n.endswith(data_suffix) and os.path.isfile(os.path.join(path, n)))
    datas, rgbs = [], []
    for n in names:
        lp = os.path.join(path, n[:len(n) - len(data_suffix)] + labels_suffix)
        if os.path.exists(lp):
            datas.append(data_loader.load(os.path.join(path, n)))
            rgbs.append(read_pnm(lp))
    labels = labels_loader.convert_batch(rgbs) if rgbs else []
    return sampled_training_set(n_classes, datas, labels, sampler)


def synth_depth(seed: int, n_images: int, width: int, height: int, *, first_image: int = 0, min_ellipses: int = 1,
                max_ellipses: int = 3, parts: int = 0, samples_per_image: int = 500, bg_permille: int = 100):
    """Seeded synthetic depth maps (uint16 mm), labels and sorted sample lists."""
    px = np.zeros((n_images, height, width), np.uint16)
    lb = np.zeros((n_images, height, width), np.uint8)
    sm = np.zeros((n_images, samples_per_image), np.uint32)
    check(lib().pd_synth_depth(seed, first_image, n_images, width, height, min_ellipses, max_ellipses, parts,
                               samples_per_image, bg_permille, _ptr(px), _ptr(lb), _ptr(sm)))
    return px, lb, sm


def synth_rgb(seed: int, n_images: int, width: int, height: int, *, first_image: int = 0, n_classes: int = 21,
              samples_per_image: int = 2000):
    """Seeded synthetic RGB Voronoi images (uint8 HxWx3), labels and sorted sample lists."""
    px = np.zeros((n_images, height, width, 3), np.uint8)
    lb = np.zeros((n_images, height, width), np.uint8)
    sm = np.zeros((n_images, samples_per_image), np.uint32)
    check(lib().pd_synth_rgb(seed, first_image, n_images, width, height, n_classes, samples_per_image, _ptr(px),
                             _ptr(lb), _ptr(sm)))
    return px, lb, sm


def training_set(n_classes: int, pixels: np.ndarray, labels: np.ndarray, samples: np.ndarray) -> TrainingSet:
    """TrainingSet from stacked arrays (priors = mean of per-image priors)."""
    return TrainingSet(n_classes, [TrainingSetImage(pixels[i], labels[i], n_classes, samples[i])
                                   for i in range(len(pixels))])
