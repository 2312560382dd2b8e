#!/usr/bin/env python3
"""Benchmark of the Padenti training hot path on one GB300 (or N replicas).

Workload: 2000 synthetic 640x480 uint16 depth maps (2-5 ellipse bodies, 8 angular
part labels + background = 9 classes), 2000 sampled pixels per image, 2000
candidates x 50 thresholds per node, trees of depth 16 (levels 1..15 split),
min 20 pixels per leaf.  One step trains one whole tree through the C ABI
(pd_train_tree).  Metric: train feature-evals/s (one eval = one (sample,
candidate) response with its 50 threshold comparisons folded into the class
histogram).  Secondary: forest prediction Mpix/s over 500 held-out images.

The images (1.23 GB) are larger than L2, so no L2 flush is needed between steps.
`--impl reference` times the CPU restatement of the reference algorithm (the
reference itself needs OpenCL/Boost/OpenCV and does not build here) on all host
cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "train feature-evals/s"
UNIT = "evals/s"
WORKLOAD = "depth-diff forest, 2000x640x480 uint16 depth maps, 9 classes, 2000 samples/image, F=2000, T=50, depth 16"


def args_():
    a = argparse.ArgumentParser()
    a.add_argument("--gpus", type=int, default=1)
    a.add_argument("--steps", type=int, default=3)
    a.add_argument("--warmup", type=int, default=3)
    a.add_argument("--impl", default="ours", choices=["ours", "reference"])
    a.add_argument("--images", type=int, default=2000)
    a.add_argument("--width", type=int, default=640)
    a.add_argument("--height", type=int, default=480)
    a.add_argument("--samples", type=int, default=2000)
    a.add_argument("--features", type=int, default=2000)
    a.add_argument("--thresholds", type=int, default=50)
    a.add_argument("--depth", type=int, default=16)
    a.add_argument("--min-leaf", type=int, default=20)
    a.add_argument("--predict-images", type=int, default=500)
    a.add_argument("--e2e-steps", type=int, default=None)
    a.add_argument("--sampler-images", type=int, default=2000, help="images sampled by the pixel samplers (0: skip)")
    a.add_argument("--cpu-seconds", type=float, default=12.0, help="target length of the CPU baseline sample")
    a.add_argument("--no-cpu", action="store_true")
    a.add_argument("--seed", type=int, default=0)
    a.add_argument("--chunk", type=int, default=None, help="histogram work-item size (samples)")
    a.add_argument("--spi", type=int, default=None, help="samples per histogram-kernel iteration (2, 4 or 8)")
    a.add_argument("--fuse-max", type=int, default=None, help="largest node (samples) with the fused split")
    a.add_argument("--cand-order", type=int, default=None, choices=(0, 1),
                   help="1: candidate columns ordered by first-probe offset (default), 0: index order")
    a.add_argument("--learned", type=int, default=1, help="1: time the learned-proposal forest beside the plain one")
    a.add_argument("--autotune", type=int, default=1, help="1: launch shapes from pd_autotune before timing")
    a.add_argument("--mixed", type=int, default=1,
                   help="1: time the mixed-size configuration (5000 images of three sizes, depth 20)")
    a.add_argument("--fit-steps", type=int, default=100)
    a.add_argument("--fit-batch", type=int, default=4096)
    a.add_argument("--fit-lr", type=float, default=3e-3)
    a.add_argument("--only", default=None,
                   choices=["sampler_uniform", "sampler_class_weighted", "labels", "learned", "mixed", "fit"],
                   help="run one kernel family alone on --images synthetic images already in device memory "
                        "(--reps times) and print its times: the workload of the sampler and label profiles")
    a.add_argument("--reps", type=int, default=3)
    a.add_argument("--rgb-images", type=int, default=1000,
                   help="images of the RGB channel-difference configuration timed beside the headline (0: skip)")
    return a.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per histogram launch (mean over the launches of one tree of this
    workload) from the committed ncu summary profiles/k_hist_dram_2000x640x480.json."""
    p = ROOT / "profiles" / "k_hist_dram_2000x640x480.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return None
    return None


class Clocks:
    """nvidia-smi samples (SM clock, max clock, throttle reasons) during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.p = None
        return self

    def _read(self):
        for line in self.p.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def make_workload(a, rank: int):
    import padenti_gb300 as pg

    px, lb, sm = pg.synth_depth(a.seed, a.images, a.width, a.height, parts=1, min_ellipses=2, max_ellipses=5,
                                samples_per_image=a.samples, bg_permille=100)
    cfg = pg.ForestConfig("depth_diff2", 9)
    ts = pg.training_set(9, px, lb, sm)
    tp = pg.TreeTrainerParameters(a.features, a.thresholds, [-60000] * 4, [60000] * 4, -500, 500, a.min_leaf)
    return pg, cfg, ts, tp, (px, lb, sm)


def root_sample_set(a, m: int, lib_free: bool):
    """The first m images of the workload as a TrainingSet: from the library's generator, or
    (lib_free, for the reference arm) from the oracle's byte-identical restatement."""
    import padenti_gb300 as pg

    if lib_free:
        sys.path.insert(0, str(ROOT / "tests"))
        import oracle_bind as ob

        px, lb, sm = ob.synth_depth(a.seed, m, a.width, a.height, parts=1, min_ellipses=2, max_ellipses=5,
                                    samples_per_image=a.samples, bg_permille=100)
    else:
        px, lb, sm = pg.synth_depth(a.seed, m, a.width, a.height, parts=1, min_ellipses=2, max_ellipses=5,
                                    samples_per_image=a.samples, bg_permille=100)
    return pg.TrainingSet(9, [pg.TrainingSetImage(px[i], lb[i], 9, sm[i]) for i in range(m)])


def cpu_root(a, cfg, tp, sub, threads):
    """Root depth (histogram + split) of a training set on the host cores: the oracle in
    reference-cost mode (MD5 candidates regenerated per (sample, candidate), T comparisons per
    evaluation, as kernels/hist_update.cl does).  Returns (evals/s, seconds, samples)."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_bind as ob

    p = ob.params(cfg, tp)
    ds = ob.OracleSet(sub, cfg)
    node = np.zeros(ds.n_samples, np.int32)
    t0 = time.perf_counter()
    h = ob.hist(p, ds, 0, node, [0], reference_cost=True, threads=threads)
    labels = np.concatenate([im.labels.reshape(-1)[im.samples] for im in sub.images]).astype(np.int64) - 1
    ctot = np.bincount(labels, minlength=9).astype(np.uint32)[None, :]
    ob.split(p, h, ctot)
    dt = time.perf_counter() - t0
    return ds.n_samples * tp.n_features / dt, dt, ds.n_samples


def root_sample_text(m, n, tp, dt):
    return (f"root depth (histogram + split) of the first {m} images ({n} samples x {tp.n_features} candidates x "
            f"{tp.n_thresholds} thresholds), MD5 candidates regenerated per (sample, candidate) as the reference "
            f"kernel does; {dt:.1f} s")


def cpu_sample(a, cfg, tp, seconds: float, lib_free: bool = False):
    """The CPU baseline sample: the root depth of as many leading images as fill about `seconds`
    on all host cores."""
    threads = os.cpu_count() or 1
    _, dt, _ = cpu_root(a, cfg, tp, root_sample_set(a, 1, lib_free), threads)
    m = int(max(1, min(a.images, round(seconds / max(dt, 1e-3)))))
    rate, dt, n = cpu_root(a, cfg, tp, root_sample_set(a, m, lib_free), threads)
    return dict(value=rate, unit=UNIT, cores=threads, kind="port", sample=root_sample_text(m, n, tp, dt)), m


def gpu_root_sample(a, pg, cfg, tp, m: int, device: int):
    """The GPU on exactly the CPU baseline's sample: root depth (histogram + split) of the first
    m images through pd_train_tree with end_depth 2, inputs resident, median of 5 calls (CUDA
    events around the call on the context's stream)."""
    import torch
    from padenti_gb300 import _native as N

    sub = root_sample_set(a, m, False)
    tr = pg.TreeTrainer(cfg, device=device)
    tr.upload(sub)
    stream = torch.cuda.ExternalStream(N.lib().pd_ctx_stream(tr.h))
    times = []
    for r in range(7):
        tree = pg.Tree(cfg, 0, 2)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        tr.train(tree, sub, tp, 1, 2)
        e1.record(stream)
        e1.synchronize()
        if r >= 2:
            times.append(e0.elapsed_time(e1))
    ms = float(np.median(times))
    evals = sub.n_samples * tp.n_features
    return dict(value=evals / (ms / 1000), unit=UNIT, ms=ms, sample=f"root depth (histogram + split) of the "
                f"first {m} images ({sub.n_samples} samples x {tp.n_features} candidates x {tp.n_thresholds} "
                f"thresholds): the cpu_baseline's own sample; pd_train_tree with end_depth 2, median of 5 calls")


def profile_dram_per_image(kernel: str):
    """DRAM bytes per 640x480 image of a sampler or label kernel launch, from the committed
    ncu summary profiles/sampler_dram_640x480.json (None when absent)."""
    p = ROOT / "profiles" / "sampler_dram_640x480.json"
    try:
        d = json.loads(p.read_text())[kernel]
        return d["dram_bytes"] / d["images"]
    except Exception:
        return None


def sampler_bench(a, pg, N, px, lb):
    """UniformImageSampler / ClassWeightedImageSampler over the training images (2000 samples per
    image, 9 classes): device-resident (pd_sample_device, CUDA-event kernel times) and from host
    buffers (pd_sample, wall clock), with the oracle on the host cores beside them."""
    import torch

    n = min(a.sampler_images, len(px))
    h = pg._sampler_ctx(torch.cuda.current_device())
    dpx = torch.from_numpy(px[:n].view(np.int16)).cuda()
    dlb = torch.from_numpy(lb[:n]).cuda()
    peak, _ = measured_peaks()
    out = {}
    for name, sm in [("uniform", pg.UniformImageSampler(a.samples, 0)),
                     ("class_weighted", pg.ClassWeightedImageSampler(a.samples, 9, seed=0))]:
        stride = sm.stride
        dout = torch.zeros((n, stride), dtype=torch.int32, device="cuda")
        dcnt = torch.zeros(n, dtype=torch.int32, device="cuda")
        sc = sm._c(2)

        def dstep():
            N.check(N.lib().pd_sample_device(h, C.byref(sc), n, dpx.data_ptr(), dlb.data_ptr(), a.width, a.height,
                                             stride, dout.data_ptr(), dcnt.data_ptr()))

        torch.cuda.synchronize()
        for _ in range(3):
            dstep()
        reps, scan, draw = 5, [], []
        t0 = time.perf_counter()
        for _ in range(reps):
            dstep()
            st = sm.stats()
            scan.append(st["ms_scan"])
            draw.append(st["ms_draw"])
        wall = (time.perf_counter() - t0) * 1000 / reps
        ms_scan, ms_draw = float(np.median(scan)), float(np.median(draw))
        scan_bytes = n * a.width * a.height * 3  # image bytes (2 per pixel) + label bytes (1 per pixel)
        # host buffers in, samples out
        imgs, lbs = px[:n], lb[:n]  # the stacked-array form of sample_batch
        sm.sample_batch(imgs, lbs)
        t0 = time.perf_counter()
        e_reps = 2
        for _ in range(e_reps):
            sm.sample_batch(imgs, lbs)
        e2e_ms = (time.perf_counter() - t0) * 1000 / e_reps
        est = sm.stats()
        out[name] = dict(
            metric="sampled images/s", value=n / ((ms_scan + ms_draw) / 1000), unit="images/s", images=n,
            ms_kernels=ms_scan + ms_draw, ms_scan=ms_scan, ms_draw=ms_draw, ms_call=wall,
            roofline=dict(kernel="k_sample_scan", bound="hbm", achieved=scan_bytes / (ms_scan / 1000) / 1e9,
                          peak=peak, unit="GB/s", frac=scan_bytes / (ms_scan / 1000) / 1e9 / peak,
                          algorithmic_bytes=scan_bytes,
                          traffic=(lambda v: None if v is None else v * n)(profile_dram_per_image("k_sample_scan")),
                          traffic_note="DRAM bytes of a 300-image ncu capture, scaled by the images"),
            e2e=dict(value=n / (e2e_ms / 1000), unit="images/s", ms=e2e_ms, h2d_bytes=est["h2d_bytes"],
                     d2h_bytes=est["d2h_bytes"]))
        del dout, dcnt
    del dpx, dlb
    if not a.no_cpu:
        sys.path.insert(0, str(ROOT / "tests"))
        import oracle_bind as ob

        m = n
        for name, kind in [("uniform", 1), ("class_weighted", 2)]:
            t0 = time.perf_counter()
            ob.sample_batch(kind, px[:m], lb[:m], a.samples, 0, n_classes=9)
            dt = time.perf_counter() - t0
            out[name]["cpu_baseline"] = dict(value=m / dt, unit="images/s", cores=os.cpu_count() or 1, kind="port",
                                             sample=f"the first {m} images, oracle restatement of the reference "
                                                    f"sampler (table CRC-32, MT19937) on all host cores; {dt:.1f} s")
    return out


def loader_bench(a, pg, N):
    """The colour-to-class step of the label loader over 500 RGB label images of the training
    size: device-resident (CUDA-event kernel time), from host buffers (wall clock), and the
    oracle on all host cores."""
    import concurrent.futures as cf

    import torch

    n, H, W = 500, a.height, a.width
    colours = np.array([[255, 0, 0], [0, 0, 255], [0, 255, 0], [255, 255, 0], [0, 255, 255], [255, 0, 255],
                        [128, 0, 0], [0, 128, 0], [0, 0, 128]], np.uint8)
    _, lb, _ = pg.synth_depth(a.seed, n, W, H, first_image=3_000_000, parts=1, min_ellipses=2, max_ellipses=5,
                              samples_per_image=1)
    rgb = colours[np.maximum(lb.astype(np.int64) - 1, 0)]
    h = pg._sampler_ctx(torch.cuda.current_device())
    src = torch.from_numpy(rgb.reshape(-1)).cuda()
    dst = torch.empty(n * H * W, dtype=torch.uint8, device="cuda")
    cmap = np.ascontiguousarray(colours.reshape(-1))
    ms = C.c_float()

    def dstep():
        N.check(N.lib().pd_rgb_to_labels_device(h, n * H * W, src.data_ptr(), 3, cmap.ctypes.data, len(colours),
                                                dst.data_ptr(), C.byref(ms)))

    torch.cuda.synchronize()
    for _ in range(3):
        dstep()
    kms = []
    for _ in range(5):
        dstep()
        kms.append(ms.value)
    k_ms = float(np.median(kms))
    peak, _ = measured_peaks()
    nbytes = n * H * W * 4  # 3 bytes in, 1 out per pixel
    loader = pg.RGBLabelsLoader(colours)
    imgs = [rgb[i] for i in range(n)]
    loader.convert_batch(imgs)
    t0 = time.perf_counter()
    loader.convert_batch(imgs)
    e_ms = (time.perf_counter() - t0) * 1000
    out = dict(metric="label images Mpix/s", value=n * H * W / (k_ms / 1000) / 1e6, unit="Mpix/s", images=n,
               ms_kernel=k_ms,
               roofline=dict(kernel="k_rgb_to_labels", bound="hbm", achieved=nbytes / (k_ms / 1000) / 1e9, peak=peak,
                             unit="GB/s", frac=nbytes / (k_ms / 1000) / 1e9 / peak, algorithmic_bytes=nbytes,
                             traffic=(lambda v: None if v is None else v * n)(profile_dram_per_image("k_rgb_to_labels")),
                             traffic_note="DRAM bytes of a 200-image ncu capture, scaled by the images (writes "
                                          "still in L2 at the end of that short launch are not counted)"),
               e2e=dict(value=n * H * W / (e_ms / 1000) / 1e6, unit="Mpix/s", ms=e_ms))
    del src, dst
    if not a.no_cpu:
        sys.path.insert(0, str(ROOT / "tests"))
        import oracle_bind as ob

        m = n
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(os.cpu_count() or 1) as ex:
            list(ex.map(lambda i: ob.rgb_to_labels(rgb[i], colours), range(m)))
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = dict(value=m * H * W / dt / 1e6, unit="Mpix/s", cores=os.cpu_count() or 1, kind="port",
                                   sample=f"{m} images, the oracle restatement of _rgb2label (per-pixel colour "
                                          f"search) on all host cores; {dt:.1f} s")
    return out


def run_only(a):
    """One kernel family alone (the pixel samplers through pd_sample_device, or the colour-to-class
    mapping through pd_rgb_to_labels_device) on a.images synthetic depth-map images already in
    device memory, a.reps times: the command the sampler and label-image profiles run."""
    import torch

    import padenti_gb300 as pg
    from padenti_gb300 import _native as N

    px, lb, _ = pg.synth_depth(a.seed, a.images, a.width, a.height, parts=1, min_ellipses=2, max_ellipses=5,
                               samples_per_image=1)
    h = pg._sampler_ctx(0)
    if a.only == "labels":
        colours = np.array([[255, 0, 0], [0, 0, 255], [0, 255, 0], [255, 255, 0], [0, 255, 255], [255, 0, 255],
                            [128, 0, 0], [0, 128, 0], [0, 0, 128]], np.uint8)
        src = torch.from_numpy(colours[np.maximum(lb.astype(np.int64) - 1, 0)].reshape(-1)).cuda()
        dst = torch.empty(lb.size, dtype=torch.uint8, device="cuda")
        cmap = np.ascontiguousarray(colours.reshape(-1))
        ms = C.c_float()
        torch.cuda.synchronize()
        for _ in range(a.reps):
            N.check(N.lib().pd_rgb_to_labels_device(h, lb.size, src.data_ptr(), 3, cmap.ctypes.data, len(colours),
                                                    dst.data_ptr(), C.byref(ms)))
            print(json.dumps(dict(kernel="k_rgb_to_labels", ms=ms.value, gbs=lb.size * 4 / ms.value / 1e6)))
        return
    sm = (pg.UniformImageSampler(a.samples) if a.only == "sampler_uniform"
          else pg.ClassWeightedImageSampler(a.samples, 9))
    dpx = torch.from_numpy(px.view(np.int16)).cuda()
    dlb = torch.from_numpy(lb).cuda()
    out = torch.zeros((a.images, sm.stride), dtype=torch.int32, device="cuda")
    cnt = torch.zeros(a.images, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    for _ in range(a.reps):
        N.check(N.lib().pd_sample_device(h, C.byref(sm._c(2)), a.images, dpx.data_ptr(), dlb.data_ptr(), a.width,
                                         a.height, sm.stride, out.data_ptr(), cnt.data_ptr()))
        st = sm.stats()
        print(json.dumps(dict(sampler=a.only, ms_scan=st["ms_scan"], ms_draw=st["ms_draw"],
                              scan_gbs=(st["data_bytes"] + st["label_bytes"]) / st["ms_scan"] / 1e6)))


def rgb_bench(a, pg, device: int):
    """The RGB configuration: 1000 synthetic 320x240 RGB Voronoi images (21 classes, 2000 samples
    per image), channel-difference feature, F=1000 x T=30, 5 trees of depth 18 (min 20 samples
    per leaf), inputs resident; then the 5-tree forest predicts 200 held-out images.  Training
    evals/s over the forest (CUDA events on the context stream) and prediction Mpix/s, with the
    oracle's reference-cost root depth on the host cores beside the training rate."""
    import torch
    from padenti_gb300 import _native as N

    W, H, n = 320, 240, a.rgb_images
    px, lb, sm = pg.synth_rgb(a.seed, n, W, H, n_classes=21, samples_per_image=2000)
    cfg = pg.ForestConfig("channel_diff", 21)
    ts = pg.training_set(21, px, lb, sm)
    tp = pg.TreeTrainerParameters(1000, 30, [0, 0, -30, -30, -30, -30], [3, 3, 30, 30, 30, 30], -255, 255, 20)
    tr = pg.TreeTrainer(cfg, device=device)
    tr.upload(ts)
    stream = torch.cuda.ExternalStream(N.lib().pd_ctx_stream(tr.h))
    tr.train(pg.Tree(cfg, 100, 18), ts, tp)  # warm-up
    trees, evals = [], 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(5):
        tree = pg.Tree(cfg, k, 18)
        tr.train(tree, ts, tp)
        evals += tr.stats()["evals"]
        trees.append(tree)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    out = dict(workload="RGB Voronoi forest, 1000x320x240 uint8x3, 21 classes, 2000 samples/image, F=1000, "
                        "T=30, 5 trees of depth 18, min 20", metric=METRIC, value=evals / (ms / 1000), unit=UNIT,
               ms_forest=ms, trees=5, evals=evals)
    clf = pg.Classifier(cfg, device=device)
    for tr_ in trees:
        clf << tr_
    hx, _, _ = pg.synth_rgb(a.seed, 200, W, H, first_image=1_000_000, n_classes=21, samples_per_image=1)
    dimg = torch.from_numpy(hx.reshape(-1)).cuda()
    dout = torch.empty((200, 21, H, W), dtype=torch.float32, device="cuda")
    cstream = torch.cuda.ExternalStream(N.lib().pd_ctx_stream(clf.h))

    def pstep():
        N.check(N.lib().pd_predict_posterior_device(clf.h, 200, dimg.data_ptr(), W, H, None, dout.data_ptr()))

    pstep()
    N.check(N.lib().pd_ctx_sync(clf.h))
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(cstream)
    for _ in range(3):
        pstep()
    p1.record(cstream)
    N.check(N.lib().pd_ctx_sync(clf.h))
    pms = p0.elapsed_time(p1) / 3
    peak, _ = measured_peaks()
    bytes_alg = 200 * W * H * (3 + 21 * 4)
    out["predict"] = dict(metric="predict Mpix/s", value=200 * W * H / (pms / 1000) / 1e6, unit="Mpix/s",
                          images=200, ms_per_batch=pms,
                          roofline=dict(kernel="k_predict_posterior", bound="hbm",
                                        achieved=bytes_alg / (pms / 1000) / 1e9, peak=peak, unit="GB/s",
                                        frac=bytes_alg / (pms / 1000) / 1e9 / peak,
                                        algorithmic_bytes_per_launch=bytes_alg,
                                        note="87 algorithmic B/px: 3 RGB bytes in, 21 float posteriors out"))
    del dimg, dout
    if not a.no_cpu:
        sys.path.insert(0, str(ROOT / "tests"))
        import oracle_bind as ob

        m = 4
        sub = pg.TrainingSet(21, ts.images[:m])
        p = ob.params(cfg, tp)
        ds = ob.OracleSet(sub, cfg)
        node = np.zeros(ds.n_samples, np.int32)
        t0 = time.perf_counter()
        ob.hist(p, ds, 0, node, [0], reference_cost=True, threads=os.cpu_count() or 1)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = dict(value=ds.n_samples * tp.n_features / dt, unit=UNIT, cores=os.cpu_count() or 1,
                                   kind="port", sample=f"root histogram of the first {m} images ({ds.n_samples} "
                                   f"samples x 1000 candidates x 30 thresholds), reference-cost oracle; {dt:.1f} s")
    return out


def fit_only(a):
    """The proposal network's fit alone, on 18 000 seeded synthetic records of the depth
    configuration's shape (9 classes, FeatDim 4), --fit-steps steps of --fit-batch records,
    twice on one network (the second run replays the captured step): the workload of the
    network's kernel profiles."""
    import padenti_gb300 as pg

    cfg = pg.ForestConfig("depth_diff2", 9)
    tr = pg.TreeTrainer(cfg)
    tp = pg.TreeTrainerParameters(300, a.thresholds, [-60000] * 4, [60000] * 4, -500, 500, a.min_leaf)
    rng = np.random.default_rng(a.seed)
    n = 18000
    rec = np.zeros(n, pg.RECORD_DTYPE)
    rec["depth"] = rng.integers(1, 16, n)
    cc = rng.integers(0, 1000, (n, 9)).astype(np.uint32)
    rec["class_count"][:, :9] = cc
    rec["count"] = cc.sum(1)
    rec["feat"][:, :4] = rng.integers(-60000, 60000, (n, 4))
    rec["thr"] = rng.integers(-500, 500, n)
    net = pg.ProposalNetwork(tr, tp, seed=a.seed)
    r1 = net.fit(rec, steps=a.fit_steps, batch=a.fit_batch, lr=a.fit_lr)
    r2 = net.fit(rec, steps=a.fit_steps, batch=a.fit_batch, lr=a.fit_lr)
    return dict(steps=a.fit_steps, batch=a.fit_batch, ms_first=r1["ms"], ms=r2["ms"],
                us_per_step=1000 * r2["ms"] / a.fit_steps, last_loss=float(r2["loss"][-1]))


def mixed_bench(a, pg, device):
    """The mixed-size frontier-batched configuration: 5000 synthetic depth maps, a third each of
    160x120, 320x240 and 640x480 (made like the headline's: 2-5 bodies, 9 classes, 2000 samples
    per image), F=2000 x T=50, one tree of depth 20 (min 20 per leaf).  Every depth's frontier
    nodes, whatever their sizes, go through one histogram launch per slice (the whole frontier
    at these sizes), with launch shapes from the autotuner.  Beside it, the per-node-launch form
    (a histogram budget of one node per slice: candidates, histogram and split launched per
    frontier node, as the reference launches per node batch and image) on the first 12 levels,
    where both forms must give the same tree."""
    import tempfile

    import torch
    from padenti_gb300 import _native as N

    sizes = [(160, 120), (320, 240), (640, 480)]
    images = []
    for k, (w, h) in enumerate(sizes):
        cnt = 5000 // 3 + (1 if k < 5000 % 3 else 0)
        px, lb, sm = pg.synth_depth(a.seed, cnt, w, h, first_image=10_000_000 + 100_000 * k, parts=1,
                                    min_ellipses=2, max_ellipses=5, samples_per_image=a.samples, bg_permille=100)
        images += [pg.TrainingSetImage(px[i], lb[i], 9, sm[i]) for i in range(cnt)]
    cfg = pg.ForestConfig("depth_diff2", 9)
    ts = pg.TrainingSet(9, images)
    tp = pg.TreeTrainerParameters(a.features, a.thresholds, [-60000] * 4, [60000] * 4, -500, 500, a.min_leaf)
    tr = pg.TreeTrainer(cfg, device=device)
    tr.upload(ts)
    stream = torch.cuda.ExternalStream(N.lib().pd_ctx_stream(tr.h))
    cache = os.path.join(tempfile.mkdtemp(), "tune.txt")
    tune = tr.autotune(ts, tp, 20, cache=cache, max_trials=6) if a.autotune else None

    def timed_tree(trainer, tid, depth):
        tree = pg.Tree(cfg, tid, depth)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s = torch.cuda.ExternalStream(N.lib().pd_ctx_stream(trainer.h))
        e0.record(s)
        trainer.train(tree, ts, tp)
        e1.record(s)
        e1.synchronize()
        return tree, e0.elapsed_time(e1), trainer.stats()

    timed_tree(tr, 90, 20)  # warm-up
    tree, ms, st = timed_tree(tr, 0, 20)
    out = dict(workload="mixed-size depth maps: 5000 images (a third each of 160x120, 320x240, 640x480), 9 classes, "
                        "2000 samples/image, F=2000, T=50, depth 20, min 20",
               metric=METRIC, value=st["evals"] / (ms / 1000), unit=UNIT, ms_per_tree=ms, samples=ts.n_samples,
               nodes_trained=st["nodes_trained"], nodes_split=st["nodes_split"], hist_launches=st["hist_launches"],
               kernel_launches=st["kernel_launches"],
               launch_shape={k: tune[k] for k in ("chunk", "hist_spi", "fuse_max", "cand_order", "persist")}
               if tune else "fixed")
    # per-node launches against the batched form on the first 12 levels
    depth_cmp = 12
    b_tree, b_ms, b_st = timed_tree(tr, 1, depth_cmp)
    per_slot = 9 * tp.n_thresholds * tp.n_features * 4 + tp.n_thresholds * tp.n_features * 9 + 4 * tp.n_features * 5
    pn = pg.TreeTrainer(cfg, device=device, hist_budget=max(1 << 20, per_slot))
    pn.upload(ts)
    timed_tree(pn, 91, 4)  # warm-up
    p_tree, p_ms, p_st = timed_tree(pn, 1, depth_cmp)
    same = all(np.array_equal(getattr(b_tree, f), getattr(p_tree, f)) for f in
               ("left_child", "features", "thresholds")) and np.array_equal(
        b_tree.posteriors.view(np.uint32), p_tree.posteriors.view(np.uint32))
    out["per_node_launch"] = dict(depth=depth_cmp, batched_ms=b_ms, batched_hist_launches=b_st["hist_launches"],
                                  per_node_ms=p_ms, per_node_hist_launches=p_st["hist_launches"],
                                  per_node_kernel_launches=p_st["kernel_launches"],
                                  speedup=p_ms / b_ms, identical_trees=bool(same))
    del pn
    return out


def forest_accuracy(pg, cfg, trees, device, hx, hl):
    """Held-out per-pixel accuracy of a forest (argmax of the posterior against the labels):
    over all pixels, and over the object (non-background) pixels."""
    clf = pg.Classifier(cfg, device=device)
    for t in trees:
        clf << t
    ok = fg_ok = fg = tot = 0
    for i in range(len(hx)):
        post = clf.predict(hx[i])
        pred = np.argmax(post, axis=0) + 1
        lab = hl[i]
        ok += int((pred == lab).sum())
        tot += lab.size
        m = lab > 1
        fg_ok += int((pred[m] == lab[m]).sum())
        fg += int(m.sum())
    return ok / tot, fg_ok / max(fg, 1)


def learned_bench(a, pg, cfg, ts, tp, device):
    """Learned candidate proposals on the depth configuration (no reference counterpart):
    the plain 3-tree forest (2000 uniform candidates per node) against the learned one -- tree 0
    plain with records, the proposal network fitted to them on the GPU, trees 1 and 2 with 250
    proposed + 50 uniform candidates per node -- and, as the method without the network, trees 1
    and 2 with 300 uniform candidates.  Training time is the GPU time of each forest (trees and
    fit, CUDA events on the context stream); accuracy is per pixel over held-out images."""
    import torch
    from padenti_gb300 import _native as N

    tr = pg.TreeTrainer(cfg, device=device)
    tr.upload(ts)
    stream = torch.cuda.ExternalStream(N.lib().pd_ctx_stream(tr.h))

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        r = fn()
        e1.record(stream)
        e1.synchronize()
        return r, e0.elapsed_time(e1)

    import tempfile

    cache = os.path.join(tempfile.mkdtemp(), "tune.txt")
    tp300 = pg.TreeTrainerParameters(300, tp.n_thresholds, tp.feat_low_bounds, tp.feat_up_bounds, tp.thr_low_bound,
                                     tp.thr_up_bound, tp.per_leaf_samples_thr)
    # launch shapes tuned once per candidate count (pd_autotune), outside the timed regions
    tuned = {}
    if a.autotune:
        tuned["F2000"] = tr.autotune(ts, tp, a.depth, cache=cache, max_trials=10)
        tuned["F300"] = tr.autotune(ts, tp300, a.depth, cache=cache, max_trials=10)
        tr.autotune(ts, tp, a.depth, cache=cache)
    tr.train(pg.Tree(cfg, 90, a.depth), ts, tp)  # warm-up
    plain, ms_plain = [], 0.0
    for k in range(3):
        t = pg.Tree(cfg, k, a.depth)
        if k == 0:
            tr.set_tuning("records", 1)
        _, ms = timed(lambda: tr.train(t, ts, tp))
        if k == 0:
            tr.set_tuning("records", 0)
            rec = tr.records()
            ms_tree0 = ms
        plain.append(t)
        ms_plain += ms
    if a.autotune:
        tr.autotune(ts, tp300, a.depth, cache=cache)  # the F=300 setting, from the cache
    net = pg.ProposalNetwork(tr, tp300, seed=a.seed)
    fit = net.fit(rec[:1], steps=1, batch=a.fit_batch, lr=a.fit_lr)  # warm-up (graph capture)
    net = pg.ProposalNetwork(tr, tp300, seed=a.seed)
    fit, ms_fit = timed(lambda: net.fit(rec, steps=a.fit_steps, batch=a.fit_batch, lr=a.fit_lr))
    learned, ms_learned = [plain[0]], ms_tree0 + ms_fit
    for k in (1, 2):
        t = pg.Tree(cfg, k, a.depth)
        _, ms = timed(lambda: tr.train_proposed(t, ts, tp300, net, 250))
        learned.append(t)
        ms_learned += ms
    uni, ms_uni = [plain[0]], ms_tree0
    for k in (1, 2):
        t = pg.Tree(cfg, k, a.depth)
        _, ms = timed(lambda: tr.train(t, ts, tp300))
        uni.append(t)
        ms_uni += ms
    # what the network gains at a small budget: one tree, 25 proposed + 5 uniform against 30 uniform
    tp30 = pg.TreeTrainerParameters(30, tp.n_thresholds, tp.feat_low_bounds, tp.feat_up_bounds, tp.thr_low_bound,
                                    tp.thr_up_bound, tp.per_leaf_samples_thr)
    net30 = pg.ProposalNetwork(tr, tp30, seed=a.seed)
    net30.params = net.params
    small_l, small_u = pg.Tree(cfg, 1, a.depth), pg.Tree(cfg, 1, a.depth)
    tr.train_proposed(small_l, ts, tp30, net30, 25)
    tr.train(small_u, ts, tp30)
    hx, hl, _ = pg.synth_depth(a.seed, 100, a.width, a.height, first_image=5_000_000, parts=1, min_ellipses=2,
                               max_ellipses=5, samples_per_image=1)
    acc = {name: forest_accuracy(pg, cfg, f, device, hx, hl) for name, f in
           (("plain", plain), ("learned", learned), ("uniform300", uni), ("tree30_learned", [small_l]),
            ("tree30_uniform", [small_u]))}
    return dict(
        metric="learned vs plain time at same accuracy", unit="ratio of GPU training times",
        value=ms_learned / ms_plain, higher_is_better=False,
        plain=dict(ms=ms_plain, accuracy=acc["plain"][0], object_accuracy=acc["plain"][1], candidates=tp.n_features),
        learned=dict(ms=ms_learned, ms_tree0=ms_tree0, ms_fit=ms_fit, accuracy=acc["learned"][0],
                     object_accuracy=acc["learned"][1], records=int(len(rec)), proposed=250, uniform=50,
                     fit_steps=a.fit_steps, fit_batch=a.fit_batch, first_loss=float(fit["loss"][0]),
                     last_loss=float(fit["loss"][-10:].mean())),
        uniform300=dict(ms=ms_uni, accuracy=acc["uniform300"][0], object_accuracy=acc["uniform300"][1]),
        single_tree_30_candidates=dict(learned=dict(accuracy=acc["tree30_learned"][0],
                                                    object_accuracy=acc["tree30_learned"][1]),
                                       uniform=dict(accuracy=acc["tree30_uniform"][0],
                                                    object_accuracy=acc["tree30_uniform"][1]),
                                       note="tree 1 alone, 25 proposed + 5 uniform against 30 uniform candidates"),
        accuracy_gap_pt=100 * (acc["plain"][0] - acc["learned"][0]),
        network_gain_pt=100 * (acc["learned"][0] - acc["uniform300"][0]),
        held_out="100 synthetic 640x480 images of the same generator (not trained on)",
        launch_shapes={k: {q: v[q] for q in ("chunk", "hist_spi", "fuse_max", "cand_order", "persist", "ms_start",
                                            "ms_best", "trials")} for k, v in tuned.items()},
        note="tree 0 is the plain tree in both forests; the learned forest's time counts it, the fit and "
             "trees 1-2")


def cpu_predict(a, cfg, trees, hx):
    """The oracle's forest posterior (cl_classifier_impl.hpp:356-557 restated) on all host cores
    over the first held-out images, about 10 s of work: Mpix/s."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_bind as ob

    import padenti_gb300 as pg

    tp = pg.TreeTrainerParameters(a.features, a.thresholds, [-60000] * 4, [60000] * 4, -500, 500, a.min_leaf)
    p = ob.params(cfg, tp)
    tt = [(t.depth, t.left_child, np.asarray(t.features, np.int32), np.asarray(t.thresholds, np.int32), t.posteriors)
          for t in trees]
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ob.predict_posterior(p, hx[0], None, tt, threads=threads)
    one = time.perf_counter() - t0
    m = int(max(1, min(len(hx), round(10.0 / max(one, 1e-3)))))
    t0 = time.perf_counter()
    for i in range(m):
        ob.predict_posterior(p, hx[i], None, tt, threads=threads)
    dt = time.perf_counter() - t0
    px = m * hx.shape[1] * hx.shape[2]
    return dict(value=px / dt / 1e6, unit="Mpix/s", cores=threads, kind="port",
                sample=f"the first {m} held-out images through the {len(tt)}-tree forest, oracle restatement of "
                       f"the reference's per-tree traversal and posterior sum on all host cores; {dt:.1f} s")


def run_reference(a):
    """The reference algorithm on the host cores (the oracle port in reference-cost mode), on a
    bounded sample of the workload: the root depth of the first m images.  Its inputs come from
    the oracle's restatement of the synthetic generator, so the CUDA library is never loaded."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import padenti_gb300 as pg

    cfg = pg.ForestConfig("depth_diff2", 9)
    tp = pg.TreeTrainerParameters(a.features, a.thresholds, [-60000] * 4, [60000] * 4, -500, 500, a.min_leaf)
    base, m = cpu_sample(a, cfg, tp, a.cpu_seconds, lib_free=True)
    sub = root_sample_set(a, m, True)
    times, evals, n = [], 0, 0
    for _ in range(a.steps):
        rate, dt, n = cpu_root(a, cfg, tp, sub, base["cores"])
        times.append(dt)
        evals += n * tp.n_features
    value = evals / sum(times)
    base["value"] = value
    base["sample"] = root_sample_text(m, n, tp, sum(times) / len(times))
    line = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=a.gpus, steps=a.steps, warmup=a.warmup,
                ms_per_step=1000 * sum(times) / len(times), higher_is_better=True, scaling="weak", vs_baseline=None,
                dtype="int32", data="synthetic (the oracle's restatement of the seeded generator)", impl="reference",
                config=dict(workload=WORKLOAD, sample=base["sample"], sample_images=m), cpu_baseline=base,
                e2e=dict(value=value, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)


def run_ours(a):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    def allmax(x):
        if world > 1:
            import torch.distributed as dist

            t = torch.tensor([x], dtype=torch.float64, device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            return float(t.item())
        return x

    def allsum(x):
        if world > 1:
            import torch.distributed as dist

            t = torch.tensor([x], dtype=torch.float64, device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.SUM)
            return float(t.item())
        return x

    pg, cfg, ts, tp, (px, lb, sm) = make_workload(a, rank)
    from padenti_gb300 import _native as N

    tr = pg.TreeTrainer(cfg, device=local)
    if a.chunk:
        tr.set_tuning("chunk", a.chunk)
    if a.spi:
        tr.set_tuning("hist_spi", a.spi)
    if a.fuse_max is not None:
        tr.set_tuning("fuse_max", a.fuse_max)
    if a.cand_order is not None:
        tr.set_tuning("cand_order", a.cand_order)
    tr.upload(ts)
    stream = torch.cuda.ExternalStream(N.lib().pd_ctx_stream(tr.h))
    tune = None
    if a.autotune and not (a.chunk or a.spi or a.fuse_max is not None or a.cand_order is not None):
        # launch shapes from the autotuner (whole trees timed on this training set; results never change)
        tune = tr.autotune(ts, tp, a.depth, max_trials=10)

    def tree_step(tid):
        tree = pg.Tree(cfg, tid, a.depth)
        tr.train(tree, ts, tp)
        return tree, tr.stats()

    for w in range(a.warmup):
        tree_step(10_000 + rank * 1000 + w)

    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    evals = hist_ms = hist_bytes = launches = hist_launches = 0
    phases = dict(ms_candidates=0.0, ms_hist=0.0, ms_split=0.0, ms_reassign=0.0, ms_total=0.0, split_rechecked=0,
                  nodes_split=0)
    trees = []
    with Clocks(local) as clk:
        e0.record(stream)
        for s in range(a.steps):
            tree, st = tree_step(rank * 1000 + s)
            trees.append(tree)
            evals += st["evals"]
            hist_ms += st["ms_hist"]
            hist_bytes += st["hist_bytes"]
            launches += st["kernel_launches"]
            hist_launches += st["hist_launches"]
            for k in phases:
                phases[k] += st[k]
        e1.record(stream)
        barrier()
    ms = allmax(e0.elapsed_time(e1))
    total_evals = allsum(evals)
    value = total_evals / (ms / 1000.0)

    # ---- end to end through the public API with host buffers ----
    e2e_steps = a.e2e_steps if a.e2e_steps is not None else a.steps
    flat = ts.flat()
    pinned = {}
    for k, v in flat.items():
        t = torch.empty(v.nbytes, dtype=torch.uint8, pin_memory=True)
        t.numpy()[:] = v.view(np.uint8).reshape(-1)
        pinned[k] = t
    pinned_flat = {k: pinned[k].numpy().view(flat[k].dtype) for k in pinned}
    desc = pg.TrainingSet.desc(pinned_flat)
    h0 = C.c_uint64()
    d0 = C.c_uint64()
    N.check(N.lib().pd_ctx_transfer_bytes(tr.h, C.byref(h0), C.byref(d0)))
    barrier()
    t0 = time.perf_counter()
    e2e_evals = 0
    upload_s = 0.0
    up_samples = up_device = 0.0
    for s in range(e2e_steps):
        tu = time.perf_counter()
        N.check(N.lib().pd_dataset_upload(tr.h, C.byref(desc)))
        upload_s += time.perf_counter() - tu
        us = N.UploadStats()
        N.check(N.lib().pd_dataset_upload_stats(tr.h, C.byref(us)))
        up_samples += us.ms_samples
        up_device += us.ms_device
        tr._uploaded = None
        tree = pg.Tree(cfg, 500 + rank * 1000 + s, a.depth)
        prior = np.ascontiguousarray(ts.priors, np.float32)
        N.check(N.lib().pd_train_tree(tr.h, C.byref(tp.c()), tree.id, 1, a.depth, prior.ctypes.data,
                                      tree.left_child.ctypes.data, tree.features.ctypes.data,
                                      tree.thresholds.ctypes.data, tree.posteriors.ctypes.data))
        e2e_evals += tr.stats()["evals"]
    barrier()
    e2e_s = allmax(time.perf_counter() - t0)
    h1 = C.c_uint64()
    d1 = C.c_uint64()
    N.check(N.lib().pd_ctx_transfer_bytes(tr.h, C.byref(h1), C.byref(d1)))
    e2e = dict(value=allsum(e2e_evals) / e2e_s, unit=UNIT,
               h2d_bytes_per_step=int((h1.value - h0.value) / max(1, e2e_steps)),
               d2h_bytes_per_step=int((d1.value - d0.value) / max(1, e2e_steps)),
               upload_ms_per_step=1000 * upload_s / max(1, e2e_steps),
               upload_host_samples_ms=up_samples / max(1, e2e_steps),
               upload_device_ms=up_device / max(1, e2e_steps),
               ms_per_step=1000 * e2e_s / max(1, e2e_steps),
               note="per step: pd_dataset_upload of the whole training set from pinned host memory + "
                    "pd_train_tree with the tree arrays in host memory; wall clock")

    # ---- prediction of held-out images with the forest of the timed trees ----
    pred = None
    if a.predict_images > 0:
        clf = pg.Classifier(cfg, device=local)
        for t in trees:
            clf << t
        n_p = a.predict_images
        hx, _, _ = pg.synth_depth(a.seed, n_p, a.width, a.height, first_image=1_000_000, parts=1, min_ellipses=2,
                                  max_ellipses=5, samples_per_image=1)
        dimg = torch.from_numpy(hx.view(np.int16)).cuda()
        dout = torch.empty((n_p, 9, a.height, a.width), dtype=torch.float32, device="cuda")
        cstream = torch.cuda.ExternalStream(N.lib().pd_ctx_stream(clf.h))

        def pstep():
            N.check(N.lib().pd_predict_posterior_device(clf.h, n_p, dimg.data_ptr(), a.width, a.height, None,
                                                        dout.data_ptr()))

        torch.cuda.synchronize()
        pstep()
        N.check(N.lib().pd_ctx_sync(clf.h))
        pe0 = torch.cuda.Event(enable_timing=True)
        pe1 = torch.cuda.Event(enable_timing=True)
        reps = 3
        pe0.record(cstream)
        for _ in range(reps):
            pstep()
        pe1.record(cstream)
        N.check(N.lib().pd_ctx_sync(clf.h))
        pms = pe0.elapsed_time(pe1) / reps
        px_total = n_p * a.width * a.height
        bytes_alg = px_total * (2 + 9 * 4)
        peak_p, peak_kind_p = measured_peaks()
        pred = dict(metric="predict Mpix/s", value=px_total / (pms / 1000) / 1e6, unit="Mpix/s",
                    images=n_p, trees=len(trees), ms_per_batch=pms,
                    roofline=dict(kernel="k_predict_posterior", bound="hbm",
                                  achieved=bytes_alg / (pms / 1000) / 1e9, peak=peak_p, unit="GB/s",
                                  frac=bytes_alg / (pms / 1000) / 1e9 / peak_p,
                                  algorithmic_bytes_per_launch=bytes_alg,
                                  traffic=None, peak_source=f"{peak_kind_p} (hbm_gbs)",
                                  note="38 algorithmic B/px: the 2-byte depth read once and 9 float posteriors "
                                       "written once; the forest's nodes stay in L2; the kernel is bound by "
                                       "instruction issue (tree walks), not HBM"),
                    note="500 held-out 640x480 images in one launch, forest of the timed trees, 38 algorithmic B/px")
        if not a.no_cpu:
            pred["cpu_baseline"] = cpu_predict(a, cfg, trees, hx)
        del dimg, dout
        # mixed-size serving batch: 256 images, a third each of 160x120,
        # 320x240 and 640x480, host buffers in and out, one graph-replayed launch per batch
        sizes = [(160, 120), (320, 240), (640, 480)]
        mims = []
        for k, (w, h) in enumerate(sizes):
            cnt = 256 // 3 + (1 if k < 256 % 3 else 0)
            mx, _, _ = pg.synth_depth(a.seed, cnt, w, h, first_image=2_000_000 + 1000 * k, parts=1,
                                      min_ellipses=2, max_ellipses=5, samples_per_image=1)
            mims += [np.ascontiguousarray(mx[i]) for i in range(cnt)]
        mouts = [np.empty((9, im.shape[0], im.shape[1]), np.float32) for im in mims]
        for o in mouts:
            o.fill(0)  # touch the pages once, outside the timed region
        nb = len(mims)
        PV = C.c_void_p * nb
        ip, op = PV(*[im.ctypes.data for im in mims]), PV(*[o.ctypes.data for o in mouts])
        mw = (C.c_uint32 * nb)(*[im.shape[1] for im in mims])
        mh = (C.c_uint32 * nb)(*[im.shape[0] for im in mims])

        def bstep():
            N.check(N.lib().pd_predict_posterior_batch(clf.h, nb, ip, mw, mh, None, op))

        bstep()
        bstep()
        t0 = time.perf_counter()
        for _ in range(reps):
            bstep()
        bms = (time.perf_counter() - t0) * 1000 / reps
        bpx = sum(im.size for im in mims)
        pred["mixed_batch"] = dict(value=bpx / (bms / 1000) / 1e6, unit="Mpix/s", images=nb, ms_per_batch=bms,
                                   note="256 images of 160x120/320x240/640x480 (a third each) through "
                                        "pd_predict_posterior_batch from host buffers: per-image copies in, one "
                                        "CUDA-graph replay of the batch kernel, posteriors out; wall clock")

    learned = learned_bench(a, pg, cfg, ts, tp, local) if a.learned and world == 1 else None
    samp = sampler_bench(a, pg, N, px, lb) if a.sampler_images > 0 else None
    rgb = rgb_bench(a, pg, local) if a.rgb_images > 0 else None
    mixed = mixed_bench(a, pg, local) if a.mixed and world == 1 else None
    if samp is not None:
        samp["label_images"] = loader_bench(a, pg, N)

    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    hist_s = hist_ms / 1000.0
    achieved = (hist_bytes / max(1, hist_launches)) / (hist_s / max(1, hist_launches)) / 1e9 if hist_s > 0 else 0.0
    tr_prof = profile_traffic()
    roof = dict(bound="hbm", achieved=achieved, peak=peak, unit="GB/s", frac=achieved / peak,
                traffic=(tr_prof or {}).get("dram_bytes_per_launch"),
                kernel="k_hist", peak_source=f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs, burst)" if peak_kind == "measured" else "fallback 6800 GB/s",
                algorithmic_bytes_per_launch=hist_bytes / max(1, hist_launches),
                launch_ms=hist_ms / max(1, hist_launches),
                evals_per_s_in_kernel=evals / hist_s if hist_s > 0 else None,
                note="the histogram kernel is bound by instruction issue and the L1 data pipe (probe gathers, "
                     "threshold search), not by HBM")
    # the histogram kernel's own bound: instruction issue (lane slots of warp instructions)
    issue_roof = None
    ip = ROOT / "profiles" / "k_hist_issue_300x640x480.json"
    clk_sum = clk.summary()
    if ip.exists() and hist_s > 0 and clk_sum.get("sm_mhz"):
        ipe = json.loads(ip.read_text())["thread_instr_per_eval"]
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        ach = evals / hist_s * ipe
        pk = sms * 4 * 32 * clk_sum["sm_mhz"] * 1e6
        issue_roof = dict(bound="issue", kernel="k_hist", achieved=ach, peak=pk, unit="thread-instr/s", frac=ach / pk,
                          thread_instr_per_eval=ipe,
                          note="achieved = live evaluations/s x instruction slots per evaluation from "
                               "profiles/k_hist_issue_300x640x480.json; peak = SMs x 4 schedulers x 32 lanes x the "
                               "median SM clock sampled during the timed region")
    atomic_roof = None
    if hist_s > 0:
        rate = C.c_double()
        ctas = C.c_int32()
        if N.lib().pd_measure_smem_atomics(local, C.byref(rate), C.byref(ctas)) == 0 and rate.value > 0:
            ach = evals / hist_s
            atomic_roof = dict(bound="smem_atomic", kernel="k_hist", achieved=ach, peak=rate.value, unit="adds/s",
                               frac=ach / rate.value, adds_per_eval=1, peak_ctas_per_sm=ctas.value,
                               note="one conflict-free shared-memory atomic add per evaluation; peak = "
                                    "pd_measure_smem_atomics (the same add in the same [class][rank][lane] "
                                    "layout, 8 in flight per thread, best of 2/4/8 CTAs per SM), CUDA events")
    base = same = None
    if not a.no_cpu:
        base, m = cpu_sample(a, cfg, tp, a.cpu_seconds)
        same = gpu_root_sample(a, pg, cfg, tp, m, local)
    line = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=a.steps, warmup=a.warmup,
                ms_per_step=ms / a.steps, higher_is_better=True, scaling="weak", vs_baseline=None, dtype="int32",
                data="synthetic (seeded depth maps generated on the host; see config)",
                config=dict(workload=WORKLOAD, images=a.images, width=a.width, height=a.height,
                            samples_per_image=a.samples, features=a.features, thresholds=a.thresholds,
                            depth=a.depth, min_leaf=a.min_leaf, trees_per_step=1,
                            chunk=(tune or {}).get("chunk", a.chunk or 16384),
                            fuse_max=(tune or {}).get("fuse_max", 4096 if a.fuse_max is None else a.fuse_max),
                            hist_spi=(tune or {}).get("hist_spi", a.spi or 8),
                            cand_order=(tune or {}).get("cand_order", 1 if a.cand_order is None else a.cand_order),
                            persist=(tune or {}).get("persist", 0),
                            launch_shape="pd_autotune (%d settings timed)" % tune["trials"] if tune else "fixed",
                            parallelism=f"replicas x{world} (one tree per GPU per step)",
                            l2="inputs 1.23 GB > L2 (129 MB), no flush"),
                roofline=roof, roofline_issue=issue_roof, roofline_atomic=atomic_roof, cpu_baseline=base,
                gpu_on_cpu_sample=same, rgb_config=rgb, learned_proposals=learned, mixed_sizes=mixed, e2e=e2e, gpu_launches=launches, clocks=clk.summary(),
                predict=pred, sampler=samp, phases_per_step={k: v / a.steps for k, v in phases.items()}, impl="ours")
    print(json.dumps(line), flush=True)


def main():
    a = args_()
    if a.only == "fit":
        print(json.dumps(fit_only(a)), flush=True)
    elif a.only == "mixed":
        import padenti_gb300 as pg

        print(json.dumps(mixed_bench(a, pg, 0)), flush=True)
    elif a.only == "learned":
        import padenti_gb300 as pg

        pg_, cfg, ts, tp, _ = make_workload(a, 0)
        print(json.dumps(learned_bench(a, pg, cfg, ts, tp, 0)), flush=True)
    elif a.only:
        run_only(a)
    elif a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
