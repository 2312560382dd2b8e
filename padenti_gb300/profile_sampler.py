"""Runs the pixel samplers (or the label-colour mapping) on a batch of synthetic
images already in device memory (pd_sample_device, pd_rgb_to_labels_device),
for profiling those kernels:

    python -m padenti_gb300.profile_sampler --images 300 --kind uniform
    python -m padenti_gb300.profile_sampler --images 300 --kind labels
"""
from __future__ import annotations

import argparse
import ctypes as C

import numpy as np


def main() -> None:
    import torch

    import padenti_gb300 as pg
    from padenti_gb300 import _native as N

    a = argparse.ArgumentParser()
    a.add_argument("--images", type=int, default=300)
    a.add_argument("--width", type=int, default=640)
    a.add_argument("--height", type=int, default=480)
    a.add_argument("--samples", type=int, default=2000)
    a.add_argument("--kind", choices=["uniform", "class_weighted", "labels"], default="uniform")
    a.add_argument("--reps", type=int, default=3)
    a = a.parse_args()
    px, lb, _ = pg.synth_depth(0, a.images, a.width, a.height, parts=1, min_ellipses=2, max_ellipses=5,
                               samples_per_image=1)
    if a.kind == "labels":
        colours = np.array([[255, 0, 0], [0, 0, 255], [0, 255, 0], [255, 255, 0], [0, 255, 255], [255, 0, 255],
                            [128, 0, 0], [0, 128, 0], [0, 0, 128]], np.uint8)
        src = torch.from_numpy(colours[np.maximum(lb.astype(np.int64) - 1, 0)].reshape(-1)).cuda()
        dst = torch.empty(lb.size, dtype=torch.uint8, device="cuda")
        cmap = np.ascontiguousarray(colours.reshape(-1))
        ms = C.c_float()
        torch.cuda.synchronize()
        for _ in range(a.reps):
            N.check(N.lib().pd_rgb_to_labels_device(pg._sampler_ctx(0), lb.size, src.data_ptr(), 3, cmap.ctypes.data,
                                                    len(colours), dst.data_ptr(), C.byref(ms)))
            print(f"labels {ms.value:.3f} ms  {lb.size * 4 / ms.value / 1e6:.0f} GB/s")
        return
    sm = pg.UniformImageSampler(a.samples) if a.kind == "uniform" else pg.ClassWeightedImageSampler(a.samples, 9)
    h = pg._sampler_ctx(0)
    dpx = torch.from_numpy(px.view(np.int16)).cuda()
    dlb = torch.from_numpy(lb).cuda()
    out = torch.zeros((a.images, sm.stride), dtype=torch.int32, device="cuda")
    cnt = torch.zeros(a.images, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    for _ in range(a.reps):
        N.check(N.lib().pd_sample_device(h, C.byref(sm._c(2)), a.images, dpx.data_ptr(), dlb.data_ptr(), a.width,
                                         a.height, sm.stride, out.data_ptr(), cnt.data_ptr()))
        st = sm.stats()
        print(f"scan {st['ms_scan']:.3f} ms  draw {st['ms_draw']:.3f} ms  "
              f"scan {(st['data_bytes'] + st['label_bytes']) / st['ms_scan'] / 1e6:.0f} GB/s")


if __name__ == "__main__":
    main()
