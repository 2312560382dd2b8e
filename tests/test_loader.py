"""Label images and the directory constructor of TrainingSet: the colour-to-class step of
CVRGBLabelsLoader (_rgb2label) on the GPU against the oracle, binary PGM/PPM files standing in
for the OpenCV loaders, and TrainingSet(dir, …, loaders, sampler)."""
import ctypes as C

import numpy as np
import pytest

import oracle_bind as ob
import padenti_gb300 as pg
from padenti_gb300 import _native as N


def _numpy_rgb2label(img, colours):
    """An independent restatement: the first matching colour wins."""
    out = np.zeros(img.shape[:2], np.uint8)
    done = np.zeros(img.shape[:2], bool)
    for k, c in enumerate(np.asarray(colours, np.uint8)):
        m = (img[..., 0] == c[0]) & (img[..., 1] == c[1]) & (img[..., 2] == c[2]) & ~done
        out[m] = k + 1
        done |= m
    return out


def _label_image(rng, h, w, colours, channels=3, unknown=0.1):
    idx = rng.integers(0, len(colours), (h, w))
    img = np.asarray(colours, np.uint8)[idx]
    off = rng.random((h, w)) < unknown
    img[off] = rng.integers(0, 256, (int(off.sum()), 3), dtype=np.uint8)
    if channels == 4:
        img = np.concatenate([img, rng.integers(0, 256, (h, w, 1), dtype=np.uint8)], axis=2)
    return img


COLOURS = [(255, 0, 0), (0, 0, 255), (0, 255, 0), (255, 0, 0), (10, 20, 30)]  # class 3 repeats class 0


def test_oracle_rgb2label_matches_numpy_restatement():
    rng = np.random.default_rng(0)
    for ch in (3, 4):
        img = _label_image(rng, 37, 53, COLOURS, ch)
        got = ob.rgb_to_labels(img, COLOURS)
        assert np.array_equal(got, _numpy_rgb2label(img, COLOURS))
        assert set(np.unique(got)) <= {0, 1, 2, 3, 5}  # the repeated colour keeps its first class


def test_pnm_round_trip_and_loader_types(tmp_path):
    a = (np.arange(6 * 11, dtype=np.uint16) * 997).reshape(6, 11)
    pg.write_pnm(tmp_path / "d.pgm", a)
    raw = (tmp_path / "d.pgm").read_bytes()
    (tmp_path / "c.pgm").write_bytes(raw.replace(b"P5\n", b"P5\n# a comment\n", 1))
    assert np.array_equal(pg.read_pnm(tmp_path / "c.pgm"), a)
    assert np.array_equal(pg.PNMImageLoader(np.uint16, 1).load(tmp_path / "d.pgm"), a)
    with pytest.raises(ValueError, match="different from the expected"):
        pg.PNMImageLoader(np.uint8, 3).load(tmp_path / "d.pgm")
    rgb = np.random.default_rng(1).integers(0, 256, (4, 5, 3), dtype=np.uint8)
    pg.write_pnm(tmp_path / "l.ppm", rgb)
    assert np.array_equal(pg.read_pnm(tmp_path / "l.ppm"), rgb)


def test_rgb_to_labels_rejects_bad_maps():
    with pytest.raises(ValueError, match="1 to 255"):
        pg.RGBLabelsLoader(np.zeros((0, 3), np.uint8))
    with pytest.raises(ValueError):
        pg.RGBLabelsLoader(COLOURS).convert_batch([np.zeros((4, 4, 2), np.uint8)])


@pytest.mark.gpu
def test_gpu_rgb_to_labels_matches_the_oracle():
    rng = np.random.default_rng(2)
    many = [tuple(int(x) for x in rng.integers(0, 256, 3)) for _ in range(250)] + [(7, 7, 7)] * 5
    for colours in (COLOURS, many):
        for ch in (3, 4):
            imgs = [_label_image(rng, h, w, colours, ch) for (h, w) in [(37, 53), (1, 1), (120, 160), (3, 17)]]
            got = pg.RGBLabelsLoader(colours).convert_batch(imgs)
            for im, g in zip(imgs, got):
                assert np.array_equal(g, ob.rgb_to_labels(im, colours))


@pytest.mark.gpu
def test_gpu_rgb_to_labels_device_entry():
    import torch

    rng = np.random.default_rng(3)
    img = _label_image(rng, 480, 640, COLOURS, 3)
    src = torch.from_numpy(img.reshape(-1)).cuda()
    dst = torch.zeros(480 * 640, dtype=torch.uint8, device="cuda")
    cmap = np.ascontiguousarray(COLOURS, np.uint8).reshape(-1)
    ms = C.c_float()
    torch.cuda.synchronize()
    N.check(N.lib().pd_rgb_to_labels_device(pg._sampler_ctx(0), 480 * 640, src.data_ptr(), 3, cmap.ctypes.data,
                                            len(COLOURS), dst.data_ptr(), C.byref(ms)))
    assert np.array_equal(dst.cpu().numpy().reshape(480, 640), ob.rgb_to_labels(img, COLOURS))
    assert ms.value > 0


@pytest.mark.gpu
def test_training_set_from_a_directory(tmp_path):
    """load_training_set = TrainingSet(dir, "_depth.pgm", "_labels.ppm", K, loaders, sampler):
    labels and samples are those of the oracle; a pair of different sizes is skipped."""
    colours = [(255, 0, 0), (0, 0, 255), (0, 255, 0)]
    px, lb, _ = pg.synth_depth(9, 5, 96, 72, parts=0, samples_per_image=4)
    for i in range(5):
        pg.write_pnm(tmp_path / f"img{i}_depth.pgm", px[i])
        rgb = np.zeros(lb[i].shape + (3,), np.uint8)
        for k in range(3):
            rgb[lb[i] == k + 1] = colours[k]
        if i == 3:
            rgb = rgb[:-1]  # a labels image of another size: skipped
        pg.write_pnm(tmp_path / f"img{i}_labels.ppm", rgb)
    (tmp_path / "img9_depth.pgm").write_bytes((tmp_path / "img0_depth.pgm").read_bytes())  # no labels: ignored
    sampler = pg.ClassWeightedImageSampler(300, 3, seed=11)
    ts = pg.load_training_set(tmp_path, "_depth.pgm", "_labels.ppm", 3, pg.PNMImageLoader(np.uint16, 1),
                              pg.RGBLabelsLoader(colours), sampler)
    assert len(ts.images) == 4
    for im, i in zip(ts.images, [0, 1, 2, 4]):
        assert np.array_equal(im.data, px[i]) and np.array_equal(im.labels, lb[i])
        assert np.array_equal(im.samples, ob.sample_class_weighted(px[i], lb[i], 300, 3, None, 11))


def _write_set(tmp_path):
    colours = [(255, 0, 0), (0, 0, 255), (0, 255, 0)]
    px, lb, _ = pg.synth_depth(9, 5, 96, 72, parts=0, samples_per_image=4)
    for i in range(5):
        pg.write_pnm(tmp_path / f"img{i}_depth.pgm", px[i])
        rgb = np.zeros(lb[i].shape + (3,), np.uint8)
        for k in range(3):
            rgb[lb[i] == k + 1] = colours[k]
        if i == 3:
            rgb = rgb[:-1]
        pg.write_pnm(tmp_path / f"img{i}_labels.ppm", rgb)
    return px, lb


def test_cpp_loader_facade_compiles(tmp_path):
    from test_cpp_facade import CPP, _compile

    _compile(CPP / "facade_load.cpp", tmp_path / "facade_load", link=True)


@pytest.mark.gpu
def test_cpp_loader_facade_matches_python(tmp_path):
    import subprocess

    from test_cpp_facade import CPP, _compile

    exe = tmp_path / "facade_load"
    _compile(CPP / "facade_load.cpp", exe, link=True)
    d = tmp_path / "set"
    d.mkdir()
    px, lb = _write_set(d)
    r = subprocess.run([str(exe), str(d), str(tmp_path / "out.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    got = np.fromfile(tmp_path / "out.bin", np.uint32)
    pos = 0
    for i in [0, 1, 2, 4]:
        w, h = int(got[pos]), int(got[pos + 1])
        assert (w, h) == (96, 72)
        assert np.array_equal(got[pos + 2:pos + 2 + w * h].astype(np.uint8).reshape(h, w), lb[i])
        pos += 2 + w * h
        n = int(got[pos])
        assert np.array_equal(got[pos + 1:pos + 1 + n], ob.sample_class_weighted(px[i], lb[i], 300, 3, None, 11))
        pos += 1 + n
    assert pos == got.size


def _roi_by_flood_fill(mask):
    """An independent restatement: 8-connected components by breadth-first search, the
    one-pixel border counting as zero, the largest bounding rectangle, first in raster order."""
    from collections import deque

    h, w = mask.shape
    m = mask.copy()
    m[0, :] = m[-1, :] = False
    m[:, 0] = m[:, -1] = False
    seen = np.zeros_like(m)
    best, best_area = None, 0
    for y in range(h):
        for x in range(w):
            if not m[y, x] or seen[y, x]:
                continue
            q = deque([(y, x)])
            seen[y, x] = True
            y0 = y1 = y
            x0 = x1 = x
            while q:
                cy, cx = q.popleft()
                y0, y1, x0, x1 = min(y0, cy), max(y1, cy), min(x0, cx), max(x1, cx)
                for dy in (-1, 0, 1):
                    for dx in (-1, 0, 1):
                        ny, nx = cy + dy, cx + dx
                        if 0 <= ny < h and 0 <= nx < w and m[ny, nx] and not seen[ny, nx]:
                            seen[ny, nx] = True
                            q.append((ny, nx))
            area = (x1 - x0 + 1) * (y1 - y0 + 1)
            if area > best_area:
                best, best_area = (x0, y0, x1 - x0 + 1, y1 - y0 + 1), area
    return best


def test_image_roi_matches_flood_fill():
    rng = np.random.default_rng(4)
    for trial in range(30):
        h, w = int(rng.integers(3, 40)), int(rng.integers(3, 40))
        img = (rng.random((h, w)) < rng.uniform(0.05, 0.5)).astype(np.uint16) * rng.integers(1, 5000, (h, w))
        img = img.astype(np.uint16)
        if not (img[1:-1, 1:-1] != 0).any():
            with pytest.raises(pg.PadentiError, match="no pixel > 0"):
                pg.image_roi(img)
            continue
        assert pg.image_roi(img) == _roi_by_flood_fill(img != 0), trial
    # two components with equal rectangles: the first in raster order wins
    img = np.zeros((10, 12), np.uint8)
    img[2:4, 2:4] = 1
    img[6:8, 7:9] = 1
    assert pg.image_roi(img) == (2, 2, 2, 2)


def test_image_roi_compares_in_the_element_type():
    """The reference's mask is img > 0: negative pixels (int16 depth, float) and -0.0f are
    background, not foreground."""
    rng = np.random.default_rng(5)
    for dtype in (np.int16, np.int32, np.float32):
        for trial in range(10):
            h, w = int(rng.integers(5, 30)), int(rng.integers(5, 30))
            img = rng.integers(-3, 3, (h, w)).astype(dtype)
            if dtype == np.float32:
                img[img == 0] = -0.0
            if not (img[1:-1, 1:-1] > 0).any():
                continue
            assert pg.image_roi(img) == _roi_by_flood_fill(img > 0), (dtype, trial)
    # a large negative region beside a small positive one: only the positive one counts
    img = np.full((12, 12), -5, np.int16)
    img[0, :] = img[-1, :] = img[:, 0] = img[:, -1] = 0
    img[3:5, 6:9] = 7
    assert pg.image_roi(img) == (6, 3, 3, 2)
    with pytest.raises(ValueError):
        pg.image_roi(np.ones((4, 4), np.float64))


def test_roi_loaders_crop(tmp_path):
    depth = np.zeros((30, 40), np.uint16)
    depth[5:12, 6:20] = 900
    depth[20:22, 30:32] = 800  # a smaller component
    pg.write_pnm(tmp_path / "d.pgm", depth)
    ld = pg.PNMImageROILoader(np.uint16, 1)
    crop = ld.load(tmp_path / "d.pgm")
    assert (ld.roi_x, ld.roi_y) == (6, 5) and crop.shape == (7, 14) and np.all(crop == 900)


def test_cpp_roi_loader(tmp_path):
    """PNMImageROILoader of the C++ facade crops as the Python loader does (host code, no GPU)."""
    import subprocess

    from test_cpp_facade import CPP, _compile

    exe = tmp_path / "facade_roi"
    _compile(CPP / "facade_roi.cpp", exe, link=True)
    depth = np.zeros((30, 40), np.uint16)
    depth[5:12, 6:20] = 900
    depth[6, 7] = 901
    depth[20:22, 30:32] = 800
    pg.write_pnm(tmp_path / "d.pgm", depth)
    r = subprocess.run([str(exe), str(tmp_path / "d.pgm")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ld = pg.PNMImageROILoader(np.uint16, 1)
    crop = ld.load(tmp_path / "d.pgm")
    want = f"{crop.shape[1]} {crop.shape[0]} {ld.roi_x} {ld.roi_y} {crop[0, 0]}"
    assert r.stdout.split("\n")[:2] == [want, want]


@pytest.mark.gpu
def test_rgb_labels_roi_loader(tmp_path):
    colours = [(255, 0, 0), (0, 0, 255)]
    rgb = np.zeros((40, 50, 3), np.uint8)
    rgb[8:30, 10:22] = colours[0]
    rgb[12:16, 12:18] = colours[1]
    rgb[33:35, 40:45] = colours[1]  # a smaller component
    rgb[2, 2] = (9, 9, 9)           # an unknown colour: unlabelled
    pg.write_pnm(tmp_path / "l.ppm", rgb)
    ld = pg.RGBLabelsROILoader(colours)
    lab = ld.load(tmp_path / "l.ppm")
    full = ob.rgb_to_labels(rgb, colours)
    x, y, w, h = _roi_by_flood_fill(full != 0)
    assert (ld.roi_x, ld.roi_y, lab.shape[1], lab.shape[0]) == (x, y, w, h) == (10, 8, 12, 22)
    assert np.array_equal(lab, full[y:y + h, x:x + w])
