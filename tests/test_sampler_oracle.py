"""The CPU restatement of the pixel samplers (oracle/image_sampler.c) against its pins:
zlib's CRC-32, the C++ standard's MT19937 known answer and numpy's MT19937, Boost's
bucket method on ranges where it has a closed form, and the reference's own
UniformImageSampler / ClassWeightedImageSampler compiled from their sources
(oracle/_ref/libref_sampler.so, skipped where the Padenti sources were absent at build
time)."""
import zlib

import numpy as np
import pytest

import oracle_bind as ob
import padenti_gb300 as pg


def test_crc32_matches_zlib():
    assert ob.crc32(np.frombuffer(b"123456789", np.uint8)) == 0xCBF43926
    rng = np.random.default_rng(3)
    for n in [0, 1, 15, 16, 17, 1000, 614400]:
        b = rng.integers(0, 256, n, dtype=np.uint8)
        assert ob.crc32(b) == zlib.crc32(b.tobytes())


def test_mt19937_known_answer_and_numpy():
    assert int(ob.mt_outputs(5489, 10000)[-1]) == 4123659995  # the C++ standard's check value
    for seed in [0, 1, 0xDEADBEEF, 0xFFFFFFFF]:
        rs = np.random.RandomState(seed)
        want = rs.randint(0, 2**32, size=2000, dtype=np.uint64).astype(np.uint32)
        assert np.array_equal(ob.mt_outputs(seed, 2000), want)


def test_uniform_int_bucket_method():
    raw = ob.mt_outputs(77, 4000).astype(np.uint64)
    # a power-of-two range: no rejection, the top bits of each draw
    assert np.array_equal(ob.uniform_ints(77, 1023, 1000), (raw[:1000] >> 22).astype(np.uint32))
    # range 0: no draw at all
    assert np.array_equal(ob.uniform_ints(77, 0, 5), np.zeros(5, np.uint32))
    # a general range: quotient by floor(2^32/n), rejected above the range
    n = 300007
    bucket = (1 << 32) // n
    q = raw // bucket
    want = q[q < n][:1000]
    assert np.array_equal(ob.uniform_ints(77, n - 1, 1000), want.astype(np.uint32))


def _images():
    px, lb, _ = pg.synth_depth(5, 3, 80, 60, parts=1, min_ellipses=2, max_ellipses=4, samples_per_image=10)
    rgb, rlb, _ = pg.synth_rgb(5, 2, 48, 40, n_classes=6, samples_per_image=10)
    sparse = lb[0].copy()
    sparse[:] = 0
    sparse[10, 7], sparse[30, 50] = 2, 5
    single = np.zeros_like(lb[1])
    single[20, 20] = 1
    return [(2, px[0], lb[0], 9), (2, px[1], lb[1], 9), (2, px[2], sparse, 9), (2, px[2], single, 9),
            (1, rgb[0], rlb[0], 6), (1, rgb[1], rlb[1], 6)]


@pytest.mark.parametrize("n_samples,seed", [(500, 0), (37, 123456), (2000, 7)])
def test_uniform_sampler_matches_reference_source(n_samples, seed):
    if ob.ref("sampler") is None:
        pytest.skip("reference sampler not built (Padenti sources absent at build time)")
    for img_type, data, labels, _ in _images():
        got = ob.sample_uniform(data, labels, n_samples, seed)
        want = ob.ref_sample_uniform(img_type, data, labels, n_samples, seed)
        assert np.array_equal(got, want)
        assert got.size == n_samples and np.all(np.diff(got.astype(np.int64)) >= 0)
        assert np.all(labels.reshape(-1)[got] != 0)


@pytest.mark.parametrize("weights", [None, "skewed", "zero"])
@pytest.mark.parametrize("n_samples,seed", [(300, 0), (2000, 99)])
def test_class_weighted_sampler_matches_reference_source(weights, n_samples, seed):
    if ob.ref("sampler") is None:
        pytest.skip("reference sampler not built (Padenti sources absent at build time)")
    for img_type, data, labels, k in _images():
        w = None
        if weights == "skewed":
            w = np.linspace(0.02, 0.3, k).astype(np.float32)
        elif weights == "zero":
            w = np.full(k, 1.0 / (k - 1), np.float32)
            w[1] = 0
        got = ob.sample_class_weighted(data, labels, n_samples, k, w, seed)
        want = ob.ref_sample_class_weighted(img_type, data, labels, n_samples, k, w, seed)
        assert np.array_equal(got, want)
        sizes = ob.bucket_sizes(n_samples, k, w)
        counts = np.bincount(labels.reshape(-1), minlength=k + 1)[1:]
        assert got.size == int(np.minimum(sizes, counts).sum())


def test_uniform_sampler_without_labelled_pixels_returns_nothing():
    px, lb, _ = pg.synth_depth(5, 1, 32, 24, samples_per_image=4)
    assert ob.sample_uniform(px[0], np.zeros_like(lb[0]), 100, 0).size == 0
