"""Pins of the CPU oracle (no GPU).

- MD5 counter RNG: RFC-1321 known answers (Python hashlib) and the reference's
  own src/padenti/prng.hpp compiled from source (oracle/_ref).
- Candidate draws: an independent numpy restatement of the float formula of
  kernels/hist_update.cl:94-111,150-151.
- Split rule: the reference's own learnBestFeature kernel
  (kernels/learn_best_feature.cl) compiled from source, on the same histograms.
- Single-offset plugin: the reference's own test/feature.cl compiled from source.
- The exact log2 table against the platform libm.
"""
import ctypes as C
import hashlib
import math
import struct

import numpy as np
import pytest

import oracle_bind as ob


def _md5_words(w):
    return struct.unpack("<4I", hashlib.md5(struct.pack("<4I", *w)).digest())


def test_md5_matches_hashlib():
    rng = np.random.default_rng(0)
    cases = [(0, 0, 0, 0), (0xFFFFFFFF,) * 4, (3, 7, 123, 1)] + [tuple(int(x) for x in rng.integers(0, 2**32, 4))
                                                                for _ in range(3000)]
    for w in cases:
        assert ob.md5(w) == _md5_words(w), w
    assert ob.md5((3, 7, 123, 1)) == (0x68FB9095, 0x5C236288, 0x1B05FDFD, 0x56231E08)


def test_md5_matches_reference_prng():
    ref = ob.ref("prng")
    if ref is None:
        pytest.skip("reference prng.hpp not compiled here (oracle/_ref absent)")
    rng = np.random.default_rng(1)
    U4 = C.c_uint32 * 4
    for _ in range(3000):
        w = [int(x) for x in rng.integers(0, 2**32, 4)]
        out = U4()
        ref.ref_md5Rand(U4(*w), out)
        assert tuple(out) == ob.md5(w)


def _draw32(r, lo, hi, narrow=np.int32):
    x = np.float32(np.float32(r) / np.float32(4294967296.0)) * np.float32(hi - lo)
    x = np.float32(x)
    return int(narrow(np.int32(lo) + np.int32(np.trunc(x))))


def test_candidate_draws_independent_restatement():
    import padenti_gb300 as pg

    cfg = pg.ForestConfig("depth_diff2", 3)
    tp = pg.TreeTrainerParameters(10, 9, [-60000, -50000, -1, 0], [60000, 50000, 1, 7], -500, 500)
    p = ob.params(cfg, tp)
    for node, f in [(0, 0), (5, 3), (1234, 9), (2**20, 7)]:
        feat, thr = ob.candidate(p, 11, node, f)
        seed = _md5_words((11, node, f, 0))
        exp = [_draw32(seed[j], tp.feat_low_bounds[j], tp.feat_up_bounds[j]) for j in range(4)]
        assert list(feat) == exp
        s = (11, node, f, 1)
        exp_t = []
        for t in range(9):
            if t % 4 == 0:
                s = _md5_words(s)
            exp_t.append(_draw32(s[t % 4], -500, 500))
        assert list(thr) == exp_t


def _exact_gain(h, tot, t, f):
    """Canonical gain of candidate (t, f) in float64 (entropy with the p <= 1e-6 cutoff)."""
    def ent(c, n):
        c = c[(c > 0) & (c * 1e6 > n)].astype(np.float64)
        return float(-(c / n * np.log2(c / n)).sum()) if n else 0.0

    cl = h[:, t, f].astype(np.float64)
    cr = tot.astype(np.float64) - cl
    N, nl, nr = float(tot.sum()), float(cl.sum()), float(cr.sum())
    return ent(tot.astype(np.float64), N) - (nl / N * ent(cl, nl) + nr / N * ent(cr, nr))


def _ref_learn(hist, tot, F, T, K):
    """Run the reference learnBestFeature kernel + host max_element (learn_best_featthr.hpp:86-112)."""
    ref = ob.ref("learn")
    n = hist.shape[0]
    per_thread = 64
    n_threads = n * F * T // per_thread
    bf = np.zeros(n_threads, np.uint32)
    bt = np.zeros(n_threads, np.uint32)
    be = np.zeros(n_threads, np.float32)
    h = np.ascontiguousarray(hist, np.uint32)
    tt = np.ascontiguousarray(tot, np.uint32)
    ref.ref_learn_best_feature(ob.P(h), ob.P(tt), C.c_uint(F), C.c_uint(T), C.c_uint(K), C.c_uint(per_thread),
                               ob.P(bf), ob.P(bt), ob.P(be), C.c_size_t(n_threads))
    per_node = n_threads // n
    out = []
    for i in range(n):
        e = be[i * per_node:(i + 1) * per_node]
        b = int(np.argmax(e))  # first maximum, as std::max_element
        out.append((int(bt[i * per_node + b]), int(bf[i * per_node + b]), float(e[b])))
    return out


@pytest.mark.parametrize("K,T,F", [(3, 16, 64), (9, 8, 128), (21, 4, 96)])
def test_split_agrees_with_reference_kernel(K, T, F):
    if ob.ref("learn") is None:
        pytest.skip("reference learn_best_feature.cl not compiled here (oracle/_ref absent)")
    import padenti_gb300 as pg

    rng = np.random.default_rng(K * 100 + T)
    n = 24
    tot = rng.integers(1, 400, size=(n, K)).astype(np.uint32)
    tot[:, 0] += 500
    # cumulative-style histograms: left counts in [0, tot]
    hist = (rng.random((n, K, T, F)) * tot[:, :, None, None]).astype(np.uint32)
    cfg = pg.ForestConfig("depth_diff2", K)
    tp = pg.TreeTrainerParameters(F, T, [0] * 4, [1] * 4, 0, 1)
    p = ob.params(cfg, tp)
    t, f, g, g32, err = ob.split(p, hist, tot)
    ref = _ref_learn(hist, tot, F, T, K)
    eps = (3 * K + 3) * 4.4e-7
    agree = 0
    for i in range(n):
        rt, rf, rg = ref[i]
        # the FP32 reference gain of the oracle winner is within FP32 error of the reference best
        assert abs(rg - g[i]) < 1e-4
        if (rt, rf) == (int(t[i]), int(f[i])):
            agree += 1
            continue
        # every disagreement is an FP32 near-tie: the reference's winner is, in exact arithmetic,
        # within 2 eps(K) of the oracle's (the FP32 gains of both lie within eps of their exact values)
        gap = g[i] - _exact_gain(hist[i], tot[i], rt, rf)
        assert -1e-12 <= gap <= 2 * eps, (i, gap)
    assert agree >= n - 2
    # the FP32 error bound the CUDA split sizes its FP64 recheck window from
    assert err < eps


def test_split_ties_lowest_index_and_empty():
    import padenti_gb300 as pg

    cfg = pg.ForestConfig("depth_diff2", 3)
    tp = pg.TreeTrainerParameters(8, 4, [0] * 4, [1] * 4, 0, 1)
    p = ob.params(cfg, tp)
    tot = np.array([[10, 10, 10], [0, 0, 0]], np.uint32)
    h = np.zeros((2, 3, 4, 8), np.uint32)
    h[0] = 5
    h[0, :, 2, 5] = [10, 0, 0]
    h[0, :, 1, 7] = [10, 0, 0]
    t, f, g, _, _ = ob.split(p, h, tot)
    assert (t[0], f[0]) == (1, 7)
    assert (t[1], f[1]) == (-1, -1)


def test_reference_feature_plugin():
    ref = ob.ref("feature")
    if ref is None:
        pytest.skip("reference test/feature.cl not compiled here (oracle/_ref absent)")
    import padenti_gb300 as pg

    px, lb, sm = pg.synth_depth(3, 2, 160, 120)
    img = np.ascontiguousarray(px[0])
    rng = np.random.default_rng(4)
    lib = ob.lib()
    ref.ref_compute_feature.restype = C.c_int
    for _ in range(5000):
        x, y = int(rng.integers(0, 160)), int(rng.integers(0, 120))
        feat = rng.integers(-60, 61, size=2).astype(np.int16)
        r = ref.ref_compute_feature(ob.P(img), C.c_uint(160), C.c_uint(120), C.c_int(x), C.c_int(y), ob.P(feat))
        f32 = feat.astype(np.int32)
        o = lib.or_feature(2, 1, ob.P(img), C.c_uint32(160), C.c_uint32(120), C.c_uint32(1), C.c_int32(x),
                           C.c_int32(y), ob.P(f32))
        assert r == o, (x, y, feat)


def test_log2_table_against_libm():
    n = 1 << 20
    t = ob.log2_table(n)
    assert t[0] == 0.0 and t[1] == 0.0
    idx = np.arange(2, n)
    lib = np.array([math.log2(int(i)) for i in idx[:: 97]])
    assert np.max(np.abs(t[2::97] - lib) / lib) < 2.3e-16
    # powers of two are exact
    for k in range(1, 20):
        assert t[1 << k] == float(k)
    # where the table and libm disagree, the table is the correctly rounded one
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    dense = np.array([math.log2(i) for i in range(2, 200_000)])
    bad = np.nonzero(t[2:200_000] != dense)[0] + 2
    assert len(bad) < 100
    for i in bad:
        assert t[i] == float(mpmath.log(int(i), 2)), i
