"""The FP32 filter of the fused split stays within its stated error bound.

The histogram kernel's fused split ranks candidates by -(S_L + S_R) in FP32,
S(c, n) = n log2 n - sum_l c_l log2 c_l, with a float table of c log2 c and
sequential sums, and re-evaluates in exact FP64 every candidate within
2 (2K + 5) u N log2 N of the FP32 maximum.  That is safe when the FP32 error is
at most (K + 3) u N log2 N (u = 2^-24).  This test emulates the kernel's
arithmetic in numpy float32 and checks that bound on random and skewed class
counts (nodes of up to 65535 samples, the largest a fused split sees).
"""
import numpy as np

U = 2.0 ** -24


def _xlog2(c):
    c = np.asarray(c, np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(c > 0, c * np.log2(np.maximum(c, 1)), 0.0)


def _filter32(X, left, tot):
    nL = int(left.sum())
    N = int(tot.sum())
    sl, sr = X[nL], X[N - nL]
    for cl, t in zip(left, tot):
        sl = np.float32(sl - X[int(cl)])
        sr = np.float32(sr - X[int(t - cl)])
    return float(np.float32(sl + sr))


def _exact(left, tot):
    nL, N = left.sum(), tot.sum()
    return float(_xlog2(nL) - _xlog2(left).sum() + _xlog2(N - nL) - _xlog2(tot - left).sum())


def test_fused_filter_error_bound():
    rng = np.random.default_rng(7)
    X = _xlog2(np.arange(65536)).astype(np.float32)
    worst = 0.0
    for trial in range(3000):
        K = int(rng.choice([2, 3, 9, 21, 64]))
        N = int(rng.choice([21, 100, 1000, 4096, 16384, 65535]))
        if trial % 3 == 0:  # skewed: one dominant class
            p = np.full(K, 0.01 / max(K - 1, 1))
            p[rng.integers(K)] = 0.99
        else:
            p = rng.dirichlet(np.full(K, 0.5))
        tot = rng.multinomial(N, p / p.sum())
        left = rng.binomial(tot, rng.uniform())
        err = abs(_filter32(X, left, tot) - _exact(left, tot))
        bound = (K + 3) * U * N * np.log2(N)
        assert err <= bound, (K, N, err, bound)
        worst = max(worst, err / bound)
    assert worst < 0.5  # the bound is not tight; the kernel's window is twice it plus margin
