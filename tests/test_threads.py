"""Threading contract of the C ABI: one stream per context, calls on one context serialised by
the caller, separate contexts usable from separate threads; the last error is per thread."""
import ctypes as C
import threading

import numpy as np
import pytest

import padenti_gb300 as pg
from cases import depth_case
from padenti_gb300 import _native as N


def test_last_error_is_per_thread():
    msgs = {}

    def fail(tag, cfg):
        h = C.c_void_p()
        rc = N.lib().pd_ctx_create(C.byref(cfg), 0, C.byref(h))
        msgs[tag] = (rc, N.lib().pd_last_error())

    bad_k = pg.ForestConfig("depth_diff2", 3).c()
    bad_k.n_classes = 1000
    bad_plugin = pg.ForestConfig("depth_diff2", 3).c()
    bad_plugin.plugin = 77
    ts = [threading.Thread(target=fail, args=("k", bad_k)), threading.Thread(target=fail, args=("p", bad_plugin))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert msgs["k"][0] != 0 and b"nClasses" in msgs["k"][1]
    assert msgs["p"][0] != 0 and b"nClasses" not in msgs["p"][1]


@pytest.mark.gpu
def test_contexts_train_concurrently_in_threads():
    cfg, ts, tp, _ = depth_case(n_images=12, n_features=48, n_thresholds=16)
    want = {}
    for tid in (1, 2):
        t = pg.Tree(cfg, tid, 7)
        pg.TreeTrainer(cfg).train(t, ts, tp)
        want[tid] = t
    got, errors = {}, []

    def run(tid):
        try:
            tr = pg.TreeTrainer(cfg)
            for _ in range(2):
                t = pg.Tree(cfg, tid, 7)
                tr.train(t, ts, tp)
            got[tid] = t
        except Exception as e:  # reported below
            errors.append(e)

    threads = [threading.Thread(target=run, args=(tid,)) for tid in (1, 2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for tid in (1, 2):
        assert np.array_equal(got[tid].left_child, want[tid].left_child)
        assert np.array_equal(got[tid].thresholds, want[tid].thresholds)
        assert np.array_equal(got[tid].posteriors.view(np.uint32), want[tid].posteriors.view(np.uint32))
