"""pd_split_noalloc -- the best split for callers that cannot allocate device
memory (a host that only lends memory from its own pool, a runtime whose
allocator must not be bypassed).  It works in a fixed array inside the library instead of allocating, and
must give exactly what pd_split gives.  Two calls in a row check that the shared
array is reset between calls.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import oracle_bind as ob
import padenti_gb300 as pg
from cases import depth_case, sample_labels
from padenti_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _case(nodes, seed):
    cfg, ts, tp, _ = depth_case(n_images=12, n_features=96, n_thresholds=20)
    rng = np.random.default_rng(seed)
    sample_node = rng.choice(nodes, size=ts.n_samples).astype(np.int32)
    hist = ob.hist(ob.params(cfg, tp), ob.OracleSet(ts, cfg), 1, sample_node, nodes)
    labels = sample_labels(ts)
    ctot = np.stack([np.bincount(labels[sample_node == n], minlength=cfg.n_classes) for n in nodes]).astype(np.uint32)
    return cfg, tp, hist, ctot


def test_split_noalloc_matches_pd_split_twice_in_a_row():
    torch = pytest.importorskip("torch")  # the caller's own device buffers
    for nodes, seed in (([3, 4, 5, 6], 0), ([7, 8, 9], 1)):
        cfg, tp, hist, ctot = _case(nodes, seed)
        t_ref, f_ref, g_ref = pg.TreeTrainer(cfg).split(tp, hist, ctot)
        n = len(nodes)
        d_hist = torch.from_numpy(hist.view(np.int32)).cuda()
        d_tot = torch.from_numpy(ctot.view(np.int32)).cuda()
        d_t = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        d_f = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        d_g = torch.zeros(n, dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        rc = N.lib().pd_split_noalloc(C.byref(tp.c()), cfg.n_classes, d_hist.data_ptr(), d_tot.data_ptr(), n,
                                      d_t.data_ptr(), d_f.data_ptr(), d_g.data_ptr(), stream)
        N.check(rc)
        assert np.array_equal(d_t.cpu().numpy(), t_ref)
        assert np.array_equal(d_f.cpu().numpy(), f_ref)
        assert np.array_equal(d_g.cpu().numpy().view(np.uint64), g_ref.view(np.uint64))


def test_split_noalloc_rejects_oversized_work():
    cfg = pg.ForestConfig("depth_diff2", 9)
    tp = pg.TreeTrainerParameters(2000, 50, [0] * 4, [1] * 4, 0, 1)
    fake = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = N.lib().pd_split_noalloc(C.byref(tp.c()), 9, fake, fake, 1000, fake, fake, fake, None)
    assert rc == -4 and b"working memory" in N.lib().pd_last_error()
