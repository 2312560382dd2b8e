"""Learned candidate proposals: the proposal network's forward pass and gradients against the
CPU oracle (oracle/proposal.c), its fit, and trees trained with it.

The oracle's gradient is itself checked against central finite differences of its loss in
double precision (no BF16 rounding).  The GPU kernels compute with BF16 operands and FP32
accumulation; the oracle mirrors the BF16 rounding points, and the comparison tolerance is
stated in each test: outputs within 2e-2 of their scale, loss within 1e-3 relative, gradients
within 3e-2 relative L2 per parameter block with cosine above 0.999.
"""
import numpy as np
import pytest

import oracle_bind as ob

IN, OUT, DY, G = 16, 176, 5, 16


def _layout(IN, H, OUT):
    din, dn = [IN, H, H, H], [H, H, H, OUT]
    blocks, o = [], 0
    for l in range(4):
        blocks.append((f"W{l}", o, o + din[l] * dn[l]))
        o += din[l] * dn[l]
        blocks.append((f"b{l}", o, o + dn[l]))
        o += dn[l]
    return blocks, o


def _init(IN, H, OUT, rng, scale=1.0):
    blocks, P = _layout(IN, H, OUT)
    p = np.zeros(P, np.float32)
    din = [IN, H, H, H]
    dn = [H, H, H, OUT]
    for l in range(4):
        _, a, b = blocks[2 * l]
        lim = np.sqrt(6.0 / (din[l] + dn[l])) * scale
        p[a:b] = rng.uniform(-lim, lim, b - a)
        _, a, b = blocks[2 * l + 1]
        p[a:b] = rng.normal(0, 0.1, b - a)
    return p


def _rows(n, rng, IN=IN, K=9):
    x = np.zeros((n, IN), np.float32)
    x[:, 0] = rng.integers(1, 16, n) / 24.0
    x[:, 1] = rng.uniform(4, 22, n) / 24.0
    c = rng.dirichlet(np.ones(K), n)
    x[:, 2:2 + K] = c
    y = rng.uniform(-1, 1, (n, DY)).astype(np.float32)
    w = rng.uniform(0.5, 1.5, n).astype(np.float32)
    return x, y, w


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    H = 32
    p = _init(IN, H, OUT, rng)
    x, y, w = _rows(6, rng)
    loss, g = ob.prop_loss_grad(p, IN, H, OUT, DY, x, y, w, bf16=False)
    blocks, P = _layout(IN, H, OUT)
    idx = np.concatenate([rng.integers(a, b, 6) for _, a, b in blocks])
    for i in idx:
        h = 1e-3 * max(1.0, abs(float(p[i])))
        pp, pm = p.astype(np.float64), p.astype(np.float64)
        pp = pp.copy(); pm = pm.copy()
        pp[i] += h
        pm[i] -= h
        # the oracle takes float32 parameters: use steps exactly representable around p[i]
        hp = np.float32(pp[i]) - p[i]
        hm = p[i] - np.float32(pm[i])
        lp, _ = ob.prop_loss_grad(pp.astype(np.float32), IN, H, OUT, DY, x, y, w, bf16=False)
        lm, _ = ob.prop_loss_grad(pm.astype(np.float32), IN, H, OUT, DY, x, y, w, bf16=False)
        fd = (lp - lm) / (float(hp) + float(hm))
        assert abs(fd - g[i]) <= 1e-4 * max(1.0, abs(g[i])) + 1e-6, (i, fd, g[i])


def _proposer(K=9):
    import padenti_gb300 as pg

    cfg = pg.ForestConfig("depth_diff2", K)
    tr = pg.TreeTrainer(cfg)
    tp = pg.TreeTrainerParameters(300, 50, [-60000] * 4, [60000] * 4, -500, 500, 20)
    return tr, tp, pg.ProposalNetwork(tr, tp, seed=7)


@pytest.mark.gpu
def test_gpu_forward_and_gradient_match_oracle():
    tr, tp, net = _proposer()
    assert (net.in_dim, net.hidden, net.out_dim, net.components, net.drawn) == (IN, 256, OUT, G, DY)
    rng = np.random.default_rng(1)
    for trial, p in enumerate([net.params, _init(IN, 256, OUT, rng, scale=1.5)]):
        net.params = p
        x, y, w = _rows(300, rng)
        out = net.forward(x)
        ref = ob.prop_forward(p, IN, 256, OUT, x, bf16=True)
        scale = np.abs(ref).max()
        assert np.abs(out - ref).max() <= 2e-2 * scale, (trial, np.abs(out - ref).max(), scale)
        loss, g = net.loss_grad(x, y, w)
        rl, rg = ob.prop_loss_grad(p, IN, 256, OUT, DY, x, y, w, bf16=True)
        assert abs(loss - rl) <= 1e-3 * abs(rl), (trial, loss, rl)
        blocks, P = _layout(IN, 256, OUT)
        assert g.size == P
        for name, a, b in blocks:
            gb, rb = g[a:b].astype(np.float64), rg[a:b]
            nr = np.linalg.norm(rb)
            if nr == 0:
                continue
            rel = np.linalg.norm(gb - rb) / nr
            cos = float(gb @ rb) / (np.linalg.norm(gb) * nr)
            assert rel < 3e-2 and cos > 0.999, (trial, name, rel, cos)


@pytest.mark.gpu
def test_gpu_fit_lowers_the_loss_and_is_deterministic():
    import padenti_gb300 as pg

    tr, tp, net = _proposer()
    rng = np.random.default_rng(2)
    n = 5000
    rec = np.zeros(n, pg.RECORD_DTYPE)
    rec["depth"] = rng.integers(1, 16, n)
    rec["count"] = rng.integers(21, 100000, n)
    cc = (rng.dirichlet(np.ones(9), n) * rec["count"][:, None]).astype(np.uint32)
    rec["class_count"][:, :9] = cc
    rec["count"] = cc.sum(1)
    # winners concentrated around a depth-dependent offset: something to learn
    centre = (rec["depth"][:, None] * 3000 - 24000).astype(np.int64)
    rec["feat"][:, :4] = np.clip(centre + rng.normal(0, 2000, (n, 4)), -60000, 60000).astype(np.int32)
    rec["thr"] = rng.integers(-100, 100, n)
    p0 = net.params
    r1 = net.fit(rec, steps=200, batch=1024, lr=2e-3)
    loss = r1["loss"]
    assert np.all(np.isfinite(loss)) and loss[-20:].mean() < loss[:20].mean() - 1.0, loss[[0, 19, -20, -1]]
    p1 = net.params
    net.params = p0
    r2 = net.fit(rec, steps=200, batch=1024, lr=2e-3)
    assert np.array_equal(r2["loss"], loss) and np.array_equal(net.params, p1)


@pytest.mark.gpu
def test_proposed_tree_without_proposals_is_the_plain_tree():
    """n_proposed = 0: every candidate is the reference's uniform one, so the tree is the
    plain trainer's, bit for bit (the candidate column order does not change results)."""
    import padenti_gb300 as pg
    from cases import depth_case

    cfg, ts, tp, _ = depth_case(n_images=10, n_features=96, n_thresholds=20, parts=1)
    tr = pg.TreeTrainer(cfg)
    net = pg.ProposalNetwork(tr, tp, seed=3)
    a = pg.Tree(cfg, 2, 9)
    tr.train(a, ts, tp)
    b = pg.Tree(cfg, 2, 9)
    tr.train_proposed(b, ts, tp, net, 0)
    for f in ("left_child", "features", "thresholds"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    assert np.array_equal(a.posteriors.view(np.uint32), b.posteriors.view(np.uint32))


@pytest.mark.gpu
def test_proposed_tree_is_valid_deterministic_and_records_match():
    """A tree with 48 proposed + 48 uniform candidates per node: identical on a second run,
    its split values within the bounds, every node's posterior equal to the class frequencies
    of its samples, and the records of the plain trainer equal to its split nodes."""
    import padenti_gb300 as pg
    from cases import depth_case, sample_labels

    cfg, ts, tp, _ = depth_case(n_images=10, n_features=96, n_thresholds=20, parts=1)
    tr = pg.TreeTrainer(cfg)
    tr.set_tuning("records", 1)
    plain = pg.Tree(cfg, 0, 9)
    tr.train(plain, ts, tp)
    rec = tr.records()
    split = np.nonzero(plain.left_child >= 0)[0]
    assert sorted(rec["node"].tolist()) == sorted(split.tolist())
    for r in rec:
        assert np.array_equal(r["feat"][:4], plain.features[r["node"]]) and r["thr"] == plain.thresholds[r["node"]]
    net = pg.ProposalNetwork(tr, tp, seed=3)
    net.fit(rec, steps=50, batch=256)
    t1, t2 = pg.Tree(cfg, 1, 9), pg.Tree(cfg, 1, 9)
    tr.train_proposed(t1, ts, tp, net, 48)
    tr.train_proposed(t2, ts, tp, net, 48)
    for f in ("left_child", "features", "thresholds", "posteriors"):
        assert np.array_equal(getattr(t1, f), getattr(t2, f)), f
    # the candidate tables sorted in shared memory instead of registers: the same tree
    tr.set_tuning("cand_regs", 0)
    t3 = pg.Tree(cfg, 1, 9)
    tr.train_proposed(t3, ts, tp, net, 48)
    tr.set_tuning("cand_regs", 1)
    for f in ("left_child", "features", "thresholds", "posteriors"):
        assert np.array_equal(getattr(t1, f), getattr(t3, f)), f
    s = t1.left_child >= 0
    assert s.sum() >= 10
    assert np.all(t1.features[s] >= -60000) and np.all(t1.features[s] <= 60000)
    assert np.all(t1.thresholds[s] >= -500) and np.all(t1.thresholds[s] <= 500)
    labels = sample_labels(ts)
    final = tr.sample_nodes(ts.n_samples).astype(np.int64)
    for node in np.nonzero(t1.left_child == -1)[0][:50]:
        # every sample under a leaf: class frequencies of the samples that reached it
        on = final == node
        if not on.any():
            continue
        c = np.bincount(labels[on], minlength=9).astype(np.float32)
        assert np.array_equal(t1.posteriors[node].view(np.uint32), (c / np.float32(c.sum())).view(np.uint32))


@pytest.mark.gpu
def test_network_gain_over_uniform_candidates():
    """What the trained network gains over the method without it: one tree with 25 proposed + 5
    uniform candidates per node against 30 uniform ones, on 150 synthetic 640x480 depth maps
    (9 classes, 2000 samples each), depth 12; the network is fitted to the records of a plain
    2000-candidate tree.  Held-out per-pixel accuracy on the object (non-background) pixels of
    30 unseen images must be at least 0.5 pt higher with the network (measured: about +2 pt)."""
    import padenti_gb300 as pg
    from bench import forest_accuracy

    px, lb, sm = pg.synth_depth(0, 150, 640, 480, parts=1, min_ellipses=2, max_ellipses=5, samples_per_image=2000,
                                bg_permille=100)
    cfg = pg.ForestConfig("depth_diff2", 9)
    ts = pg.training_set(9, px, lb, sm)
    tp = pg.TreeTrainerParameters(2000, 50, [-60000] * 4, [60000] * 4, -500, 500, 20)
    tr = pg.TreeTrainer(cfg)
    tr.set_tuning("records", 1)
    tr.train(pg.Tree(cfg, 0, 12), ts, tp)
    rec = tr.records()
    tr.set_tuning("records", 0)
    tp30 = pg.TreeTrainerParameters(30, 50, [-60000] * 4, [60000] * 4, -500, 500, 20)
    net = pg.ProposalNetwork(tr, tp30, seed=0)
    fit = net.fit(rec, steps=200, batch=2048, lr=2e-3)
    assert fit["loss"][-10:].mean() < fit["loss"][:10].mean() - 0.5
    hx, hl, _ = pg.synth_depth(0, 30, 640, 480, first_image=5_000_000, parts=1, min_ellipses=2, max_ellipses=5,
                               samples_per_image=1)
    learned, uniform = pg.Tree(cfg, 1, 12), pg.Tree(cfg, 1, 12)
    tr.train_proposed(learned, ts, tp30, net, 25)
    tr.train(uniform, ts, tp30)
    acc_l = forest_accuracy(pg, cfg, [learned], 0, hx, hl)
    acc_u = forest_accuracy(pg, cfg, [uniform], 0, hx, hl)
    assert acc_l[1] >= acc_u[1] + 0.005, (acc_l, acc_u)
