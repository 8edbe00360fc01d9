"""Reference options off the default path, on the GPU: gradient noise
(src/algos/ep/mod.rs:140-146, 239-247) and feature dropout (max_features,
src/algos/ep/model.rs:257-278 with src/algos/utils.rs:193-216)."""
import math

import numpy as np
import pytest

from cloverleaf_gb300 import _native
from tests._cases import random_problem, sample_batch

pytestmark = pytest.mark.gpu


def _ctx(prob, form=_native.FORM_PLAIN_FP32, noise=0.0, passes=1, batch_size=64, max_features=None):
    cfg = _native.default_config()
    cfg.dims, cfg.loss, cfg.gamma, cfg.negatives = prob["dims"], _native.LOSS_STARSPACE, 0.5, 4
    cfg.form, cfg.noise, cfg.passes, cfg.batch_size, cfg.valid_pct = form, noise, passes, batch_size, 0.0
    if max_features is not None:
        cfg.max_features_kind, cfg.max_features = max_features
    ctx = _native.Context(cfg)
    ctx.upload_graph(prob["rows"], prob["cols"], None)
    ctx.upload_features(prob["fptr"], prob["fids"], prob["n_feat"])
    ctx.set_table(prob["table"])
    return ctx


def test_noise_schedule_matches_reference():
    # sigma(step) = noise * decay^step, decay = exp((ln 1e-9 - ln noise) / total_updates)
    prob = random_problem(3, n=1000, n_feat=300, dims=32)
    noise, passes, B = 0.05, 3, 64
    ctx = _ctx(prob, noise=noise, passes=passes, batch_size=B)
    stats = ctx.train(passes)
    steps = -(-1000 // B)
    total = steps * passes
    decay = math.exp((math.log(1e-9) - math.log(noise)) / total)
    for p, s in enumerate(stats, start=1):
        want = noise * decay ** (p * steps)     # the last step of pass p
        assert s["noise_last"] == pytest.approx(want, rel=1e-4), (p, s["noise_last"], want)
    off = _ctx(prob).train(1)
    assert off[0]["noise_last"] == 0.0


def test_noise_is_applied_to_the_update():
    # First Adam step from zero moments moves each touched element by about
    # lr * 0.74 * sign(g + sigma * z): with sigma far above |g| about half of
    # the signs disagree with the noiseless step; with sigma = 0 none do.
    prob = random_problem(12, n=200, n_feat=120, dims=32)
    smp = sample_batch(13, prob, B=64, K=5, R=4)
    s = _native.Context.samples(smp["anchors"], smp["nbr_ptr"], smp["nbr"], smp["nbr_w"], smp["neg"])
    lr, t0 = 0.05, prob["table"]
    clean = _ctx(prob)
    clean.batch_step(s, lr, 1)
    d_clean = clean.get_table(prob["n_feat"], prob["dims"]) - t0
    noisy = _ctx(prob, noise=1e3)
    noisy.batch_step(s, lr, 1)
    t_noisy = noisy.get_table(prob["n_feat"], prob["dims"])
    d_noisy = t_noisy - t0
    touched = np.abs(d_clean) > 0.5 * lr * 0.74
    assert touched.sum() > 500
    flips = np.mean(np.sign(d_noisy[touched]) != np.sign(d_clean[touched]))
    assert 0.4 < flips < 0.6, flips
    assert np.array_equal(d_noisy[~touched.any(axis=1)], d_clean[~touched.any(axis=1)])
    again = _ctx(prob, noise=1e3)
    again.batch_step(s, lr, 1)
    assert np.array_equal(again.get_table(prob["n_feat"], prob["dims"]), t_noisy)   # same stream, same result


def _grad(ctx, prob, smp):
    s = _native.Context.samples(smp["anchors"], smp["nbr_ptr"], smp["nbr"], smp["nbr_w"], smp["neg"])
    return ctx.batch_grad(s, prob["n_feat"], prob["dims"])


def test_feature_dropout_fixed_k_at_least_n_is_no_dropout():
    # Fixed(k) with k >= every node's feature count keeps everything with
    # scalar n / n = 1: the same weights as All, bit for bit
    prob = random_problem(21, n=300, n_feat=200, dims=64, feats=(1, 6))
    smp = sample_batch(22, prob, B=96, K=5, R=4)
    a = _grad(_ctx(prob), prob, smp)
    b = _grad(_ctx(prob, max_features=(_native.SAMPLE_FIXED, 6.0)), prob, smp)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_feature_dropout_item_counts():
    prob = random_problem(23, n=2000, n_feat=500, dims=32, feats=(1, 8))
    full = _ctx(prob).train_batches(4)
    one = _ctx(prob, max_features=(_native.SAMPLE_FIXED, 1.0)).train_batches(4)
    # Fixed(1): one item per role node (every node has a feature)
    assert one["items"] == one["anchors"] * (1 + 4) + one["sampled_neighbors"]
    half = _ctx(prob, max_features=(_native.SAMPLE_PROB, 0.5)).train_batches(4)
    ratio = half["items"] / full["items"]
    assert 0.45 < ratio < 0.65, ratio        # E[max(Bin(n, 1/2), 1)] / E[n] = 0.53 for n uniform in 1..8
    for s in (one, half):
        assert np.isfinite(s["train_loss"]) and s["kept_anchors"] > 0


def test_feature_dropout_gradient_touches_a_subset():
    prob = random_problem(25, n=300, n_feat=200, dims=32, feats=(2, 8))
    smp = sample_batch(26, prob, B=96, K=5, R=4)
    _, _, ids_all, _ = _grad(_ctx(prob), prob, smp)
    _, st, ids, rows = _grad(_ctx(prob, max_features=(_native.SAMPLE_FIXED, 2.0)), prob, smp)
    assert set(ids.tolist()) < set(ids_all.tolist())
    assert np.isfinite(rows).all() and (st == 0).any()


def test_feature_dropout_recall_matches_cpu_reference(oracle):
    # both sides train with Fixed(3) feature dropout (their own random
    # streams); community recall@10 within 1 point, as for the default path
    import cloverleaf_gb300 as cl
    from cloverleaf_gb300 import datagen
    from tests._eval import community_recall
    w = datagen.workload("sbm10k")
    ep = w["ep"]
    g = cl.Graph.from_csr(w["rows"], w["cols"], w["weights"])
    fs = cl.FeatureSet.from_csr(g, w["fptr"], w["fids"], w["n_feat"])
    prop = cl.EmbeddingPropagator(alpha=ep["alpha"], loss=cl.EPLoss.starspace(ep["gamma"], ep["negatives"]),
                                  batch_size=ep["batch_size"], dims=ep["dims"], passes=ep["passes"],
                                  max_nodes=ep["max_nodes"], max_features=3, valid_pct=0.0, indicator=False,
                                  form="fused")
    emb = prop.learn_features(g, fs)
    r_gpu = community_recall(w["fptr"], w["fids"], emb.table, w["community"])
    table, _ = oracle.train(w["rows"], w["cols"], w["weights"], w["fptr"], w["fids"], w["n_feat"], dims=ep["dims"],
                            alpha=ep["alpha"], loss=oracle.LOSS_STARSPACE, gamma=ep["gamma"],
                            negatives=ep["negatives"], batch_size=ep["batch_size"], passes=ep["passes"],
                            max_nodes=(oracle.SAMPLE_FIXED, ep["max_nodes"]),
                            max_features=(oracle.SAMPLE_FIXED, 3.0), threads=0)
    r_cpu = community_recall(w["fptr"], w["fids"], table, w["community"])
    assert abs(r_gpu - r_cpu) <= 0.01, (r_gpu, r_cpu)


def _bfs(rows, cols, src, limit=10):
    dist = {src: 0}
    frontier = [src]
    for d in range(1, limit + 1):
        nxt = []
        for u in frontier:
            for x in cols[int(rows[u]):int(rows[u + 1])].tolist():
                if x not in dist:
                    dist[x] = d
                    nxt.append(x)
        frontier = nxt
    return dist


def test_hard_negatives_are_walk_ends_off_the_neighbourhood():
    # RandomWalkHardSampler (node_sampler.rs:83-145): the first negatives are
    # distinct end nodes of short restart walks, neither the anchor nor one
    # of its neighbours; the rest are uniform over the training ids
    prob = random_problem(31, n=4000, n_feat=300, dims=16, deg=(2, 4))
    H, R, B = 3, 6, 256
    cfg = _native.default_config()
    cfg.dims, cfg.negatives, cfg.hard_negatives, cfg.batch_size, cfg.valid_pct = 16, R, H, B, 0.0
    cfg.max_nodes_kind, cfg.max_nodes = _native.SAMPLE_FIXED, 3.0
    ctx = _native.Context(cfg)
    ctx.upload_graph(prob["rows"], prob["cols"], None)
    ctx.upload_features(prob["fptr"], prob["fids"], prob["n_feat"])
    ctx.set_table(None)
    rows, cols = prob["rows"], prob["cols"]
    stride = int(np.diff(rows).max())
    anchors = np.arange(B, dtype=np.uint32) * 7
    cnt, nbr, _, neg = ctx.sample(anchors, 5, stride)
    again = ctx.sample(anchors, 5, stride)
    assert all(np.array_equal(x, y) for x, y in zip((cnt, nbr, neg), (again[0], again[1], again[3])))
    other = ctx.sample(anchors, 6, stride)
    assert not np.array_equal(neg, other[3])
    good, d_hard, d_uni = 0, [], []
    for a, v in enumerate(anchors.tolist()):
        nb = set(cols[int(rows[v]):int(rows[v + 1])].tolist())
        dist = _bfs(rows, cols, v, 10)
        hard = neg[a, :H].tolist()
        ok = len(set(hard)) == H and all(u != v and u not in nb and u in dist for u in hard)
        good += ok
        if ok:
            d_hard += [dist[u] for u in hard]
            d_uni += [dist.get(u, 11) for u in neg[a, H:].tolist()]
    assert good >= 0.9 * B, good
    assert np.mean(d_hard) + 1.0 < np.mean(d_uni), (np.mean(d_hard), np.mean(d_uni))


def test_hard_negatives_recall_matches_cpu_reference(oracle):
    import cloverleaf_gb300 as cl
    from cloverleaf_gb300 import datagen
    from tests._eval import community_recall
    w = datagen.workload("sbm10k")
    ep = w["ep"]
    g = cl.Graph.from_csr(w["rows"], w["cols"], w["weights"])
    fs = cl.FeatureSet.from_csr(g, w["fptr"], w["fids"], w["n_feat"])
    prop = cl.EmbeddingPropagator(alpha=ep["alpha"], loss=cl.EPLoss.starspace(ep["gamma"], ep["negatives"]),
                                  batch_size=ep["batch_size"], dims=ep["dims"], passes=ep["passes"],
                                  max_nodes=ep["max_nodes"], hard_negatives=2, valid_pct=0.0, indicator=False,
                                  form="fused")
    emb = prop.learn_features(g, fs)
    r_gpu = community_recall(w["fptr"], w["fids"], emb.table, w["community"])
    table, _ = oracle.train(w["rows"], w["cols"], w["weights"], w["fptr"], w["fids"], w["n_feat"], dims=ep["dims"],
                            alpha=ep["alpha"], loss=oracle.LOSS_STARSPACE, gamma=ep["gamma"],
                            negatives=ep["negatives"], batch_size=ep["batch_size"], passes=ep["passes"],
                            max_nodes=(oracle.SAMPLE_FIXED, ep["max_nodes"]), hard_negatives=2, threads=0)
    r_cpu = community_recall(w["fptr"], w["fids"], table, w["community"])
    assert abs(r_gpu - r_cpu) <= 0.01, (r_gpu, r_cpu)


def test_weighted_sampling_matches_a_res_inclusion_probabilities():
    # weighted_neighbor_sampling + weighted_neighbor_averaging: the sampled
    # neighbours are weighted_reservoir_sample (utils.rs:147-161) by the
    # averaging weights.  256 anchors share the same 40 neighbours with
    # weights (j+1)^2; K = 5.  The device's inclusion frequency of each
    # neighbour over 2048 samples matches a numpy Monte-Carlo of the same
    # A-Res rule (keys U^(1/w), the K largest kept).
    A, D, K = 256, 40, 5
    n = A + D
    rows = np.zeros(n + 1, np.uint64)
    rows[1:A + 1] = np.arange(1, A + 1) * D
    rows[A + 1:] = A * D
    cols = np.tile(np.arange(A, A + D, dtype=np.uint32), A)
    wts = np.tile(((np.arange(D) + 1.0) ** 2).astype(np.float32), A)
    wcdf = _native.cdf_convert(rows, wts.copy())
    fptr = np.arange(n + 1, dtype=np.uint64)
    fids = (np.arange(n) % 50).astype(np.uint32)
    cfg = _native.default_config()
    cfg.dims, cfg.negatives, cfg.batch_size, cfg.valid_pct = 16, 2, A, 0.0
    cfg.max_nodes_kind, cfg.max_nodes = _native.SAMPLE_FIXED, float(K)
    cfg.weighted_neighbor_sampling = cfg.weighted_neighbor_averaging = 1
    ctx = _native.Context(cfg)
    ctx.upload_graph(rows, cols, wcdf)
    ctx.upload_features(fptr, fids, 50)
    ctx.set_table(None)
    counts = np.zeros(D)
    anchors = np.arange(A, dtype=np.uint32)
    for step in range(1, 9):
        cnt, nbr, w, _ = ctx.sample(anchors, step, D)
        assert (cnt == K).all()
        for a in range(A):
            got = nbr[a, :K].astype(np.int64) - A
            assert len(set(got.tolist())) == K
            counts[got] += 1
            # weights are the averaging weights scale * p_i * deg
            p = ((got + 1.0) ** 2) / ((np.arange(D) + 1.0) ** 2).sum()
            assert np.allclose(w[a, :K], (D / K) * p * D, rtol=1e-4)   # p from float32 CDF differences
    freq = counts / (8 * A)
    rng = np.random.default_rng(0)
    u = rng.random((100000, D))
    keys = u ** (1.0 / ((np.arange(D) + 1.0) ** 2))
    top = np.argsort(-keys, axis=1)[:, :K]
    want = np.bincount(top.ravel(), minlength=D) / 100000
    assert np.abs(freq - want).max() < 0.045, np.abs(freq - want).max()
    # far from uniform (K / D each): the heaviest 2.7x, the lightest rarely
    assert freq[-1] > 2 * K / D and want[-1] > 2 * K / D
    assert freq[0] < 0.25 * K / D


@pytest.mark.parametrize("kind,val", [("fixed", 40.0), ("prob", 0.5)])
def test_weighted_sampling_many_neighbours(kind, val):
    # counts above 32 (Fixed 40 of 100) and Probability counts (Binomial(100,
    # .5), then that many by weight) use the radix selection of the r largest
    # A-Res keys; inclusion frequencies over 1024 draws match a numpy
    # Monte-Carlo of the same rule, and Fixed draws exactly 40 distinct
    A, D = 128, 100
    n = A + D
    rows = np.zeros(n + 1, np.uint64)
    rows[1:A + 1] = np.arange(1, A + 1) * D
    rows[A + 1:] = A * D
    cols = np.tile(np.arange(A, A + D, dtype=np.uint32), A)
    base = ((np.arange(D) + 1.0) ** 1.5).astype(np.float32)
    wcdf = _native.cdf_convert(rows, np.tile(base, A).copy())
    fptr = np.arange(n + 1, dtype=np.uint64)
    fids = (np.arange(n) % 50).astype(np.uint32)
    cfg = _native.default_config()
    cfg.dims, cfg.negatives, cfg.batch_size, cfg.valid_pct = 16, 2, A, 0.0
    cfg.max_nodes_kind = _native.SAMPLE_FIXED if kind == "fixed" else _native.SAMPLE_PROB
    cfg.max_nodes = val
    cfg.weighted_neighbor_sampling = cfg.weighted_neighbor_averaging = 1
    ctx = _native.Context(cfg)
    ctx.upload_graph(rows, cols, wcdf)
    ctx.upload_features(fptr, fids, 50)
    ctx.set_table(None)
    counts = np.zeros(D)
    sizes = []
    anchors = np.arange(A, dtype=np.uint32)
    p = base.astype(np.float64) / base.sum()
    for step in range(1, 9):
        cnt, nbr, w, _ = ctx.sample(anchors, step, D)
        for a in range(A):
            r = int(cnt[a])
            got = nbr[a, :r].astype(np.int64) - A
            assert len(set(got.tolist())) == r and (got >= 0).all() and (got < D).all()
            counts[got] += 1
            sizes.append(r)
            scale = D / r if kind == "fixed" else 1 / val
            assert np.allclose(w[a, :r], scale * p[got] * D, rtol=1e-3)
    sizes = np.array(sizes)
    rng = np.random.default_rng(1)
    if kind == "fixed":
        assert (sizes == 40).all()
        want_sizes = np.full(20000, 40)
    else:
        assert abs(sizes.mean() - 50) < 1.5 and sizes.min() >= 1
        want_sizes = rng.binomial(D, val, 20000)
    # Monte-Carlo of the rule: per draw, the r largest U^(1/w) (w ~ p, scale-free)
    u = rng.random((20000, D))
    keys = np.log(u) / p
    order = np.argsort(-keys, axis=1)
    mask = np.arange(D)[None, :] < want_sizes[:, None]
    want = np.zeros(D)
    np.add.at(want, order[mask], 1)
    want /= 20000
    freq = counts / (8 * A)
    assert np.abs(freq - want).max() < 0.06, np.abs(freq - want).max()
    assert freq[-1] > freq[0] + 0.3          # heavy neighbours far more often
