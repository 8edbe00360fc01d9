"""Distribution of the default device sampler, through the C ABI.

Defaults of the reference (EmbeddingPropagator with max_nodes = Fixed(K),
no weighted sampling, no hard negatives):
  * neighbours: min(K, deg) distinct positions of the anchor's row, a uniform
    subset (reconstruct_node_embedding, src/algos/ep/model.rs:342-386, with
    reservoir_sample, src/algos/utils.rs:128-145; here Floyd's algorithm),
    every chosen neighbour weighted deg / r (Sample::sample,
    src/algos/utils.rs:193-216);
  * negatives: R uniform draws with replacement from the training ids only
    (sample_negatives, src/algos/grad_utils/node_sampler.rs:83-107).
Frequencies are checked with chi-square tests at p > 1e-4 (the streams are
seeded, so the outcome is fixed).
"""
import itertools

import numpy as np
import pytest
from scipy import stats

from cloverleaf_gb300 import _native

pytestmark = pytest.mark.gpu


def star_graph(n_anchor, deg, n_total):
    """Anchors 0..n_anchor-1, each with `deg` distinct neighbours among the
    other nodes; every node carries one feature."""
    rows = np.zeros(n_total + 1, np.uint64)
    cols = []
    for a in range(n_total):
        if a < n_anchor:
            cols.extend(n_anchor + (a * deg + j) % (n_total - n_anchor) for j in range(deg))
        else:
            cols.append(a % n_anchor)
        rows[a + 1] = len(cols)
    fptr = np.arange(n_total + 1, dtype=np.uint64)
    fids = (np.arange(n_total) % 97).astype(np.uint32)
    return rows, np.array(cols, np.uint32), fptr, fids


def sampler_ctx(rows, cols, fptr, fids, K, R, valid_pct=0.0, batch=256):
    cfg = _native.default_config()
    cfg.dims, cfg.negatives, cfg.loss, cfg.gamma = 8, R, _native.LOSS_STARSPACE, 0.5
    cfg.batch_size, cfg.passes, cfg.valid_pct = batch, 1, valid_pct
    cfg.max_nodes_kind, cfg.max_nodes = _native.SAMPLE_FIXED, float(K)
    ctx = _native.Context(cfg)
    ctx.upload_graph(rows, cols, None)
    ctx.upload_features(fptr, fids, 97)
    ctx.set_table(None)
    return ctx


def test_neighbour_inclusion_is_uniform_with_scale_weight():
    n_anchor, deg, K = 200, 40, 10
    rows, cols, fptr, fids = star_graph(n_anchor, deg, 2000)
    ctx = sampler_ctx(rows, cols, fptr, fids, K, R=2)
    anchors = np.arange(n_anchor, dtype=np.uint32)
    counts = np.zeros(deg, np.int64)
    steps = 150
    for step in range(1, steps + 1):
        cnt, nbr, w, _ = ctx.sample(anchors, step, K)
        assert (cnt == K).all()
        # scale weight deg / r, exactly (utils.rs:200-203)
        assert (w[:, :K] == np.float32(deg) / np.float32(K)).all()
        for a in range(n_anchor):
            row = cols[int(rows[a]):int(rows[a + 1])]
            pos = np.searchsorted(row, nbr[a, :K]) if (np.diff(row) > 0).all() else \
                np.array([np.nonzero(row == x)[0][0] for x in nbr[a, :K]])
            assert (row[pos] == nbr[a, :K]).all()
            assert len(set(pos.tolist())) == K               # without replacement
            counts[pos] += 1
    # each position is chosen with probability K / deg
    expected = np.full(deg, n_anchor * steps * K / deg)
    assert stats.chisquare(counts, expected).pvalue > 1e-4, counts


def test_neighbour_subsets_are_uniform():
    # deg 6, K 3: all C(6, 3) = 20 subsets equally likely (a uniform
    # K-subset, not just uniform single inclusions)
    n_anchor, deg, K = 256, 6, 3
    rows, cols, fptr, fids = star_graph(n_anchor, deg, 1000)
    ctx = sampler_ctx(rows, cols, fptr, fids, K, R=1)
    subsets = {s: i for i, s in enumerate(itertools.combinations(range(deg), K))}
    counts = np.zeros(len(subsets), np.int64)
    anchors = np.arange(n_anchor, dtype=np.uint32)
    for step in range(1, 101):
        cnt, nbr, w, _ = ctx.sample(anchors, step, K)
        assert (cnt == K).all() and (w[:, :K] == np.float32(2.0)).all()
        for a in range(n_anchor):
            row = cols[int(rows[a]):int(rows[a + 1])]
            pos = tuple(sorted(int(np.nonzero(row == x)[0][0]) for x in nbr[a, :K]))
            counts[subsets[pos]] += 1
    assert stats.chisquare(counts).pvalue > 1e-4, counts


def test_low_degree_takes_every_neighbour_with_weight_one():
    n_anchor, deg, K = 64, 5, 10
    rows, cols, fptr, fids = star_graph(n_anchor, deg, 400)
    ctx = sampler_ctx(rows, cols, fptr, fids, K, R=1)
    cnt, nbr, w, _ = ctx.sample(np.arange(n_anchor, dtype=np.uint32), 7, K)
    assert (cnt == deg).all()
    assert (w[:, :deg] == 1.0).all()
    for a in range(n_anchor):
        assert sorted(nbr[a, :deg].tolist()) == sorted(cols[int(rows[a]):int(rows[a + 1])].tolist())


def test_negatives_are_uniform_over_training_ids():
    n = 2000
    rows, cols, fptr, fids = star_graph(200, 8, n)
    R = 10
    ctx = sampler_ctx(rows, cols, fptr, fids, K=5, R=R, valid_pct=0.3)
    train, valid = ctx.split()
    assert len(valid) == int(np.float32(n) * np.float32(0.3)) and len(train) + len(valid) == n
    assert len(np.intersect1d(train, valid)) == 0
    anchors = np.arange(200, dtype=np.uint32)
    counts = np.zeros(n, np.int64)
    steps = 250
    for step in range(1, steps + 1):
        _, _, _, neg = ctx.sample(anchors, step, 8)
        np.add.at(counts, neg.reshape(-1).astype(np.int64), 1)
    assert counts[valid].sum() == 0, "a validation id was drawn as a negative"
    observed = counts[train]
    assert stats.chisquare(observed).pvalue > 1e-4
    assert observed.sum() == 200 * R * steps
