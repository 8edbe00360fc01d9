"""The host-side pieces `scripts/learn.py` of the reference calls around
training: FeatureSet.new_from_file (src/lib.rs:1440-1517), FeaturePropagator
(src/lib.rs:1695-1770, src/algos/feat_propagation.rs:13-93) and
FeatureAggregator save / load / Attention (src/lib.rs:1772-2000).  No GPU."""
import numpy as np
import pytest

import cloverleaf_gb300 as cl
from cloverleaf_gb300 import _native


def _propagate_restated(rows, cols, cdf, lists, max_iters, k, threshold):
    """feat_propagation.rs:13-93 in plain Python with f32 arithmetic; equal
    weights ordered by feature id."""
    f32 = np.float32
    lists = [list(x) for x in lists]
    done = [len(x) > 0 for x in lists]
    for _ in range(max_iters):
        all_final = True
        for v in range(len(lists)):
            if done[v]:
                continue
            acc, final, prev = {}, True, f32(0)
            for e in range(int(rows[v]), int(rows[v + 1])):
                px = f32(cdf[e] - prev)
                prev = f32(cdf[e])
                fu = lists[int(cols[e])]
                final = final and len(fu) > 0
                for f in fu:
                    acc[f] = f32(acc.get(f, f32(0)) + px)
            order = sorted(acc.items(), key=lambda t: (-t[1], t[0]))
            sq = f32(0)
            for _, w in order:
                sq = f32(sq + f32(w * w))
            norm = f32(np.sqrt(sq))
            with np.errstate(invalid="ignore", divide="ignore"):
                lists[v] = [f for f, w in order if f32(w / norm) > f32(threshold)][:k]
            if final:
                done[v] = True
            else:
                all_final = False
        if all_final:
            break
    return lists


@pytest.mark.parametrize("seed,k,threshold,iters", [(1, 3, 0.0, 20), (2, 1, 0.0, 1), (3, 5, 0.3, 20), (4, 2, 0.0, 3)])
def test_feature_propagation_matches_restatement(seed, k, threshold, iters):
    rng = np.random.default_rng(seed)
    n = 300
    src = rng.integers(0, n, 900)
    dst = rng.integers(0, n, 900)
    w = rng.uniform(0.5, 4.0, 900).astype(np.float32)
    rows, cols, wr = _native.csr_from_edges(np.concatenate([src, dst]), np.concatenate([dst, src]),
                                            np.concatenate([w, w]), True)
    cdf = _native.cdf_convert(rows, wr)
    nn = len(rows) - 1
    lists = [sorted(set(rng.integers(0, 40, rng.integers(1, 4)).tolist())) if rng.random() < 0.3 else []
             for _ in range(nn)]
    g = cl.Graph(rows, cols, cdf, cl.Vocab.anonymous(nn))
    fs = cl.FeatureSet(g.vocab_, nn)
    for i in range(40):
        fs.feature_vocab.get_or_insert("feat", str(i))
    fs._feats = [list(x) for x in lists]
    fp = cl.FeaturePropagator(k, threshold, iters)
    fp.propagate(g, fs)
    want = _propagate_restated(rows, cols, cdf, lists, iters, k, threshold)
    got = fs._lists()
    assert got == want
    filled = sum(1 for a, b in zip(lists, got) if not a and b)
    assert filled > 0
    for a, b in zip(lists, got):           # nodes that had features keep them
        if a:
            assert a == b


def test_feature_propagation_chain_and_repr():
    # a path 0 - 1 - 2 - 3 with features only on node 0: one sweep fills all
    # (in-place updates), and a second confirms every node is final
    rows, cols, w = _native.csr_from_edges(np.array([0, 1, 1, 2, 2, 3]), np.array([1, 0, 2, 1, 3, 2]),
                                           np.ones(6, np.float32), True)
    g = cl.Graph.from_csr(rows, cols, w)
    fs = cl.FeatureSet(g.vocab_, 4)
    fs.set_features(("node", "0"), [("feat", "a"), ("feat", "b")])
    cl.FeaturePropagator(1).propagate(g, fs)
    assert [fs.get_features(("node", str(i))) for i in range(4)] == [[("feat", "a"), ("feat", "b")]] + \
        [[("feat", "a")]] * 3
    assert repr(cl.FeaturePropagator(3, 0.25, 7)) == "FeaturePropagator<k=3,threshold=0.25,max_iters=7>"
    assert repr(cl.FeaturePropagator(3)) == "FeaturePropagator<k=3,threshold=0,max_iters=20>"


def test_feature_set_new_from_file(tmp_path):
    p = str(tmp_path / "feats.tsv")
    with open(p, "w") as f:
        f.write("user\tu1\tred big\nitem\ti7\tred\nuser\tu2\tsmall\n")
    fs = cl.FeatureSet.new_from_file(p)
    assert fs.nodes() == 3 and list(fs.vocab()) == [("user", "u1"), ("item", "i7"), ("user", "u2")]
    assert fs.get_features(("item", "i7")) == [("feat", "red")]
    assert fs.num_features() == 3
    fs2 = cl.FeatureSet.new_from_file(p, cl.FeatureNamespace.node_type())
    assert fs2.get_features(("user", "u1")) == [("user", "red"), ("user", "big")]
    with open(p, "a") as f:
        f.write("broken line\n")
    with pytest.raises(ValueError):
        cl.FeatureSet.new_from_file(p)


def test_aggregator_save_load(tmp_path):
    g = cl.Graph.from_csr(np.array([0, 1, 2, 2], np.uint64), np.array([1, 0], np.uint32))
    fs = cl.FeatureSet(g.vocab_, 3)
    fs.set_features(("node", "0"), [("feat", "a"), ("feat", "b")])
    fs.set_features(("node", "1"), [("feat", "a")])
    fs.set_features(("node", "2"), [("feat", "c"), ("feat", "a")])
    agg = cl.FeatureAggregator.Weighted(0.1, fs)
    assert repr(agg) == "FeatureAggregator<Weighted<alpha=0.1>>"
    p = str(tmp_path / "agg")
    agg.save(p)
    lines = open(p).read().splitlines()
    # alpha as an f32, each probability as the f64 image of an f32
    assert lines[:2] == ["Weighted", "0.1"]
    assert lines[2] == "feat\ta\t0.6000000238418579" and lines[3] == "feat\tb\t0.20000000298023224"
    back = cl.FeatureAggregator.load(p)
    assert back.kind == "weighted" and back.alpha == np.float32(0.1)
    assert np.array_equal(back.unigrams, agg.unigrams) and list(back.vocab) == list(agg.vocab)
    for a in (cl.FeatureAggregator.Averaged(), cl.FeatureAggregator.Attention(4, 16, None),
              cl.FeatureAggregator.Attention(2, 8, 5)):
        a.save(p)
        b = cl.FeatureAggregator.load(p)
        assert repr(b) == repr(a)
    assert open(p).read() == "Attention\n2\n8\n5\n"
    assert repr(cl.FeatureAggregator.Attention(2, 8)) == "FeatureAggregator<Attention<num_heads=2,d_k=8,window=None>"
    with open(p, "w") as f:
        f.write("Weighted\n0.5\nfeat\ta\t0.5\nfeat\ta\t0.5\n")
    with pytest.raises(ValueError, match="Duplicate"):
        cl.FeatureAggregator.load(p)
    with open(p, "w") as f:
        f.write("Median\n")
    with pytest.raises(ValueError, match="Unknown aggregator"):
        cl.FeatureAggregator.load(p)


def test_attention_aggregation_is_refused():
    g = cl.Graph.from_csr(np.array([0, 1, 2], np.uint64), np.array([1, 0], np.uint32))
    fs = cl.FeatureSet(g.vocab_, 2)
    emb = cl.NodeEmbeddings(cl.Vocab.anonymous(2, "feat"), np.ones((2, 4), np.float32))
    with pytest.raises(cl.UnsupportedOption):
        cl.NodeEmbedder(cl.FeatureAggregator.Attention(2, 4)).embed_feature_set(fs, emb)
